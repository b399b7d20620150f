// Replay stand-in for the generator's random-number class (include/Graniitti/MRandom.h).
//
// Same public interface as the reference class; the only difference is the type of
// the uniform distribution member `flat`: its draws come from a per-thread replay
// queue while the queue holds values, and from the real ranlux48-driven uniform
// distribution otherwise. The reference's own MRandom.cc is compiled against this
// header unchanged. The golden-vector driver loads the queue before each
// EventWeight call so that draws made inside the reference (off-shell masses,
// decay angles) take given values ("lifted" hypercube coordinates), which makes
// the reference's per-point weight a pure function of the input vector.
#ifndef MRANDOM_H
#define MRANDOM_H

#include <complex>
#include <deque>
#include <random>
#include <stdexcept>
#include <string>
#include <vector>

namespace gra {
namespace replay {
inline std::deque<double> &queue() {
  static thread_local std::deque<double> q;
  return q;
}
inline void push(double u) { queue().push_back(u); }
inline void clear() { queue().clear(); }
inline std::size_t remaining() { return queue().size(); }
}  // namespace replay

class ReplayUniform {
 public:
  ReplayUniform(double a = 0.0, double b = 1.0) : dist_(a, b) {}
  template <typename Engine>
  double operator()(Engine &rng) {
    std::deque<double> &q = replay::queue();
    if (!q.empty()) {
      const double v = q.front();
      q.pop_front();
      return v;
    }
    return dist_(rng);
  }

 private:
  std::uniform_real_distribution<double> dist_;
};

class MRandom {
 public:
  MRandom() : flat(0, 1), gaussian(0, 1) { rng.seed(); }
  ~MRandom() {}

  void SetSeed(int seed) {
    const int SEEDMAX = 2147483647;
    if (seed > SEEDMAX) throw std::invalid_argument("MRandom::SetSeed: invalid seed");
    rng.seed(seed);
    RNDSEED = seed;
  }
  unsigned int GetSeed() const { return RNDSEED; }

  double U(double a, double b);
  double G(double mu, double sigma);
  double PowerRandom(double a, double b, double alpha);
  double RelativisticBWRandom(double m0, double Gamma, double LIMIT = 5.0, double M_MIN = 0.0);
  double CauchyRandom(double m0, double Gamma, double LIMIT = 5.0, double M_MIN = 0.0);
  int    NBDRandom(double avgN, double k, int maxvalue);
  int    PoissonRandom(double lambda);
  double ExpRandom(double lambda);
  int    LogRandom(double p, int maxvalue);
  void   DirRandom(const std::vector<double> &alpha, std::vector<double> &y);

  double NBDpdf(int n, double avgN, double k);
  double Logpdf(int k, double p);

  std::ranlux48                    rng;
  ReplayUniform                    flat;
  std::normal_distribution<double> gaussian;
  unsigned int                     RNDSEED = 0;
};

}  // namespace gra

#endif
