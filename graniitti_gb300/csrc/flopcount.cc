// flopcount.cc — algorithmic work of the kt-loop, by instrumentation.
//
// Instantiates the device loop arithmetic (grn_physics.cuh, loop_point_amp<T> and
// regge_me4<T>) on the host with a counting scalar and evaluates it on sampled
// events of the benchmark workload. Prints, per loop point, the mean numbers of
// FP32 add/sub, mul, div and of transcendental calls (exp, log, sqrt, sincospi),
// plus the compensated-summation adds of the loop integral.
#include <cmath>
#include <cstdio>
#include <cstdint>
#include <cstring>

#include "grn_physics.cuh"

struct Cnt {
  double add = 0, mul = 0, div = 0, exp = 0, log = 0, sqrt = 0, sincos = 0, cmp = 0;
};
static Cnt g_cnt;

struct CF {
  float v;
  CF() : v(0) {}
  CF(double x) : v(static_cast<float>(x)) {}
  explicit operator double() const { return v; }
};
inline CF operator+(CF a, CF b) { g_cnt.add++; return CF(a.v + b.v); }
inline CF operator-(CF a, CF b) { g_cnt.add++; return CF(a.v - b.v); }
inline CF operator*(CF a, CF b) { g_cnt.mul++; return CF(a.v * b.v); }
inline CF operator/(CF a, CF b) { g_cnt.div++; return CF(a.v / b.v); }
inline CF operator-(CF a) { return CF(-a.v); }
inline bool operator>(CF a, CF b) { g_cnt.cmp++; return a.v > b.v; }
inline bool operator<(CF a, CF b) { g_cnt.cmp++; return a.v < b.v; }
inline CF exp(CF a) { g_cnt.exp++; return CF(std::exp(a.v)); }
inline CF log(CF a) { g_cnt.log++; return CF(std::log(a.v)); }
inline CF sqrt(CF a) { g_cnt.sqrt++; return CF(std::sqrt(a.v)); }
inline CF fabs(CF a) { return CF(std::fabs(a.v)); }
inline CF fast_log(CF a) { g_cnt.log++; return CF(std::log(a.v)); }
inline CF fast_exp(CF a) { g_cnt.exp++; return CF(std::exp(a.v)); }
inline CF fast_log2(CF a) { g_cnt.log++; return CF(std::log2(a.v)); }
inline CF fast_exp2(CF a) { g_cnt.exp++; return CF(std::exp2(a.v)); }
inline CF fast_div(CF a, CF b) { g_cnt.div++; return CF(a.v / b.v); }
inline void sincos_pi(CF x, CF &s, CF &c) {
  g_cnt.sincos++;
  s = CF(std::sin(grn::kPi * x.v));
  c = CF(std::cos(grn::kPi * x.v));
}
inline void fast_sincos_pi(CF x, CF &s, CF &c) { sincos_pi(x, s, c); }

int main() {
  grn_process_params P;
  // Benchmark workload parameters (TUNE0, pi+ pi-, ALICE-like cuts).
  std::memset(&P, 0, sizeof(P));
  P.process = GRN_PROC_REGGE_CON; P.phase_space = GRN_PS_CONTINUUM; P.n_central = 2;
  P.sqrt_s = 13000.0; P.m_beam = 0.938272081; P.m_central[0] = P.m_central[1] = 0.13957061;
  P.s_factor = 1.0;
  P.gcuts = {-0.9, 0.9, 0.0, 5.0, 0.0, 2.5, -0.9, 0.9, 0.0, 5.0};
  P.soft.gN_P = 8.2; P.soft.fc1 = 0.34; P.soft.fc2 = 5.0;
  P.regge.a0[0] = 1.088; P.regge.ap[0] = 0.20; P.regge.sgn[0] = 1; P.regge.s0 = 1.0;
  P.regge.active[0] = 1; P.regge.offshellFF = 2; P.regge.b_POW = 0.5; P.regge.c[0] = 35.00184;
  grn::Consts K{};
  const double E = 6500.0, pz = std::sqrt(E * E - P.m_beam * P.m_beam);
  K.s = 13000.0 * 13000.0; K.sqrt_s = 13000.0; K.L = E + pz; K.eps = P.m_beam * P.m_beam / K.L;
  K.mp2 = P.m_beam * P.m_beam; K.m3sq = K.m4sq = P.m_central[0] * P.m_central[0];
  K.lnpt_lo = std::log(1e-12); K.lnpt_hi = std::log(2.5); K.M2prop = K.m3sq;
  K.g2 = 1.0; K.gN2 = 1.0; K.n_active = 1; K.active[0] = 1; K.eta0_re[0] = 1.0;

  const int n_ev = 512, n_kt = 64, n_phi = 34;
  uint64_t st = 88172645463325252ull;
  auto rnd = [&]() {
    st ^= st << 13; st ^= st >> 7; st ^= st << 17;
    return static_cast<double>(st >> 11) * 0x1.0p-53;
  };
  double points = 0;
  for (int ev = 0; ev < n_ev; ++ev) {
    double u[8];
    for (double &x : u) x = rnd();
    grn::Born b;
    if (!grn::born_kinematics(P, K, u, b)) continue;
    grn::LoopEventF<CF> le;
    grn::make_loop_event_fast<CF>(P, K, b, le);
    for (int j = 0; j < n_kt; ++j)
      for (int i = 0; i < n_phi; ++i) {
        const double kt = 1e-4 + j * (3.0 - 1e-4) / (n_kt - 1), ph = 2 * grn::kPi * i / (n_phi - 1);
        grn::cx<CF> A;
        const CF kx = CF(kt) * CF(std::cos(ph)), ky = CF(kt) * CF(std::sin(ph));
        grn::loop_point_amp_fast<CF>(le, kx, ky, CF(kt * kt), A);
        points += 1;
      }
  }
  // Per point in the loop integral: 2 compensated adds (4 flops each) and the
  // weighting product U_i * A (2 mul); per kt row: complex product + 2 compensated adds
  // + k^2. (kx, ky = kt cos, kt sin are counted by the loop above.)
  const double kahan = 2 * 4 + 2 + (4 + 2 * 4 + 1) / static_cast<double>(n_phi);
  const double arith = (g_cnt.add + g_cnt.mul + g_cnt.div) / points;
  const double trans = (g_cnt.exp + g_cnt.log + g_cnt.sqrt + g_cnt.sincos) / points;
  std::printf("{\"points\": %.0f, \"add\": %.3f, \"mul\": %.3f, \"div\": %.3f, \"exp\": %.3f, "
              "\"log\": %.3f, \"sqrt\": %.3f, \"sincospi\": %.3f, \"summation\": %.3f, "
              "\"flops\": %.3f, \"transcendentals\": %.3f}\n",
              points, g_cnt.add / points, g_cnt.mul / points, g_cnt.div / points,
              g_cnt.exp / points, g_cnt.log / points, g_cnt.sqrt / points,
              g_cnt.sincos / points, kahan, arith + kahan, trans);
  return 0;
}
