// flopcount.cc — algorithmic work of the kt-loop, by instrumentation.
//
// Instantiates the loop integral that the record-mode kernels run (grn_loop3.cuh,
// loop_integral3<V>: the azimuth-outer loop of two events on FP32x2 pairs) on the host with
// a counting pair type, and evaluates it on sampled event pairs of the benchmark workload
// (63 x 33 loop grid, kt <= 3 GeV). Prints, per loop point (per event), the mean numbers of
// FP32 operations (an FMA counts two: multiply and add) and of special-function calls
// (log2, exp2, sincos, reciprocal division, sinpi, sqrt), everything the function executes
// including the per-phi-node projections and the compensated summation.
#include <cmath>
#include <cstdio>
#include <cstdint>
#include <cstring>

#include <vector>

#include "grn_physics.cuh"
#include "grn_loop3.cuh"

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
inline CF atan2(CF y, CF x) { g_cnt.sincos++; return CF(std::atan2(y.v, x.v)); }
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

// FP32x2 pair with counting lane operations (the float2 operations of the device kernel).
struct CF2 {
  CF x, y;
};
namespace grn {
template <>
inline CF2 splat<CF2>(float a) {
  return {CF(a), CF(a)};
}
}  // namespace grn
inline CF2 add2(CF2 a, CF2 b) { return {a.x + b.x, a.y + b.y}; }
inline CF2 mul2(CF2 a, CF2 b) { return {a.x * b.x, a.y * b.y}; }
inline CF2 fma2(CF2 a, CF2 b, CF2 c) { return {a.x * b.x + c.x, a.y * b.y + c.y}; }
inline CF2 sub2(CF2 a, CF2 b) { return {a.x - b.x, a.y - b.y}; }
inline CF2 log2_2(CF2 a) { return {fast_log2(a.x), fast_log2(a.y)}; }
inline CF2 exp2_2(CF2 a) { return {fast_exp2(a.x), fast_exp2(a.y)}; }
inline CF2 div2(CF2 a, CF2 b) { return {fast_div(a.x, b.x), fast_div(a.y, b.y)}; }
inline CF2 abs2(CF2 a) { return {fabs(a.x), fabs(a.y)}; }
inline CF2 sqrt2(CF2 a) { return {sqrt(a.x), sqrt(a.y)}; }
inline void sincos_turns2(CF2 h, CF2 &s, CF2 &c) {  // reduction: one subtraction per lane
  g_cnt.add += 2;
  sincos_pi(CF(2.0 * h.x.v), s.x, c.x);
  sincos_pi(CF(2.0 * h.y.v), s.y, c.y);
  g_cnt.mul += 2;  // 2 pi r
}
inline CF2 sinpi_turns2(CF2 d) {
  g_cnt.sincos += 2;
  return {CF(std::sin(grn::kPi * d.x.v)), CF(std::sin(grn::kPi * d.y.v))};
}
struct KtNodeC {
  CF2 kt, k2, cre, cim, ncim, cabs;
};
struct PhiNodeC {
  CF2 c, s, u, t;
};

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
  K.invL = 1.0 / K.L; K.invL2 = 1.0 / (K.L * K.L);
  K.ifc1 = 1.0 / P.soft.fc1; K.ifc2 = 1.0 / P.soft.fc2;
  K.mp2 = P.m_beam * P.m_beam; K.m3 = K.m4 = P.m_central[0]; K.m3sq = K.m4sq = K.m3 * K.m3;
  K.lnpt_lo = std::log(1e-12); K.lnpt_hi = std::log(2.5); K.M2prop = K.m3sq;
  K.g2 = 1.0; K.gN2 = 1.0; K.n_active = 1; K.active[0] = 1; K.eta0_re[0] = 1.0;

  // loop grid of the benchmark: 64 kt nodes up to 3 GeV, 34 phi nodes (Simpson weights are
  // values only; they do not change the operation count)
  const int n_kt = 64, n_phi = 34;
  std::vector<KtNodeC> kt(n_kt);
  std::vector<PhiNodeC> ph(n_phi);
  for (int j = 0; j < n_kt; ++j) {
    const float k = float(1e-4 + j * (3.0 - 1e-4) / (n_kt - 1));
    kt[j] = {grn::splat<CF2>(k), grn::splat<CF2>(k * k), grn::splat<CF2>(1.f),
             grn::splat<CF2>(0.5f), grn::splat<CF2>(-0.5f), grn::splat<CF2>(1.118f)};
  }
  for (int i = 0; i < n_phi; ++i) {
    const double a = 2 * grn::kPi * i / (n_phi - 1);
    ph[i] = {grn::splat<CF2>(float(std::cos(a))), grn::splat<CF2>(float(std::sin(a))),
             grn::splat<CF2>(1.f), grn::splat<CF2>(float(a / (2 * grn::kPi)))};
  }
  uint64_t st = 88172645463325252ull;
  auto rnd = [&]() {
    st ^= st << 13; st ^= st >> 7; st ^= st << 17;
    return static_cast<double>(st >> 11) * 0x1.0p-53;
  };
  auto event = [&](grn::LoopEventF<CF> &le) {
    while (true) {
      double u[8];
      for (double &x : u) x = rnd();
      grn::Born b;
      if (!grn::born_kinematics(P, K, u, b)) continue;
      grn::make_loop_event_fast<CF>(P, K, b, le);
      return;
    }
  };
  const int n_pairs = 256;
  double points = 0;
  g_cnt = Cnt{};
  for (int q = 0; q < n_pairs; ++q) {
    grn::LoopEventF<CF> a, b;
    const Cnt keep = g_cnt;
    event(a);
    event(b);
    g_cnt = keep;  // record building (stage A) is not loop-stage work
    grn::Loop3<CF2> e;
    grn::make_loop3<CF2>(a, b, [](CF x, CF y) { return CF2{x, y}; }, e);
    CF2 sr, si, sm;
    grn::loop_integral3(e, n_kt, n_phi, kt.data(), ph.data(), sr, si, sm);
    g_cnt.mul += 2 * 4;
    g_cnt.add += 2 * 2;
    points += 2.0 * n_kt * n_phi;
  }
  const double arith = (g_cnt.add + g_cnt.mul + g_cnt.div) / points;
  const double trans = (g_cnt.exp + g_cnt.log + g_cnt.sqrt + g_cnt.sincos) / points;
  std::printf("{\"points\": %.0f, \"add\": %.3f, \"mul\": %.3f, \"div\": %.3f, \"exp\": %.3f, "
              "\"log\": %.3f, \"sqrt\": %.3f, \"sincospi\": %.3f, \"summation\": 0, "
              "\"flops\": %.3f, \"transcendentals\": %.3f}\n",
              points, g_cnt.add / points, g_cnt.mul / points, g_cnt.div / points,
              g_cnt.exp / points, g_cnt.log / points, g_cnt.sqrt / points,
              g_cnt.sincos / points, arith, trans);
  return 0;
}
