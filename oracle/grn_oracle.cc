// grn_oracle.cc — CPU ORACLE for the GB300 event-weight engine.
//
// TEST INFRASTRUCTURE ONLY. This file restates, in plain FP64 C++, the reference
// generator's algorithm for the engine's hot path so that the tests and the
// benchmark's CPU baseline have an independent checker. The product (the CUDA
// library under graniitti_gb300/) never links, loads or calls it. Only tests/,
// __graft_entry__.smoke() and bench.py's CPU legs use it.
//
// Parity pin: the restatement is checked against golden vectors produced by the
// UNMODIFIED reference sources (oracle/refbuild + tests/golden/make_golden.py).
//
// The restatement follows the reference's own formulation (4-vectors, the
// two-body longitudinal solution, Lorentz scalars from 4-vector sums); the GPU
// kernels use a light-cone formulation of the same physics, so agreement between
// the two is a check of both. File:line citations refer to the GRANIITTI tree.

#include <algorithm>
#include <array>
#include <cmath>
#include <complex>
#include <cstdint>
#include <cstring>
#include <thread>
#include <vector>

#include "graniitti_gb300.h"

namespace orc {

// Arithmetic type of the restatement: double, or long double for the extended-precision
// build (liborc_ld.so) that shows which side of an FP64 disagreement sits nearer the exact
// value of the reference's own formulas (same inputs and constants, smaller rounding).
#ifndef ORC_REAL
#define ORC_REAL double
#endif
using real = ORC_REAL;

using cplx = std::complex<real>;
// Mixed operations of the complex type with double constants and parameters (needed when
// real is long double; the double build never selects them).
template <typename D, typename = std::enable_if_t<std::is_same<D, double>::value &&
                                                  !std::is_same<real, double>::value>>
inline cplx operator*(const cplx &a, D b) { return a * real(b); }
template <typename D, typename = std::enable_if_t<std::is_same<D, double>::value &&
                                                  !std::is_same<real, double>::value>>
inline cplx operator*(D b, const cplx &a) { return real(b) * a; }
template <typename D, typename = std::enable_if_t<std::is_same<D, double>::value &&
                                                  !std::is_same<real, double>::value>>
inline cplx operator/(const cplx &a, D b) { return a / real(b); }
template <typename D, typename = std::enable_if_t<std::is_same<D, double>::value &&
                                                  !std::is_same<real, double>::value>>
inline cplx operator/(D b, const cplx &a) { return real(b) / a; }
template <typename D, typename = std::enable_if_t<std::is_same<D, double>::value &&
                                                  !std::is_same<real, double>::value>>
inline cplx operator+(D b, const cplx &a) { return real(b) + a; }
template <typename D, typename = std::enable_if_t<std::is_same<D, double>::value &&
                                                  !std::is_same<real, double>::value>>
inline cplx operator+(const cplx &a, D b) { return a + real(b); }
template <typename D, typename = std::enable_if_t<std::is_same<D, double>::value &&
                                                  !std::is_same<real, double>::value>>
inline cplx operator-(D b, const cplx &a) { return real(b) - a; }
template <typename D, typename = std::enable_if_t<std::is_same<D, double>::value &&
                                                  !std::is_same<real, double>::value>>
inline cplx operator-(const cplx &a, D b) { return a - real(b); }

constexpr real PI       = 3.14159265358979323846264338327950288;
constexpr real ZERO_EPS = 1e-12;  // MProcess.h: ZERO_EPS used as log(0 + ZERO_EPS)
// Unit conversions (include/Graniitti/MPDG.h:63-78).
constexpr real HBAR     = 6.582119514E-25;
constexpr real C_LIGHT  = 2.99792458E8;
constexpr real GEV2M    = HBAR * C_LIGHT;
constexpr real GEV2FM   = GEV2M * 1E15;
constexpr real GEV2BARN = (GEV2M * GEV2M) / 1E-28;
constexpr real MPI_SOFT = 0.13957018;  // PDG::mpi used by S3PomAlpha (MPDG.h:56)

// Eikonal numerics constants (include/Graniitti/MEikonal.h:27-40).
constexpr real MIN_KT2 = 1E-6, MAX_KT2 = 25.0;
constexpr real MIN_BT = 1E-6;
constexpr real MAX_BT = 10.0 / GEV2FM;
constexpr real FB_MIN_KT = 1E-9, FB_MAX_KT = 30.0;
constexpr int    FB_N = 10000;

inline real sq(real x) { return x * x; }
inline real msqrt(real x) { return std::sqrt(std::max<real>(0, x)); }

// ---------------------------------------------------------------------------
// Minimal 4-vector (px, py, pz, E), metric (+,-,-,-).
struct V4 {
  real x = 0, y = 0, z = 0, e = 0;
  V4() {}
  V4(real x_, real y_, real z_, real e_) : x(x_), y(y_), z(z_), e(e_) {}
  V4     operator+(const V4 &o) const { return V4(x + o.x, y + o.y, z + o.z, e + o.e); }
  V4     operator-(const V4 &o) const { return V4(x - o.x, y - o.y, z - o.z, e - o.e); }
  real m2() const { return e * e - (x * x + y * y + z * z); }
  real m() const { const real v = m2(); return v > 0 ? std::sqrt(v) : -std::sqrt(-v); }
  real pt2() const { return x * x + y * y; }
  real pt() const { return msqrt(pt2()); }
  real p3() const { return msqrt(x * x + y * y + z * z); }
  real rap() const { return 0.5 * std::log((e + z) / (e - z)); }
  real eta() const { const real p = p3(); return 0.5 * std::log((p + z) / (p - z)); }
  real mt() const { return msqrt(m2() + pt2()); }
};

// ---------------------------------------------------------------------------
// Bessel J0: rational approximation for |x| < 8 and the asymptotic modulus/phase
// form for |x| >= 8, as published in Abramowitz & Stegun (1965) 9.4 and used by
// the reference's BESSJ0 (libs/extmath.hpp:12-46). The coefficient tables are the
// published ones; they must be identical for table parity.
real bessel_j0(real x) {
  if (x == 0.0) return 1.0;
  const real ax = std::fabs(x);
  if (ax < 8.0) {
    const real y   = x * x;
    const real num = 57568490574.0 +
                       y * (-13362590354.0 + y * (651619640.7 + y * (-11214424.18 +
                       y * (77392.33017 + y * (-184.9052456)))));
    const real den = 57568490411.0 +
                       y * (1029532985.0 + y * (9494680.718 + y * (59272.64853 +
                       y * (267.8532712 + y * 1.0))));
    return num / den;
  }
  const real z  = 8.0 / ax;
  const real y  = z * z;
  const real xx = ax - 0.785398164;
  const real p  = 1.0 + y * (-0.1098628627E-2 + y * (0.2734510407E-4 +
                    y * (-0.2073370639E-5 + y * 0.2093887211E-6)));
  const real q  = -0.1562499995E-1 + y * (0.1430488765E-3 + y * (-0.6911147651E-5 +
                    y * (0.7621095161E-6 + y * (-0.9349451520E-7))));
  return std::sqrt(0.636619772 / ax) * (p * std::cos(xx) - z * q * std::sin(xx));
}

// Composite Simpson 1/3 rule over N+1 equidistant samples, N even
// (include/Graniitti/MMath.h:378-394).
template <typename T>
T simpson13(const std::vector<T> &f, real h) {
  const std::size_t N = f.size() - 1;
  T even = 0.0, odd = 0.0;
  for (std::size_t j = 1; j + 1 <= N / 2; ++j) even += f[2 * j];
  for (std::size_t j = 1; j <= N / 2; ++j) odd += f[2 * j - 1];
  return h * (f[0] + 2.0 * even + 4.0 * odd + f[N]) / 3.0;
}

// Simpson 3/8 weights 1,3,3,2,3,3,2,...,3,3,1 over N+1 points, N % 3 == 0
// (include/Graniitti/MMath.h:502-516).
std::vector<real> simpson38_weights(int N) {
  std::vector<real> w(N + 1, 3.0);
  w[0] = w[N] = 1.0;
  for (int i = 3; i < N; i += 3) w[i] = 2.0;
  return w;
}

// ---------------------------------------------------------------------------
// Model functions.

// Regge signature factor (src/MForm.cc:382-385).
cplx regge_eta(real alpha, real sigma) {
  const cplx i(0, 1);
  return -(1.0 + sigma * std::exp(-i * PI * alpha)) / std::sin(PI * alpha);
}
// Linear-trajectory signature factor (src/MForm.cc:394-396).
cplx regge_eta_linear(real t, real a0, real ap, real sigma) {
  const cplx i(0, 1);
  return regge_eta(a0, sigma) * std::exp(-i * PI / 2.0 * ap * t);
}
// Proton form factor, real pole (src/MForm.cc:433-435).
real proton_ff(const grn_soft_params &sp, real t) {
  return (1.0 / (1.0 - t / sp.fc1)) * (1.0 / (1.0 - t / sp.fc2));
}
// Inelastic proton vertex of an excited forward leg of mass^2 M2 (S3FINEL, src/MForm.cc:
// 443-449): (|t| / (M2 (|t| + a)))^((1 + Delta_P) / 2), Delta_P = 0.0808, a = 0.5616 GeV^2.
real proton_ff_inel(real t, real M2) {
  const real DELTA_P = 0.0808, a = 0.5616;
  return std::pow(std::fabs(t) / (M2 * (std::fabs(t) + a)), 0.5 * (1.0 + DELTA_P));
}
// Pion-loop insert of the non-linear pomeron trajectory (src/MForm.cc:418-427).
real pion_loop(const grn_soft_params &sp, real tau, real t) {
  const real sqt = std::sqrt(1.0 + tau);
  const real fpi = 1.0 / (1.0 - t / sp.fc3);
  return (4.0 / tau) * fpi * fpi *
         (2.0 * tau - std::pow(1.0 + tau, 1.5) * std::log((sqt + 1.0) / (sqt - 1.0)) +
          std::log(1.0 / (MPI_SOFT * MPI_SOFT)));
}
// Non-linear pomeron trajectory (src/MForm.cc:402-413).
real pomeron_alpha(const grn_soft_params &sp, real t) {
  const real beta_pi = (2.0 / 3.0) * sp.gN_P;
  const real pic     = (beta_pi * beta_pi * MPI_SOFT * MPI_SOFT) / (32.0 * PI * PI * PI);
  const real h       = pic * pion_loop(sp, 4.0 * MPI_SOFT * MPI_SOFT / std::fabs(t), t);
  return 1.0 + sp.delta_P + sp.alpha_P * t - h;
}
// Single pomeron elastic amplitude (src/MEikonal.cc:139-162), C-even only.
cplx elastic_amp(const grn_soft_params &sp, real s, real t) {
  const real F = proton_ff(sp, t);
  const real a = pomeron_alpha(sp, t);
  cplx A = sp.gN_P * sp.gN_P * F * F * regge_eta(a, 1.0) * std::pow(s, a);
  if (sp.odderon_on) A += sp.gN_O * sp.gN_O * F * F * regge_eta(a, -1.0) * std::pow(s, a);
  return A;
}

// Regge propagator sum (s/s0)^alpha(t) with signature factors (src/MRegge.cc:888-906).
cplx regge_prop(const grn_regge_params &rp, real s, real t) {
  cplx M(0, 0);
  for (int k = 0; k < 3; ++k) {
    if (!rp.active[k]) continue;
    const real alpha = rp.a0[k] + rp.ap[k] * t;
    M += regge_eta_linear(t, rp.a0[k], rp.ap[k], rp.sgn[k]) * std::pow(s / rp.s0, alpha);
  }
  return M;
}
// Off-shell meson form factor (src/MRegge.cc:1155-1174).
real meson_ff(const grn_regge_params &rp, real that, real M2) {
  const real tp = that - M2;
  switch (rp.offshellFF) {
    case 0: return std::exp(-rp.b_EXP * std::fabs(tp));
    case 1: return std::exp(-rp.b_OREAR * msqrt(std::fabs(tp) + sq(rp.a_OREAR)) +
                            rp.a_OREAR * rp.b_OREAR);
    default: return 1.0 / (1.0 - tp / rp.b_POW);
  }
}

// ---------------------------------------------------------------------------
// Kinematics state of one event (the part of LORENTZSCALAR the path uses).
struct Event {
  V4     pb1, pb2;         // beams
  V4     pf[9];            // pfinal[0..8]: central system, forward 1, forward 2, central a, b
                           // (c, d, ... for 4- and 6-body central states)
  V4     q;                // intermediate difference momentum (pkt_[0]), <C>
  V4     kq[5];            // <C> with 4 or 6 central particles: the difference momenta pkt_
  real dw = 0;           // <F>: 2-body phase-space weight dPhi2 (MFactorized.cc:381)
  real m2lo = 0, m2hi = 0;  // <F>: central mass^2 window of this point
  V4     leaf[6];          // cascades: final-state daughters (central 1: 0, 1; central 2: 2, 3);
                           // N-body states: the central particles
  real t1 = 0, t2 = 0, that = 0, uhat = 0, m2 = 0, Y = 0, Pt = 0;
  real ss[9][9] = {};
  // forward legs: masses (the beam mass, or the excited N* mass) and the excitation flags
  real mf1 = 0, mf2 = 0;
  bool ex1 = false, ex2 = false;
  // 4- and 6-body central states: (q1 - p_i)^2, (q2 - p_i)^2, (q1 - p_i - p_j)^2
  // (MProcess.cc:1556-1561)
  real tt1[9] = {}, tt2[9] = {}, ttxy[9][9] = {};
};

struct Setup {
  grn_process_params p;
  real             s = 0, sqrt_s = 0;
  V4                 pb1, pb2;
  const double      *msa = nullptr;  // (x, re, im) rows (the table as given, double)
  int                n_kt2 = 0;
};

void forward_masses(const Setup &S, real u_m0, real u_m1, real u_side, Event &ev);

// Longitudinal momentum of leg 3 in p1 p2 -> p3 {p5} p4 (CM frame): the two
// forward legs carry transverse masses a = m3^2+pt3^2, b = m4^2+pt4^2 and share the
// energy-momentum (E_R, pz_R) = (sqrt(s) - E5, -pz5); the forward-going root of the
// two-body problem. Same quantity as kinematics::SolvePz (MKinematics.h:220-229).
real solve_pz(real m3, real m4, real pt3, real pt4, real pz5, real E5, real s) {
  const real ER  = std::sqrt(s) - E5;
  const real pzR = -pz5;
  const real MR2 = ER * ER - pzR * pzR;
  const real a   = m3 * m3 + pt3 * pt3;
  const real b   = m4 * m4 + pt4 * pt4;
  const real lam = sq(MR2 - a - b) - 4.0 * a * b;
  return (pzR * (MR2 + a - b) + ER * std::sqrt(lam)) / (2.0 * MR2);
}

// Energy-momentum conservation check with 1e-6 tolerance (MMath.h:191-198).
bool check_emc(const V4 &d) {
  const real eps = 1e-6;
  return !(std::fabs(d.x) > eps || std::fabs(d.y) > eps || std::fabs(d.z) > eps || d.e > eps);
}

// Lorentz scalars of a 2 -> 4 event (MProcess.cc:1499-1584, Nf = 4).
bool lorentz_scalars(const Setup &S, Event &ev) {
  const int Nf = 2 + S.p.n_central;
  for (int i = 0; i <= Nf; ++i)
    for (int j = i + 1; j <= Nf; ++j) {
      ev.ss[i][j] = (ev.pf[i] + ev.pf[j]).m2();
      ev.ss[j][i] = ev.ss[i][j];
      if (ev.ss[i][j] < 0) return false;
    }
  if (ev.ss[1][0] < 0 || ev.ss[2][0] < 0) return false;
  const V4 q1 = S.pb1 - ev.pf[1];
  const V4 q2 = S.pb2 - ev.pf[2];
  ev.t1 = q1.m2();
  ev.t2 = q2.m2();
  if (ev.t1 > 0 || ev.t2 > 0) return false;
  ev.that = (q1 - ev.pf[3]).m2();
  ev.uhat = (q1 - ev.pf[4]).m2();
  if (Nf > 4) {
    for (int i = 3; i <= Nf; ++i) {
      ev.tt1[i] = (q1 - ev.pf[i]).m2();
      ev.tt2[i] = (q2 - ev.pf[i]).m2();
      for (int j = 3; j <= Nf; ++j) ev.ttxy[i][j] = (q1 - ev.pf[i] - ev.pf[j]).m2();
    }
  }
  ev.m2   = ev.pf[0].m2();
  ev.Y    = ev.pf[0].rap();
  ev.Pt   = ev.pf[0].pt();
  return true;
}

// Central particles from the 2x2 linear system (MContinuum.cc:438-550, Kf = 2):
// 2 p_a = q - w, 2 p_b = -q - w with w = p1T + p2T, then (pz, E) from rapidity.
void central_pair(const V4 &q, const V4 &p1, const V4 &p2, const real m[2], const real y[2],
                  V4 out[2]) {
  const real wx = p1.x + p2.x, wy = p1.y + p2.y;
  const real px[2] = {0.5 * (q.x - wx), 0.5 * (-q.x - wx)};
  const real py[2] = {0.5 * (q.y - wy), 0.5 * (-q.y - wy)};
  for (int i = 0; i < 2; ++i) {
    const real mt = msqrt(m[i] * m[i] + px[i] * px[i] + py[i] * py[i]);
    out[i]          = V4(px[i], py[i], mt * std::sinh(y[i]), mt * std::cosh(y[i]));
  }
}

// Forward legs from the central system (MContinuum.cc:372-384); false when the
// event fails the crude energy check or the forward-direction check.
bool forward_legs(const Setup &S, real pt1, real phi1x, real phi1y, real pt2,
                  real phi2x, real phi2y, const V4 &sumP, V4 &p1, V4 &p2, real m1, real m2) {
  const real p1z = solve_pz(m1, m2, pt1, pt2, sumP.z, sumP.e, S.s);
  const real p2z = -(sumP.z + p1z);
  if (p1z < 0 || p2z > 0) return false;
  p1 = V4(phi1x, phi1y, p1z, msqrt(m1 * m1 + pt1 * pt1 + p1z * p1z));
  p2 = V4(phi2x, phi2y, p2z, msqrt(m2 * m2 + pt2 * pt2 + p2z * p2z));
  return true;
}

// BNRandomKin + BNBuildKin for Kf = 2 (MContinuum.cc:276-435).
// Central particles of the <C> class with N = 4 or 6 central particles: transverse momenta
// from the linear system of MContinuum::BLinearSystem (MContinuum.cc:438-560),
//   2 p0 = q0 - w - (p2 + ... + p_{N-1}),  2 p1 = -q0 - w - (p2 + ... + p_{N-1}),
//   2 p_i = -q_{i-1} - w - (the sum of the p_j with j != i, i - 1),  i >= 2,  w = p1T + p2T,
// whose matrix the reference tabulates inverted; solved here by Gaussian elimination. (pz, E)
// from the rapidities and masses.
void central_n(int N, const V4 *q, const V4 &p1, const V4 &p2, const real *m, const real *y,
               V4 *out) {
  real Mx[6][7], My[6][7];
  const real wx = p1.x + p2.x, wy = p1.y + p2.y;
  for (int i = 0; i < N; ++i) {
    for (int j = 0; j < N; ++j) {
      real c = 1;
      if (i < 2) c = j == i ? 2 : (j < 2 ? 0 : 1);
      else c = j == i ? 2 : (j == i - 1 ? 0 : 1);
      Mx[i][j] = My[i][j] = c;
    }
    const V4 &qi = i == 0 ? q[0] : q[i - 1];
    const real sg = i == 0 ? 1.0 : -1.0;
    Mx[i][N] = sg * qi.x - wx;
    My[i][N] = sg * qi.y - wy;
  }
  real px[6], py[6];
  for (auto *Mp : {&Mx, &My}) {
    real (&M)[6][7] = *Mp;
    for (int c = 0; c < N; ++c) {
      int piv = c;
      for (int r = c + 1; r < N; ++r)
        if (std::fabs(M[r][c]) > std::fabs(M[piv][c])) piv = r;
      for (int k = 0; k <= N; ++k) std::swap(M[c][k], M[piv][k]);
      for (int r = 0; r < N; ++r) {
        if (r == c) continue;
        const real f = M[r][c] / M[c][c];
        for (int k = 0; k <= N; ++k) M[r][k] -= f * M[c][k];
      }
    }
    real *dst = Mp == &Mx ? px : py;
    for (int i = 0; i < N; ++i) dst[i] = M[i][N] / M[i][i];
  }
  for (int i = 0; i < N; ++i) {
    const real mt = msqrt(m[i] * m[i] + px[i] * px[i] + py[i] * py[i]);
    out[i]          = V4(px[i], py[i], mt * std::sinh(y[i]), mt * std::cosh(y[i]));
  }
}

// BNRandomKin + BNBuildKin for N = 4 or 6 central particles (MContinuum.cc:276-435): forward
// legs u[0..3], kt u[4..N+2], azimuths u[N+3..2N+1], rapidities u[2N+2..3N+1].
bool build_kinematics_cn(const Setup &S, const real *u, Event &ev) {
  const int N = S.p.n_central;
  const grn_gencuts &g = S.p.gcuts;
  const real lo  = std::log(g.fpt_min + ZERO_EPS);
  const real hi  = std::log(g.fpt_max);
  const real pt1 = std::exp(lo + (hi - lo) * u[0]);
  const real pt2 = std::exp(lo + (hi - lo) * u[1]);
  const real phi1 = 2.0 * PI * u[2];
  const real phi2 = 2.0 * PI * u[3];
  for (int i = 0; i < N - 1; ++i) {
    const real kt = g.kt_min + (g.kt_max - g.kt_min) * u[4 + i];
    const real ph = 2.0 * PI * u[N + 3 + i];
    ev.kq[i] = V4(kt * std::cos(ph), kt * std::sin(ph), 0, 0);
  }
  real y[6];
  for (int i = 0; i < N; ++i) y[i] = g.rap_min + (g.rap_max - g.rap_min) * u[2 * N + 2 + i];
  V4 p1(pt1 * std::cos(phi1), pt1 * std::sin(phi1), 0, 0);
  V4 p2(pt2 * std::cos(phi2), pt2 * std::sin(phi2), 0, 0);
  V4 c[6];
  real mc[6];
  for (int i = 0; i < N; ++i) mc[i] = S.p.m_central[i];
  central_n(N, ev.kq, p1, p2, mc, y, c);
  V4 sumP = c[0];
  for (int i = 1; i < N; ++i) sumP = sumP + c[i];
  if (sumP.e > S.sqrt_s) return false;
  forward_masses(S, 0, 0, 0, ev);
  if (!forward_legs(S, pt1, p1.x, p1.y, pt2, p2.x, p2.y, sumP, p1, p2, ev.mf1, ev.mf2))
    return false;
  ev.pf[0] = sumP;
  ev.pf[1] = p1;
  ev.pf[2] = p2;
  real msum = 0;
  for (int i = 0; i < N; ++i) {
    ev.pf[3 + i] = c[i];
    ev.leaf[i]   = c[i];
    msum += c[i].m();
  }
  if (sumP.m() < msum) return false;
  if (!check_emc((S.pb1 + S.pb2) - (p1 + p2 + sumP))) return false;
  return lorentz_scalars(S, ev);
}

void cascade_masses(const grn_process_params &p, const real *u, real &m3, real &m4);
void cascade_decays(const Setup &S, const real *u, real m3, real m4, Event &ev);

bool build_kinematics(const Setup &S, const real *u, Event &ev) {
  if (S.p.n_central >= 4) return build_kinematics_cn(S, u, ev);
  const grn_gencuts &g = S.p.gcuts;
  const real lo  = std::log(g.fpt_min + ZERO_EPS);
  const real hi  = std::log(g.fpt_max);
  const real pt1 = std::exp(lo + (hi - lo) * u[0]);
  const real pt2 = std::exp(lo + (hi - lo) * u[1]);
  const real phi1 = 2.0 * PI * u[2];
  const real phi2 = 2.0 * PI * u[3];
  const real kt   = g.kt_min + (g.kt_max - g.kt_min) * u[4];
  const real phik = 2.0 * PI * u[5];
  const real y[2] = {g.rap_min + (g.rap_max - g.rap_min) * u[6],
                       g.rap_min + (g.rap_max - g.rap_min) * u[7]};

  V4 p1(pt1 * std::cos(phi1), pt1 * std::sin(phi1), 0, 0);
  V4 p2(pt2 * std::cos(phi2), pt2 * std::sin(phi2), 0, 0);
  ev.q = V4(kt * std::cos(phik), kt * std::sin(phik), 0, 0);

  // central masses: the stable particles' masses, or the off-shell masses of a cascade
  // (BNRandomKin: GetOffShellMass of each first-level particle)
  real m[2] = {S.p.m_central[0], S.p.m_central[1]};
  if (S.p.n_decay == 2) cascade_masses(S.p, u, m[0], m[1]);
  V4 c[2];
  central_pair(ev.q, p1, p2, m, y, c);
  const V4 sumP = c[0] + c[1];
  if (sumP.e > S.sqrt_s) return false;
  // forward N* masses: u[8] (and u[9] for double excitation; the side draw for single)
  forward_masses(S, u[8], S.p.excitation == 2 ? u[9] : 0, S.p.excitation == 1 ? u[9] : 0, ev);
  if (!forward_legs(S, pt1, p1.x, p1.y, pt2, p2.x, p2.y, sumP, p1, p2, ev.mf1, ev.mf2))
    return false;

  ev.pf[0] = sumP;
  ev.pf[1] = p1;
  ev.pf[2] = p2;
  ev.pf[3] = c[0];
  ev.pf[4] = c[1];
  if (sumP.m() < c[0].m() + c[1].m()) return false;
  if (!check_emc((S.pb1 + S.pb2) - (p1 + p2 + sumP))) return false;
  // decay tree (BNBuildKin: ConstructDecayKinematics after the checks); the decays use the
  // mothers' masses from their 4-momenta (branch.p4.M())
  if (S.p.n_decay == 2) cascade_decays(S, u, c[0].m(), c[1].m(), ev);
  return lorentz_scalars(S, ev);
}

// Relativistic Breit-Wigner mass by inverse CDF in m^2, truncated to [max(M_MIN, m0 - n W),
// m0 + n W] with n = OFFSHELL widths (MRandom::RelativisticBWRandom, src/MRandom.cc:82-104),
// from the uniform R; n = 0 gives the pole mass.
real bw_mass(real m0, real W, real n, real M_MIN, real R) {
  if (W < 1e-40) return m0;
  const real m2    = m0 * m0;
  const real m2max = sq(m0 + n * W);
  const real m2min = std::max<real>(std::max<real>(0, M_MIN * M_MIN), sq(m0 - n * W));
  const real a = std::atan2(m2min - m2, m0 * W), b = std::atan2(m2max - m2, m0 * W);
  const real v = m2 + m0 * W * std::tan(a + R * (b - a));
  return std::max<real>(M_MIN, msqrt(v));
}

// OFFSHELL of a cascade: the process command's value, else 5 widths
// (include/Graniitti/MProcess.h:363, MProcess::SetOFFSHELL).
real offshell_widths(const grn_process_params &p) { return p.offshell_user ? p.offshell : 5.0; }

// First hypercube coordinate of the cascade decays: after the 8 of the 2-body point and,
// unless OFFSHELL = 0, the two Breit-Wigner mass draws.
int decay_coord(const grn_process_params &p) { return offshell_widths(p) > 0 ? 10 : 8; }

// Hypercube dimension of a process.
int point_dim(const grn_process_params &p) {
  if (p.n_central >= 4) return 3 * p.n_central + 2;  // 14 or 20
  if (p.excitation) return 10;
  return p.n_decay == 2 ? decay_coord(p) + 4 : 8;
}

// Forward N* masses (MProcess::SampleForwardMasses, src/MProcess.cc:1317-1365): M^2
// log-uniform in [1.09^2, xi_max s] from the class's mass coordinates; single excitation
// takes the side from a further draw (< 0.5: the first leg), lifted to the coordinate after.
// u_m: the mass coordinate(s); u_side: the side draw (single excitation).
void forward_masses(const Setup &S, real u_m0, real u_m1, real u_side, Event &ev) {
  ev.mf1 = ev.mf2 = S.p.m_beam;
  ev.ex1 = ev.ex2 = false;
  if (!S.p.excitation) return;
  const real lo = std::log(sq(1.09)), hi = std::log(S.p.xi_max * S.s);
  if (S.p.excitation == 1) {
    const real M = std::sqrt(std::exp(lo + (hi - lo) * u_m0));
    if (u_side < 0.5) {
      ev.mf1 = M;
      ev.ex1 = true;
    } else {
      ev.mf2 = M;
      ev.ex2 = true;
    }
  } else {
    ev.mf1 = std::sqrt(std::exp(lo + (hi - lo) * u_m0));
    ev.mf2 = std::sqrt(std::exp(lo + (hi - lo) * u_m1));
    ev.ex1 = ev.ex2 = true;
  }
}

// Off-shell masses of the two central particles of a cascade (GetOffShellMass, the
// daughters' mass sum + 1e-5 GeV bounding the Breit-Wigner from below) from u[8], u[9].
void cascade_masses(const grn_process_params &p, const real *u, real &m3, real &m4) {
  const real n = offshell_widths(p);
  m3 = p.m_central[0];
  m4 = p.m_central[1];
  if (n > 0) {
    m3 = bw_mass(m3, p.width[0], n, p.m_daughter[0] + p.m_daughter[1] + 1e-5, u[8]);
    m4 = bw_mass(m4, p.width[1], n, p.m_daughter[2] + p.m_daughter[3] + 1e-5, u[9]);
  }
}

// 2-body decay in the mother's rest frame with given (cos theta, phi), boosted to
// the lab (TwoBodyPhaseSpace + Isotropic + LorentzBoost,
// include/Graniitti/MKinematics.h:294-298, 384-459). Returns dPhi2 (MKinematics.h:267).
real two_body(const V4 &mother, real M0, real m3, real m4, real ct, real phi,
                V4 &p3, V4 &p4) {
  const real x = M0, y = m3, z = m4;
  const real pn = msqrt((x - y - z) * (x + y + z) * (x + y - z) * (x - y + z)) / (2.0 * x);
  const real st = msqrt(1.0 - ct * ct);
  const real k[3] = {pn * st * std::cos(phi), pn * st * std::sin(phi), pn * ct};
  V4 d[2] = {V4(k[0], k[1], k[2], msqrt(m3 * m3 + pn * pn)),
             V4(-k[0], -k[1], -k[2], msqrt(m4 * m4 + pn * pn))};
  const real b[3] = {mother.x / mother.e, mother.y / mother.e, mother.z / mother.e};
  const real gam = mother.e / M0;
  for (V4 &p : d) {
    const real k1 = b[0] * p.x + b[1] * p.y + b[2] * p.z;
    const real k2 = gam * (gam * k1 / (1.0 + gam) + p.e);
    p = V4(p.x + k2 * b[0], p.y + k2 * b[1], p.z + k2 * b[2], gam * (p.e + k1));
  }
  p3 = d[0];
  p4 = d[1];
  return 4.0 * PI * pn / (16.0 * PI * PI * M0);
}

// Isotropic two-body decays of the two central particles of a cascade, (cos theta, phi) from
// u[dec0..dec0 + 3] (ConstructDecayKinematics, src/MProcess.cc:1231-1283: TwoBodyPhaseSpace
// with FlatIsotropic draws in the mother's rest frame).
void cascade_decays(const Setup &S, const real *u, real m3, real m4, Event &ev) {
  const real *v = u + decay_coord(S.p);
  two_body(ev.pf[3], m3, S.p.m_daughter[0], S.p.m_daughter[1], 2.0 * v[0] - 1.0, 2.0 * PI * v[1],
           ev.leaf[0], ev.leaf[1]);
  two_body(ev.pf[4], m4, S.p.m_daughter[2], S.p.m_daughter[3], 2.0 * v[2] - 1.0, 2.0 * PI * v[3],
           ev.leaf[2], ev.leaf[3]);
}

// LorentzBoost (include/Graniitti/MKinematics.h:384-401), sign +1: p from the rest frame of
// the system b (mass M0) to the frame where b has its given momentum.
V4 boost_from_rest(const V4 &b, real M0, const V4 &p) {
  const real bx = b.x / b.e, by = b.y / b.e, bz = b.z / b.e;
  const real gam = b.e / M0;
  const real k1  = bx * p.x + by * p.y + bz * p.z;
  const real k2  = gam * (gam * k1 / (1.0 + gam) + p.e);
  return V4(p.x + k2 * bx, p.y + k2 * by, p.z + k2 * bz, gam * (p.e + k1));
}

// Flat N-body phase space, weighted (NBodySetup with unweight = false + NBodyPhaseSpace,
// include/Graniitti/MKinematics.h:523-691) for N = 4 or 6, the reference's generator draws
// taken from r: r[0..N-3] the intermediate masses (sorted ascending), then (cos theta, phi)
// pairs for particles N-1, ..., 1. Returns the weight prod(p*) x volume, or -1.
real n_body(int N, const V4 &mother, real M0, const real *m, const real *r, V4 *p) {
  real sum[6];
  for (int i = 0; i < N; ++i) sum[i] = (i ? sum[i - 1] : 0.0) + m[i];
  const real D = M0 - sum[N - 1];
  if (!(D > 0)) return -1.0;
  real rv[4];
  for (int i = 0; i < N - 2; ++i) rv[i] = r[i];
  std::sort(rv, rv + N - 2);
  real Meff[6];
  Meff[0]     = m[0];
  Meff[N - 1] = M0;
  for (int i = 1; i < N - 1; ++i) Meff[i] = sum[i] + rv[i - 1] * D;
  real pn[6] = {0, 0, 0, 0, 0, 0};
  real w = 1.0;
  for (int i = 1; i < N; ++i) {
    const real x = Meff[i], y = Meff[i - 1], z = m[i];
    pn[i] = msqrt((x - y - z) * (x + y + z) * (x + y - z) * (x - y + z)) / (2.0 * x);
    w *= pn[i];
  }
  real fact = 1.0;
  for (int i = 2; i <= N - 2; ++i) fact *= i;
  const real volume = 1.0 / (2.0 * std::pow(2.0 * PI, 2 * N - 3)) * std::pow(D, N - 2) / fact / M0;
  V4 k = mother;
  for (int i = N - 1, j = N - 2; i >= 1; --i, j += 2) {
    const real ct = 2.0 * r[j] - 1.0;
    const real st = msqrt(1.0 - ct * ct);
    const real ph = 2.0 * PI * r[j + 1];
    const V4 q(pn[i] * st * std::cos(ph), pn[i] * st * std::sin(ph), pn[i] * ct,
               msqrt(m[i] * m[i] + pn[i] * pn[i]));
    p[i] = boost_from_rest(k, k.m(), q);
    k = k - p[i];
  }
  p[0] = k;
  return w * volume;
}

// B51RandomKin + B51BuildKin for a 2-body central state, decay angles taken from
// u[6] (cos theta = 2 u6 - 1) and u[7] (phi = 2 pi u7) (MFactorized.cc:245-412).
bool build_kinematics_F(const Setup &S, const real *u, Event &ev) {
  const grn_gencuts &g = S.p.gcuts;
  const real lo  = std::log(g.fpt_min + ZERO_EPS);
  const real hi  = std::log(g.fpt_max);
  const real pt1 = std::exp(lo + (hi - lo) * u[0]);
  const real pt2 = std::exp(lo + (hi - lo) * u[1]);
  const real phi1 = 2.0 * PI * u[2];
  const real phi2 = 2.0 * PI * u[3];
  const real yX   = g.Y_min + (g.Y_max - g.Y_min) * u[4];
  real m3 = S.p.m_central[0], m4 = S.p.m_central[1];
  if (S.p.n_decay == 2) cascade_masses(S.p, u, m3, m4);  // off-shell central masses
  real msum = m3 + m4;
  if (S.p.n_central >= 4) {  // M_sum in the decay-list order (MFactorized.cc:265-270)
    msum = 0;
    for (int i = 0; i < S.p.n_central; ++i) msum += S.p.m_central[i];
  }
  const real Mmin = std::max<real>(msum + 1e-4, g.M_min);
  const real Mmax = std::min<real>(S.sqrt_s - (S.pb1.m() + S.pb2.m()), g.M_max);
  if (!(Mmin < Mmax)) return false;
  const real m2X  = Mmin * Mmin + (Mmax * Mmax - Mmin * Mmin) * u[5];
  ev.m2lo = Mmin * Mmin;
  ev.m2hi = Mmax * Mmax;
  V4 p1(pt1 * std::cos(phi1), pt1 * std::sin(phi1), 0, 0);
  V4 p2(pt2 * std::cos(phi2), pt2 * std::sin(phi2), 0, 0);
  V4 pX(-(p1.x + p2.x), -(p1.y + p2.y), 0, 0);
  const real mtX = msqrt(m2X + pX.pt2());
  pX.z = mtX * std::sinh(yX);
  pX.e = mtX * std::cosh(yX);
  // forward N* masses: u[6] (and u[7] for double excitation; the side draw u[7] for single)
  forward_masses(S, u[6], S.p.excitation == 2 ? u[7] : 0, S.p.excitation == 1 ? u[7] : 0, ev);
  if (pX.e > S.sqrt_s - (ev.mf1 + ev.mf2)) return false;  // MFactorized.cc:321
  if (!forward_legs(S, pt1, p1.x, p1.y, pt2, p2.x, p2.y, pX, p1, p2, ev.mf1, ev.mf2))
    return false;
  ev.pf[0] = pX;
  ev.pf[1] = p1;
  ev.pf[2] = p2;
  if (!check_emc((S.pb1 + S.pb2) - (p1 + p2 + pX))) return false;
  if (S.p.n_central >= 4) {
    const int N = S.p.n_central;
    real mc[6];
    for (int i = 0; i < N; ++i) mc[i] = S.p.m_central[i];
    ev.dw = n_body(N, pX, msqrt(m2X), mc, u + 6, ev.pf + 3);
    if (!(ev.dw >= 0)) return false;
    for (int k = 0; k < N; ++k) ev.leaf[k] = ev.pf[3 + k];
    return lorentz_scalars(S, ev);
  }
  // decay angles: the draws after the forward masses (u[6], u[7]; u[8], u[9] when excited)
  const int da = S.p.excitation ? 8 : 6;
  ev.dw = two_body(pX, msqrt(m2X), m3, m4, 2.0 * u[da] - 1.0, 2.0 * PI * u[da + 1], ev.pf[3],
                   ev.pf[4]);
  if (S.p.n_decay == 2) cascade_decays(S, u, m3, m4, ev);
  return lorentz_scalars(S, ev);
}

// LoopKinematics for Kf = 2 (MContinuum.cc:94-161): new forward transverse momenta,
// central pair re-solved with the tree-level difference momentum, rapidities and
// masses of the tree-level central particles.
bool loop_kinematics(const Setup &S, const Event &born, real p1x, real p1y, real p2x,
                     real p2y, Event &ev) {
  const V4 p1T(p1x, p1y, 0, 0), p2T(p2x, p2y, 0, 0);
  if (S.p.phase_space == GRN_PS_FACTORIZED) {
    // MFactorized::LoopKinematics (src/MFactorized.cc:84-139): the central system keeps
    // its mass and rapidity, its pT balances the new forward legs; the decay products
    // keep their tree-level momenta.
    const real mX = born.pf[0].m(), yX = born.pf[0].rap();
    V4 pX(-(p1x + p2x), -(p1y + p2y), 0, 0);
    const real mtX = msqrt(mX * mX + pX.pt2());
    pX.z = mtX * std::sinh(yX);
    pX.e = mtX * std::cosh(yX);
    if (pX.e > S.sqrt_s - (born.mf1 + born.mf2)) return false;
    V4 p1, p2;
    if (!forward_legs(S, p1T.pt(), p1x, p1y, p2T.pt(), p2x, p2y, pX, p1, p2, born.mf1, born.mf2))
      return false;
    ev       = born;
    ev.pf[0] = pX;
    ev.pf[1] = p1;
    ev.pf[2] = p2;
    if (!check_emc((S.pb1 + S.pb2) - (p1 + p2 + pX))) return false;
    return lorentz_scalars(S, ev);
  }
  if (S.p.n_central >= 4) {
    // MContinuum::LoopKinematics: central transverse momenta re-solved with the tree-level
    // difference momenta, rapidities and masses
    const int N = S.p.n_central;
    real m4[6], y4[6];
    for (int i = 0; i < N; ++i) {
      m4[i] = born.pf[3 + i].m();
      y4[i] = born.pf[3 + i].rap();
    }
    V4 c[6];
    central_n(N, born.kq, p1T, p2T, m4, y4, c);
    V4 sumP = c[0];
    for (int i = 1; i < N; ++i) sumP = sumP + c[i];
    V4 p1, p2;
    if (!forward_legs(S, p1T.pt(), p1x, p1y, p2T.pt(), p2x, p2y, sumP, p1, p2, born.mf1,
                      born.mf2))
      return false;
    ev       = born;
    ev.pf[0] = sumP;
    ev.pf[1] = p1;
    ev.pf[2] = p2;
    for (int i = 0; i < N; ++i) ev.pf[3 + i] = c[i];
    if (!check_emc((S.pb1 + S.pb2) - (p1 + p2 + sumP))) return false;
    return lorentz_scalars(S, ev);
  }
  const real m[2] = {born.pf[3].m(), born.pf[4].m()};
  const real y[2] = {born.pf[3].rap(), born.pf[4].rap()};
  V4 c[2];
  central_pair(born.q, p1T, p2T, m, y, c);
  const V4 sumP = c[0] + c[1];
  const real pt1 = p1T.pt(), pt2 = p2T.pt();
  V4 p1, p2;
  if (!forward_legs(S, pt1, p1x, p1y, pt2, p2x, p2y, sumP, p1, p2, born.mf1, born.mf2))
    return false;
  ev.mf1   = born.mf1;
  ev.mf2   = born.mf2;
  ev.ex1   = born.ex1;
  ev.ex2   = born.ex2;
  ev.q     = born.q;
  ev.pf[0] = sumP;
  ev.pf[1] = p1;
  ev.pf[2] = p2;
  ev.pf[3] = c[0];
  ev.pf[4] = c[1];
  if (!check_emc((S.pb1 + S.pb2) - (p1 + p2 + sumP))) return false;
  return lorentz_scalars(S, ev);
}

// Regge continuum amplitude for a 2-body central state, sign +1
// (MRegge::ME4, src/MRegge.cc:394-438; PomPomProtonVertex 637-644).
cplx regge_me4(const Setup &S, const Event &ev) {
  const grn_regge_params &rp = S.p.regge;
  const real M2  = sq(S.p.m_central[0]);
  // PomPomProtonVertex (src/MRegge.cc:637-644): elastic, or the excited leg's inelastic vertex
  const real gin = std::sqrt(S.p.soft.g3P * S.p.soft.gN_P);
  const real FFA = ev.ex1 ? gin * proton_ff_inel(ev.t1, ev.pf[1].m2())
                          : S.p.soft.gN_P * proton_ff(S.p.soft, ev.t1);
  const real FFB = ev.ex2 ? gin * proton_ff_inel(ev.t2, ev.pf[2].m2())
                          : S.p.soft.gN_P * proton_ff(S.p.soft, ev.t2);
  const real g   = rp.c[0] / S.p.soft.gN_P;
  const cplx At = regge_prop(rp, ev.ss[1][3], ev.t1) * FFA * meson_ff(rp, ev.that, M2) * g *
                  (1.0 / (ev.that - M2)) * meson_ff(rp, ev.that, M2) * g *
                  regge_prop(rp, ev.ss[2][4], ev.t2) * FFB;
  const cplx Au = regge_prop(rp, ev.ss[1][4], ev.t1) * FFA * meson_ff(rp, ev.uhat, M2) * g *
                  (1.0 / (ev.uhat - M2)) * meson_ff(rp, ev.uhat, M2) * g *
                  regge_prop(rp, ev.ss[2][3], ev.t2) * FFB;
  return At + Au;
}


// Regge continuum amplitude for a 4-body central state (MRegge::ME6, src/MRegge.cc:470-534):
// all 24 orderings (a, b, c, d) of the central particles along the ladder (GetAmpPerm(4, 1),
// include/Graniitti/MMath.h:723-770), off-shell propagator masses of the first and third
// particle of the decay list.
cplx regge_me6(const Setup &S, const Event &ev) {
  const grn_regge_params &rp = S.p.regge;
  const real MA  = sq(S.p.m_central[0]), MB = sq(S.p.m_central[2]);
  // PomPomProtonVertex (src/MRegge.cc:637-644): elastic, or the excited leg's inelastic vertex
  const real gin = std::sqrt(S.p.soft.g3P * S.p.soft.gN_P);
  const real FFA = ev.ex1 ? gin * proton_ff_inel(ev.t1, ev.pf[1].m2())
                          : S.p.soft.gN_P * proton_ff(S.p.soft, ev.t1);
  const real FFB = ev.ex2 ? gin * proton_ff_inel(ev.t2, ev.pf[2].m2())
                          : S.p.soft.gN_P * proton_ff(S.p.soft, ev.t2);
  const real g   = rp.c[0] / S.p.soft.gN_P;
  int perm[4] = {3, 4, 5, 6};
  cplx A(0, 0);
  do {
    const int a = perm[0], b = perm[1], c = perm[2], d = perm[3];
    const real tab = ev.tt1[a], tbc = ev.ttxy[a][b], tcd = ev.tt2[d];
    A += regge_prop(rp, ev.ss[1][a], ev.t1) * FFA * meson_ff(rp, tab, MA) * g *
         (1.0 / (tab - MA)) * meson_ff(rp, tbc, MA) * g * regge_prop(rp, ev.ss[b][c], tbc) *
         meson_ff(rp, tbc, MB) * g * (1.0 / (tcd - MB)) * meson_ff(rp, tcd, MB) * g *
         regge_prop(rp, ev.ss[2][d], ev.t2) * FFB;
  } while (std::next_permutation(perm, perm + 4));
  return A;
}

// Regge continuum amplitude for a 6-body central state (MRegge::ME8, src/MRegge.cc:560-627):
// all 720 orderings (a, b, c, d, e, f) of the central particles along the ladder
// (GetAmpPerm(6, 1)), with the reference's invariants and form-factor arguments as it writes
// them: t_ab = (q1 - p_a)^2, t_bc = (q1 - p_a - p_b)^2, t_cd = (q1 - p_b - p_c)^2,
// t_de = (q1 - p_c - p_d)^2, t_ef = (q2 - p_f)^2; off-shell propagator masses of the first,
// third and fifth particle of the decay list.
cplx regge_me8(const Setup &S, const Event &ev) {
  const grn_regge_params &rp = S.p.regge;
  const real MA = sq(S.p.m_central[0]), MB = sq(S.p.m_central[2]), MC = sq(S.p.m_central[4]);
  const real gin = std::sqrt(S.p.soft.g3P * S.p.soft.gN_P);
  const real FFA = ev.ex1 ? gin * proton_ff_inel(ev.t1, ev.pf[1].m2())
                          : S.p.soft.gN_P * proton_ff(S.p.soft, ev.t1);
  const real FFB = ev.ex2 ? gin * proton_ff_inel(ev.t2, ev.pf[2].m2())
                          : S.p.soft.gN_P * proton_ff(S.p.soft, ev.t2);
  const real g   = rp.c[0] / S.p.soft.gN_P;
  int perm[6] = {3, 4, 5, 6, 7, 8};
  cplx A(0, 0);
  do {
    const int a = perm[0], b = perm[1], c = perm[2], d = perm[3], e = perm[4], f = perm[5];
    const real tab = ev.tt1[a], tbc = ev.ttxy[a][b], tcd = ev.ttxy[b][c];
    const real tde = ev.ttxy[c][d], tef = ev.tt2[f];
    A += regge_prop(rp, ev.ss[1][a], ev.t1) * FFA * meson_ff(rp, tab, MA) * g *
         (1.0 / (tab - MA)) * meson_ff(rp, tbc, MA) * g * regge_prop(rp, ev.ss[b][c], tbc) *
         meson_ff(rp, tbc, MB) * g * (1.0 / (tcd - MB)) * meson_ff(rp, tde, MB) * g *
         regge_prop(rp, ev.ss[d][e], tde) * meson_ff(rp, tde, MC) * g * (1.0 / (tef - MC)) *
         meson_ff(rp, tef, MC) * g * regge_prop(rp, ev.ss[2][f], ev.t2) * FFB;
  } while (std::next_permutation(perm, perm + 6));
  return A;
}

// ---------------------------------------------------------------------------
// Tensor-pomeron continuum of two pseudoscalars (MTensorPomeron::ME4, "2xS",
// src/MTensorPomeron.cc:572-898), restated with explicit Lorentz-index sums as the
// reference contracts them (covariant components, metric diag(+,-,-,-)).
constexpr real MP_PDG = 0.938272081;  // PDG::mp (include/Graniitti/MPDG.h:54)

// Sachs form factors and the Dirac form factor F1 (src/MForm.cc:541-645): Kelly
// (PRC 70, 068202) or dipole parametrisation.
real F1_em(real Q2, bool kelly) {
  Q2 = std::fabs(Q2);
  const real tau = Q2 / sq(2.0 * MP_PDG);
  const real mu  = 2.792847337;
  real GE, GM;
  if (kelly) {
    GE = (1.0 - 0.24 * tau) / (1.0 + 10.98 * tau + 12.82 * tau * tau + 21.97 * tau * tau * tau);
    GM = mu * (1.0 + 0.12 * tau) / (1.0 + 10.97 * tau + 18.86 * tau * tau + 6.55 * tau * tau * tau);
  } else {
    GM = mu / sq(1.0 + Q2 / 0.71);
    GE = GM / mu;
  }
  return 1.0 / (tau + 1.0) * GE + tau / (tau + 1.0) * GM;
}

typedef std::array<real, 4> L4;
L4 lower(const V4 &p) { return {p.e, -p.x, -p.y, -p.z}; }
const real G_METRIC[4] = {1.0, -1.0, -1.0, -1.0};

// Rank-2 vertex tensors (covariant).
struct T2 {
  cplx c[4][4];
};
// Proton-pomeron-proton, high-energy limit (MTensorPomeron.cc:1388-1399).
T2 vertex_ppP(const grn_process_params &p, const V4 &prime, const V4 &q) {
  const V4   ps = prime + q;
  const L4   l  = lower(ps);
  const cplx f  = cplx(0, -1) * 3.0 * p.tensor.gPNN * F1_em((prime - q).m2(), p.tensor.em_kelly);
  T2 T;
  for (int u = 0; u < 4; ++u)
    for (int v = 0; v < 4; ++v) T.c[u][v] = f * l[u] * l[v];
  return T;
}
// Pomeron-pseudoscalar-pseudoscalar (MTensorPomeron.cc:2203-2215).
T2 vertex_Pss(const grn_process_params &p, const V4 &prime, const V4 &q) {
  const V4     ps = prime + q;
  const L4     l  = lower(ps);
  const real M2 = ps.m2();
  const cplx   f  = cplx(0, -1) * 2.0 * p.tensor.gPps * (1.0 / (1.0 - (prime - q).m2() / 0.5));
  T2 T;
  for (int u = 0; u < 4; ++u)
    for (int v = 0; v < 4; ++v)
      T.c[u][v] = f * (l[u] * l[v] - 0.25 * (u == v ? G_METRIC[u] : 0.0) * M2);
  return T;
}
// Pomeron propagator factor 1/(4s) (-i s ap)^(alpha(t)-1) (MTensorPomeron.cc:2288-2298);
// its index structure g_uk g_vl + g_ul g_vk - g_uv g_kl / 2 is applied in contract().
cplx pomeron_prop(const grn_process_params &p, real s, real t) {
  const real a = 1.0 + p.tensor.delta_P + p.tensor.ap_P * t;
  return 1.0 / (4.0 * s) * std::pow(cplx(0, -s * p.tensor.ap_P), a - 1.0);
}
// A_{mu nu} D^{mu nu, alpha beta} B_{alpha beta} as plain index sums.
cplx contract(const T2 &A, cplx c, const T2 &B) {
  cplx sum(0, 0);
  for (int u = 0; u < 4; ++u)
    for (int v = 0; v < 4; ++v)
      for (int k = 0; k < 4; ++k)
        for (int l = 0; l < 4; ++l) {
          const real g = (u == k && v == l ? G_METRIC[u] * G_METRIC[v] : 0.0) +
                           (u == l && v == k ? G_METRIC[u] * G_METRIC[v] : 0.0) -
                           0.5 * (u == v ? G_METRIC[u] : 0.0) * (k == l ? G_METRIC[k] : 0.0);
          if (g != 0.0) sum += A.c[u][v] * g * B.c[k][l];
        }
  return c * sum;
}

cplx tensor_me4_2xs(const Setup &S, const Event &ev) {
  const grn_process_params &p = S.p;
  const V4 &pa = S.pb1, &pb = S.pb2;
  const V4 &p1 = ev.pf[1], &p2 = ev.pf[2], &p3 = ev.pf[3], &p4 = ev.pf[4];
  const real M2  = sq(p.m_central[0]);
  const V4     pt  = pa - p1 - p3;
  const V4     pu  = p4 - pa + p1;
  const V4     mp3 = V4(-p3.x, -p3.y, -p3.z, -p3.e);
  const T2     G1a = vertex_ppP(p, p1, pa);
  const T2     G2b = vertex_ppP(p, p2, pb);
  const cplx   Mt  = contract(G1a, pomeron_prop(p, ev.ss[1][3], ev.t1), vertex_Pss(p, pt, mp3)) *
                  contract(vertex_Pss(p, p4, pt), pomeron_prop(p, ev.ss[2][4], ev.t2), G2b) *
                  (cplx(0, 1) / (pt.m2() - M2)) * sq(meson_ff(p.regge, pt.m2(), M2));
  const cplx   Mu  = contract(G1a, pomeron_prop(p, ev.ss[1][4], ev.t1), vertex_Pss(p, p4, pu)) *
                  contract(vertex_Pss(p, pu, mp3), pomeron_prop(p, ev.ss[2][3], ev.t2), G2b) *
                  (cplx(0, 1) / (pu.m2() - M2)) * sq(meson_ff(p.regge, pu.m2(), M2));
  return cplx(0, -1) * (Mt + Mu);
}

// ---------------------------------------------------------------------------
// Tensor-pomeron resonances decaying to two pseudoscalars (MTensorPomeron::ME3,
// src/MTensorPomeron.cc:164-565), restated with explicit Lorentz-index sums in the
// reference's own order: rank-6 pomeron-pomeron-tensor vertex, tensor propagator,
// decay vertex, pomeron propagators and proton vertices, contracted as plain sums over
// index values (the reference's tensors carry the index positions that make these
// sums Lorentz contractions).
inline real gm(int u, int v) { return u == v ? G_METRIC[u] : 0.0; }
inline real up(const V4 &p, int u) { return u == 0 ? p.e : (u == 1 ? p.x : (u == 2 ? p.y : p.z)); }
inline real dn(const V4 &p, int u) { return u == 0 ? p.e : -up(p, u); }
inline int    i6(int u, int v, int k, int l, int r, int s) {
  return ((((u * 4 + v) * 4 + k) * 4 + l) * 4 + r) * 4 + s;
}

// Auxiliary tensor R_{abcd} = g_ac g_bd / 2 + g_ad g_bc / 2 + g_ab g_cd / 4 with the sign of
// the last term as MTensorPomeron::CalcRTensor sets it (src/MTensorPomeron.cc:2563-2564).
real R_dddd(int a, int b, int c, int d) {
  return 0.5 * gm(a, c) * gm(b, d) + 0.5 * gm(a, d) * gm(b, c) + 0.25 * gm(a, b) * gm(c, d);
}

// Coupling structure #0 of the pomeron-pomeron-tensor vertex, kinematics independent:
// 2 i S0 R_{uv,s1 v1} R_{kl,v1 l1} R_{rs,l1 s1} with the three contractions carried by
// metric factors (iG_PPT_00, src/MTensorPomeron.cc:1701-1731).
const std::vector<cplx> &ppt_structure0() {
  static const std::vector<cplx> T = [] {
    std::vector<cplx> t(4096, cplx(0, 0));
    const cplx f(0, 2.0);
    for (int u = 0; u < 4; ++u)
      for (int v = 0; v < 4; ++v)
        for (int k = 0; k < 4; ++k)
          for (int l = 0; l < 4; ++l)
            for (int r = 0; r < 4; ++r)
              for (int s = 0; s < 4; ++s) {
                cplx sum(0, 0);
                for (int v1 = 0; v1 < 4; ++v1)
                  for (int l1 = 0; l1 < 4; ++l1)
                    for (int s1 = 0; s1 < 4; ++s1)
                      sum += f * R_dddd(u, v, s1, v1) * R_dddd(k, l, v1, l1) *
                             R_dddd(r, s, l1, s1) * G_METRIC[v1] * G_METRIC[l1] * G_METRIC[s1];
                t[i6(u, v, k, l, r, s)] = sum;
              }
    return t;
  }();
  return T;
}

// Mixed-position versions of R (MTensorPomeron::CalcRTensor, :2566-2569): raised indices
// carry the metric factor of their slot.
real R_dddu(int a, int b, int c, int d) { return R_dddd(a, b, c, d) * G_METRIC[d]; }
real R_dduu(int a, int b, int c, int d) {
  return R_dddd(a, b, c, d) * G_METRIC[c] * G_METRIC[d];
}
real R_uudd(int a, int b, int c, int d) {
  return R_dddd(a, b, c, d) * G_METRIC[a] * G_METRIC[b];
}
inline int i8(int u, int v, int k, int l, int r, int s, int a, int b) {
  return i6(u, v, k, l, r, s) * 16 + a * 4 + b;
}

// Pre-contracted R products of coupling structures #1, #2 (the FIX1/FIX2/FIX3 tensors of
// MTensorPomeron::CalcRTensor, :2583-2631).
struct PPTFix {
  std::vector<real> T1, T2, T3;
  PPTFix() : T1(4096, 0.0), T2(65536, 0.0), T3(65536, 0.0) {
    for (int u = 0; u < 4; ++u)
      for (int v = 0; v < 4; ++v)
        for (int k = 0; k < 4; ++k)
          for (int l = 0; l < 4; ++l)
            for (int r = 0; r < 4; ++r)
              for (int s = 0; s < 4; ++s)
                for (int a1 = 0; a1 < 4; ++a1)
                  for (int x = 0; x < 4; ++x)
                    for (int y = 0; y < 4; ++y) {
                      // T1: sum over a1, r1 = x, s1 = y
                      T1[i6(u, v, k, l, r, s)] +=
                          R_dddd(u, v, x, a1) * R_dddu(k, l, y, a1) * R_dduu(r, s, x, y);
                    }
    for (int u = 0; u < 4; ++u)
      for (int v = 0; v < 4; ++v)
        for (int k = 0; k < 4; ++k)
          for (int l = 0; l < 4; ++l)
            for (int r = 0; r < 4; ++r)
              for (int s = 0; s < 4; ++s)
                for (int a1 = 0; a1 < 4; ++a1)
                  for (int m = 0; m < 4; ++m)
                    for (int n = 0; n < 4; ++n) {
                      // T2(.., u1 = m, r1 = n) = sum_{a1, s1} R(u,v,u1,a1) R_DDDU(k,l,s1,a1)
                      //                                       R_DDUU(r,s,r1,s1)
                      // T3(.., u1 = m, s1 = n) = sum_{a1, r1} R(u,v,r1,a1) R_DDDU(k,l,u1,a1)
                      //                                       R_DDUU(r,s,r1,s1)
                      for (int j = 0; j < 4; ++j) {
                        T2[i8(u, v, k, l, r, s, m, n)] +=
                            R_dddd(u, v, m, a1) * R_dddu(k, l, j, a1) * R_dduu(r, s, n, j);
                        T3[i8(u, v, k, l, r, s, m, n)] +=
                            R_dddd(u, v, j, a1) * R_dddu(k, l, m, a1) * R_dduu(r, s, j, n);
                      }
                    }
  }
};
const PPTFix &ppt_fix() {
  static const PPTFix F;
  return F;
}

// Kinematics-dependent coupling structures #1..#6 (iG_PPT_12 :1738-1780, iG_PPT_03
// :1786-1834, iG_PPT_04 :1839-1906, iG_PPT_05 :1911-1983, iG_PPT_06 :1988-2014), each with its
// coupling g applied, added into T.
void ppt_structures(const V4 &q1, const V4 &q2, const real *g, std::vector<cplx> &T) {
  const real q1q2 = q1.e * q2.e - (q1.x * q2.x + q1.y * q2.y + q1.z * q2.z);
  const PPTFix &F   = ppt_fix();
  const real  EPS = 1e-6;  // structures with |g| <= 1e-6 are skipped (:1659-1670)
  for (int mode = 1; mode <= 2; ++mode) {
    if (!(std::fabs(g[mode]) > EPS)) continue;
    const cplx   f    = cplx(0, -2.0) * g[mode];
    const real sign = mode == 1 ? -1.0 : 1.0;
    for (int u = 0; u < 4; ++u)
      for (int v = 0; v < 4; ++v)
        for (int k = 0; k < 4; ++k)
          for (int l = 0; l < 4; ++l)
            for (int r = 0; r < 4; ++r)
              for (int s = 0; s < 4; ++s) {
                real t = q1q2 * F.T1[i6(u, v, k, l, r, s)];
                for (int a = 0; a < 4; ++a)
                  for (int b = 0; b < 4; ++b) {
                    t += sign * up(q2, a) * dn(q1, b) * F.T2[i8(u, v, k, l, r, s, a, b)];
                    t += sign * up(q1, a) * dn(q2, b) * F.T3[i8(u, v, k, l, r, s, a, b)];
                    t += dn(q1, a) * dn(q2, b) * R_dddd(u, v, k, l) * R_dduu(r, s, a, b);
                  }
                T[i6(u, v, k, l, r, s)] += f * t;
              }
  }
  if (std::fabs(g[3]) > EPS) {
    const cplx f = cplx(0, -1.0) * g[3];
    real A[4][4][4] = {}, B[4][4][4] = {};
    for (int u = 0; u < 4; ++u)
      for (int v = 0; v < 4; ++v)
        for (int k = 0; k < 4; ++k)
          for (int x = 0; x < 4; ++x) {
            A[u][v][k] += up(q2, x) * R_dddd(u, v, x, k);
            B[u][v][k] += up(q1, x) * R_dddd(u, v, x, k);
          }
    for (int u = 0; u < 4; ++u)
      for (int v = 0; v < 4; ++v)
        for (int k = 0; k < 4; ++k)
          for (int l = 0; l < 4; ++l)
            for (int r = 0; r < 4; ++r)
              for (int s = 0; s < 4; ++s) {
                real t = 0;
                for (int v1 = 0; v1 < 4; ++v1)
                  for (int l1 = 0; l1 < 4; ++l1)
                    t += (A[u][v][v1] * B[k][l][l1] + A[u][v][l1] * B[k][l][v1]) *
                         R_uudd(v1, l1, r, s);
                T[i6(u, v, k, l, r, s)] += f * t;
              }
  }
  if (std::fabs(g[4]) > EPS) {
    const cplx f = cplx(0, -2.0) * g[4];
    real A[4][4][4][4] = {}, B[4][4][4][4] = {}, C[4][4] = {};
    for (int u = 0; u < 4; ++u)
      for (int v = 0; v < 4; ++v)
        for (int k = 0; k < 4; ++k)
          for (int l = 0; l < 4; ++l)
            for (int u1 = 0; u1 < 4; ++u1)
              for (int v1 = 0; v1 < 4; ++v1)
                for (int a1 = 0; a1 < 4; ++a1) {
                  A[u][v][k][l] += up(q2, v1) * R_dddd(u, v, v1, a1) * up(q1, u1) *
                                   R_dddu(k, l, u1, a1);
                  B[u][v][k][l] += up(q2, u1) * R_dddd(u, v, u1, a1) * up(q1, v1) *
                                   R_dddu(k, l, v1, a1);
                }
    for (int r = 0; r < 4; ++r)
      for (int s = 0; s < 4; ++s)
        for (int a1 = 0; a1 < 4; ++a1)
          for (int l1 = 0; l1 < 4; ++l1) C[r][s] += dn(q1, a1) * dn(q2, l1) * R_uudd(a1, l1, r, s);
    for (int u = 0; u < 4; ++u)
      for (int v = 0; v < 4; ++v)
        for (int k = 0; k < 4; ++k)
          for (int l = 0; l < 4; ++l)
            for (int r = 0; r < 4; ++r)
              for (int s = 0; s < 4; ++s)
                T[i6(u, v, k, l, r, s)] +=
                    f * (A[u][v][k][l] + B[u][v][k][l] - 2.0 * q1q2 * R_dddd(u, v, k, l)) * C[r][s];
  }
  if (std::fabs(g[5]) > EPS) {
    const cplx f = cplx(0, 1.0) * g[5];
    real A[4][4][4][4] = {}, C[4][4][4][4] = {}, B[4][4] = {}, D[4][4] = {};
    for (int u = 0; u < 4; ++u)
      for (int v = 0; v < 4; ++v)
        for (int r = 0; r < 4; ++r)
          for (int s = 0; s < 4; ++s)
            for (int u1 = 0; u1 < 4; ++u1)
              for (int v1 = 0; v1 < 4; ++v1)
                for (int r1 = 0; r1 < 4; ++r1) {
                  A[u][v][r][s] += up(q2, u1) * R_dddd(u, v, u1, v1) * dn(q2, r1) *
                                   R_uudd(v1, r1, r, s);
                  C[u][v][r][s] += up(q1, u1) * R_dddd(u, v, u1, v1) * dn(q1, r1) *
                                   R_uudd(v1, r1, r, s);
                }
    for (int a = 0; a < 4; ++a)
      for (int b = 0; b < 4; ++b)
        for (int c = 0; c < 4; ++c)
          for (int d = 0; d < 4; ++d) {
            B[a][b] += up(q1, c) * up(q1, d) * R_dddd(a, b, c, d);
            D[a][b] += up(q2, c) * up(q2, d) * R_dddd(a, b, c, d);
          }
    for (int u = 0; u < 4; ++u)
      for (int v = 0; v < 4; ++v)
        for (int k = 0; k < 4; ++k)
          for (int l = 0; l < 4; ++l)
            for (int r = 0; r < 4; ++r)
              for (int s = 0; s < 4; ++s)
                T[i6(u, v, k, l, r, s)] +=
                    f * (A[u][v][r][s] * B[k][l] + C[k][l][r][s] * D[u][v]);
  }
  if (std::fabs(g[6]) > EPS) {
    const cplx f = cplx(0, -2.0) * g[6];
    real A[4][4] = {}, B[4][4] = {}, C[4][4] = {};
    for (int a = 0; a < 4; ++a)
      for (int b = 0; b < 4; ++b)
        for (int c = 0; c < 4; ++c)
          for (int d = 0; d < 4; ++d) {
            A[a][b] += up(q2, c) * up(q2, d) * R_dddd(a, b, c, d);
            B[a][b] += up(q1, c) * up(q1, d) * R_dddd(a, b, c, d);
            C[a][b] += up(q1, c) * up(q2, d) * R_dddd(a, b, c, d);
          }
    for (int u = 0; u < 4; ++u)
      for (int v = 0; v < 4; ++v)
        for (int k = 0; k < 4; ++k)
          for (int l = 0; l < 4; ++l)
            for (int r = 0; r < 4; ++r)
              for (int s = 0; s < 4; ++s)
                T[i6(u, v, k, l, r, s)] += f * A[u][v] * B[k][l] * C[r][s];
  }
}

// Resonance form factor exp(-(q^2 - M0^2)^2 / Lambda^4) (MTensorPomeron::F, :2489) and the
// pion-electromagnetic-type FM(q^2) = 1 / (1 - q^2 / Lambda^2) with Lambda^2 = 1 (:2485).
real ff_res(real q2, real M0) { return std::exp(-sq(q2 - M0 * M0)); }
real ff_M(real q2) { return 1.0 / (1.0 - q2 / 1.0); }

cplx tensor_me3(const Setup &S, const Event &ev) {
  const grn_process_params &p = S.p;
  const V4 &pa = S.pb1, &pb = S.pb2;
  const V4 &p1 = ev.pf[1], &p2 = ev.pf[2], &p3 = ev.pf[3], &p4 = ev.pf[4];
  const V4 &X  = ev.pf[0];
  const V4  q1 = pa - p1, q2 = pb - p2;
  // X1^{ab} = iG_1a(mu, nu) iDP_1(mu, nu, a, b), X2 likewise (pomeron propagators iD_P(s_i,
  // t_i) with s_i = (p_i + X)^2, src/MTensorPomeron.cc:196-197, 2288-2298)
  const T2   G1a = vertex_ppP(p, p1, pa);
  const T2   G2b = vertex_ppP(p, p2, pb);
  const cplx c1  = pomeron_prop(p, ev.ss[1][0], ev.t1);
  const cplx c2  = pomeron_prop(p, ev.ss[2][0], ev.t2);
  cplx X1[4][4], X2[4][4];
  for (int a = 0; a < 4; ++a)
    for (int b = 0; b < 4; ++b) {
      cplx s1(0, 0), s2(0, 0);
      for (int u = 0; u < 4; ++u)
        for (int v = 0; v < 4; ++v) {
          const real g = gm(u, a) * gm(v, b) + gm(u, b) * gm(v, a) - 0.5 * gm(u, v) * gm(a, b);
          if (g == 0.0) continue;
          s1 += G1a.c[u][v] * g;
          s2 += G2b.c[u][v] * g;
        }
      X1[a][b] = c1 * s1;
      X2[a][b] = c2 * s2;
    }
  const real m2   = X.m2();
  const real Ft   = ff_M(q1.m2()) * ff_M(q2.m2());  // times F((q1+q2)^2, M0) per resonance
  const V4     q12  = q1 + q2;
  cplx         A(0, 0);
  for (int r = 0; r < p.n_res; ++r) {
    const grn_resonance &R = p.res[r];
    const real F_tilde   = Ft * ff_res(q12.m2(), R.M);
    const cplx   Delta     = 1.0 / cplx(m2 - R.M * R.M, R.M * R.W);
    cplx cvtx[4][4][4][4];
    if (R.J == 2) {
      // tensor propagator, upper indices (iD_TMES, :2422-2446) x decay vertex (iG_f2psps,
      // :2121-2137), then the rank-6 vertex (iG_PPT_total, :1646-1692; only #0 is used)
      auto ghat = [&](int u, int v) { return -gm(u, v) + up(X, u) * up(X, v) / m2; };
      const V4   k   = p3 - p4;
      const cplx fd  = cplx(0, -1) * R.g_decay / 2.0 * ff_res((p3 + p4).m2(), R.M);
      const real k2 = k.m2();
      cplx dec[4][4];
      for (int u = 0; u < 4; ++u)
        for (int v = 0; v < 4; ++v) dec[u][v] = fd * (dn(k, u) * dn(k, v) - 0.25 * gm(u, v) * k2);
      cplx D[4][4];
      for (int u = 0; u < 4; ++u)
        for (int v = 0; v < 4; ++v) {
          cplx sum(0, 0);
          for (int a = 0; a < 4; ++a)
            for (int b = 0; b < 4; ++b)
              sum += cplx(0, 1) * Delta *
                     (0.5 * (ghat(u, a) * ghat(v, b) + ghat(u, b) * ghat(v, a)) -
                      1.0 / 3.0 * ghat(u, v) * ghat(a, b)) *
                     dec[a][b];
          D[u][v] = sum;
        }
      const std::vector<cplx> &G0 = ppt_structure0();
      std::vector<cplx>        Gt(4096);
      for (int i = 0; i < 4096; ++i) Gt[i] = G0[i] * R.g_tensor[0];
      real gt[7];
      for (int j = 0; j < 7; ++j) gt[j] = R.g_tensor[j];
      ppt_structures(q1, q2, gt, Gt);
      for (int u = 0; u < 4; ++u)
        for (int v = 0; v < 4; ++v)
          for (int k_ = 0; k_ < 4; ++k_)
            for (int l = 0; l < 4; ++l) {
              cplx sum(0, 0);
              for (int a = 0; a < 4; ++a)
                for (int b = 0; b < 4; ++b) sum += Gt[i6(u, v, k_, l, a, b)] * F_tilde * D[a][b];
              cvtx[u][v][k_][l] = sum;
            }
    } else {
      // scalar: (g0 iG_PPS_0 + iG_PPS_1) F_tilde (:1492-1571) x iD_MES (:2383-2387) x
      // iG_f0ss (:2028-2038)
      const real q1q2 = q1.e * q2.e - (q1.x * q2.x + q1.y * q2.y + q1.z * q2.z);
      const cplx   f1   = cplx(0, 1) * R.g_tensor[1] / 2.0;
      const cplx   tail = cplx(0, 1) * Delta * cplx(0, 1) * R.g_decay * ff_res((p3 + p4).m2(), R.M);
      for (int u = 0; u < 4; ++u)
        for (int v = 0; v < 4; ++v)
          for (int k_ = 0; k_ < 4; ++k_)
            for (int l = 0; l < 4; ++l) {
              const real gg = gm(u, k_) * gm(v, l) + gm(u, l) * gm(v, k_);
              const cplx   t0 = cplx(0, 1) * (gg - 0.5 * gm(u, v) * gm(k_, l));
              const cplx   t1 = f1 * (dn(q1, k_) * dn(q2, u) * gm(v, l) + dn(q1, k_) * dn(q2, v) * gm(u, l) +
                                    dn(q1, l) * dn(q2, u) * gm(v, k_) + dn(q1, l) * dn(q2, v) * gm(u, k_) -
                                    2.0 * q1q2 * gg);
              cvtx[u][v][k_][l] = (R.g_tensor[0] * t0 + t1) * F_tilde * tail;
            }
    }
    cplx sum(0, 0);
    for (int a = 0; a < 4; ++a)
      for (int b = 0; b < 4; ++b)
        for (int c = 0; c < 4; ++c)
          for (int d = 0; d < 4; ++d) sum += X1[a][b] * cvtx[a][b][c][d] * X2[c][d];
    A += cplx(0, -1) * sum;
  }
  return A;
}

// ---------------------------------------------------------------------------
// Tensor-pomeron continuum of two vector mesons, "2xV" (MTensorPomeron::ME4,
// src/MTensorPomeron.cc:808-888), with the explicit index sums of the reference.
typedef std::array<std::array<std::array<std::array<cplx, 4>, 4>, 4>, 4> T4;

// Gamma^(0) and Gamma^(2) of the pomeron-vector-vector vertex (:2500-2529).
real vv_gamma0(const V4 &k1, const V4 &k2, int u, int v, int k, int l) {
  const real k1k2 = k1.e * k2.e - (k1.x * k2.x + k1.y * k2.y + k1.z * k2.z);
  return (k1k2 * gm(u, v) - dn(k2, u) * dn(k1, v)) *
         (dn(k1, k) * dn(k2, l) + dn(k2, k) * dn(k1, l) - 0.5 * k1k2 * gm(k, l));
}
real vv_gamma2(const V4 &k1, const V4 &k2, int u, int v, int k, int l) {
  const real k1k2 = k1.e * k2.e - (k1.x * k2.x + k1.y * k2.y + k1.z * k2.z);
  return k1k2 * (gm(u, k) * gm(v, l) + gm(u, l) * gm(v, k)) +
         gm(u, v) * (dn(k1, k) * dn(k2, l) + dn(k2, k) * dn(k1, l)) -
         dn(k1, v) * dn(k2, l) * gm(u, k) - dn(k1, v) * dn(k2, k) * gm(u, l) -
         dn(k2, u) * dn(k1, l) * gm(v, k) - dn(k2, u) * dn(k1, k) * gm(v, l) -
         (k1k2 * gm(u, v) - dn(k2, u) * dn(k1, v)) * gm(k, l);
}
// i Gamma_{alpha beta gamma delta}(p', p) = i FM((p' - p)^2, 0.5) (2 g1 Gamma0(p', -p) -
// g2 Gamma2(p', -p)) (iG_Pvv, :2224-2237).
T4 vertex_Pvv(const grn_process_params &p, const V4 &prime, const V4 &q) {
  const V4   mq(-q.x, -q.y, -q.z, -q.e);
  const cplx f = cplx(0, 1) * (1.0 / (1.0 - (prime - q).m2() / 0.5));
  T4 T;
  for (int u = 0; u < 4; ++u)
    for (int v = 0; v < 4; ++v)
      for (int k = 0; k < 4; ++k)
        for (int l = 0; l < 4; ++l)
          T[u][v][k][l] = f * (2.0 * p.tensor.gPvv[0] * vv_gamma0(prime, mq, u, v, k, l) -
                               p.tensor.gPvv[1] * vv_gamma2(prime, mq, u, v, k, l));
  return T;
}
// Reggeized vector propagator factor -1/(m^2 - M0^2) (e^{i phi} s34 / (4 M0^2))^(alpha - 1)
// with alpha = 0.5 + 0.9 m^2 (iD_V, :2353-2369); its index structure g^{uv} is applied in
// the contraction.
cplx vector_prop(const V4 &p, real M0, real s34) {
  const real m2    = p.m2();
  const real alpha = 0.5 + 0.9 * m2;
  const real sth   = 4.0 * M0 * M0;
  const real phi   = PI / 2.0 * std::exp((sth - s34) / sth) - PI / 2.0;
  const cplx   R     = std::pow(std::exp(cplx(0, phi)) * s34 / sth, alpha - 1.0);
  return -1.0 / (m2 - M0 * M0) * R;
}

// A real basis of the polarization states of a massive vector of momentum p (upper
// components): two transverse unit vectors and the longitudinal (|p|/m, E p^/m)
// (MDirac::EpsMassiveSpin1, src/MDirac.cc:435-456, in a linear instead of the helicity
// basis; the sum over states of |amplitude|^2 is the same).
void vector_basis(const V4 &p, real e[3][4]) {
  const real P = std::sqrt(p.x * p.x + p.y * p.y + p.z * p.z);
  const real m = msqrt(p.m2());
  real n[3] = {0, 0, 1};
  if (P > 1e-12) {
    n[0] = p.x / P;
    n[1] = p.y / P;
    n[2] = p.z / P;
  }
  // first transverse direction: z x n (or x x n near the z axis), normalised
  real a[3] = {0, 0, 1};
  if (std::fabs(n[2]) > 0.9) { a[0] = 1; a[2] = 0; }
  real t1[3] = {a[1] * n[2] - a[2] * n[1], a[2] * n[0] - a[0] * n[2], a[0] * n[1] - a[1] * n[0]};
  const real nt = std::sqrt(t1[0] * t1[0] + t1[1] * t1[1] + t1[2] * t1[2]);
  for (real &x : t1) x /= nt;
  const real t2[3] = {n[1] * t1[2] - n[2] * t1[1], n[2] * t1[0] - n[0] * t1[2],
                        n[0] * t1[1] - n[1] * t1[0]};
  e[0][0] = 0; e[0][1] = t1[0]; e[0][2] = t1[1]; e[0][3] = t1[2];
  e[1][0] = 0; e[1][1] = t2[0]; e[1][2] = t2[1]; e[1][3] = t2[2];
  e[2][0] = P / m; e[2][1] = p.e / m * n[0]; e[2][2] = p.e / m * n[1]; e[2][3] = p.e / m * n[2];
}

// The nine amplitudes e3_i^a e4_j^b M_ab of one proton helicity configuration.
int tensor_me4_2xv(const Setup &S, const Event &ev, cplx *out) {
  const grn_process_params &p = S.p;
  const V4 &pa = S.pb1, &pb = S.pb2;
  const V4 &p1 = ev.pf[1], &p2 = ev.pf[2], &p3 = ev.pf[3], &p4 = ev.pf[4];
  const real M0 = p.m_central[0], M2 = M0 * M0;
  const V4     pt  = pa - p1 - p3;
  const V4     pu  = p4 - pa + p1;
  const V4     mp3 = V4(-p3.x, -p3.y, -p3.z, -p3.e);
  const V4     mpt = V4(-pt.x, -pt.y, -pt.z, -pt.e);
  const T2     G1a = vertex_ppP(p, p1, pa);
  const T2     G2b = vertex_ppP(p, p2, pb);
  // X^{ab} = G(mu, nu) iD_P(mu, nu, a, b) for the four pomeron propagators
  auto legX = [&](const T2 &G, real s, real t, cplx X[4][4]) {
    const cplx c = pomeron_prop(p, s, t);
    for (int a = 0; a < 4; ++a)
      for (int b = 0; b < 4; ++b) {
        cplx sum(0, 0);
        for (int u = 0; u < 4; ++u)
          for (int v = 0; v < 4; ++v) {
            const real g = gm(u, a) * gm(v, b) + gm(u, b) * gm(v, a) - 0.5 * gm(u, v) * gm(a, b);
            if (g != 0.0) sum += G.c[u][v] * g;
          }
        X[a][b] = c * sum;
      }
  };
  cplx X13[4][4], X24[4][4], X14[4][4], X23[4][4];
  legX(G1a, ev.ss[1][3], ev.t1, X13);
  legX(G2b, ev.ss[2][4], ev.t2, X24);
  legX(G1a, ev.ss[1][4], ev.t1, X14);
  legX(G2b, ev.ss[2][3], ev.t2, X23);
  // contract the pomeron leg into the last two indices of a vertex
  auto vblock = [&](const T4 &G, const cplx X[4][4], cplx out2[4][4]) {
    for (int u = 0; u < 4; ++u)
      for (int v = 0; v < 4; ++v) {
        cplx sum(0, 0);
        for (int a = 0; a < 4; ++a)
          for (int b = 0; b < 4; ++b) sum += X[a][b] * G[u][v][a][b];
        out2[u][v] = sum;
      }
  };
  cplx At[4][4], Bt[4][4], Au[4][4], Bu[4][4];
  vblock(vertex_Pvv(p, pt, mp3), X13, At);   // At(rho1, rho3)
  vblock(vertex_Pvv(p, p4, pt), X24, Bt);    // Bt(rho4, rho2)
  vblock(vertex_Pvv(p, p4, pu), X14, Au);    // Au(rho4, rho1)
  vblock(vertex_Pvv(p, pu, mp3), X23, Bu);   // Bu(rho2, rho3)
  (void)mpt;
  const real s34 = ev.pf[0].m2();
  const cplx   Dt  = vector_prop(pt, M0, s34) * sq(meson_ff(p.regge, pt.m2(), M2));
  const cplx   Du  = vector_prop(pu, M0, s34) * sq(meson_ff(p.regge, pu.m2(), M2));
  cplx M[4][4];
  for (int r3 = 0; r3 < 4; ++r3)
    for (int r4 = 0; r4 < 4; ++r4) {
      cplx mt(0, 0), mu(0, 0);
      for (int r1 = 0; r1 < 4; ++r1) {
        // iD_V carries g^{r1 r2}: diagonal
        mt += At[r1][r3] * G_METRIC[r1] * Bt[r4][r1];
        mu += Au[r4][r1] * G_METRIC[r1] * Bu[r1][r3];
      }
      M[r3][r4] = cplx(0, -1) * (mt * Dt + mu * Du);
    }
  real e3[3][4], e4[3][4];
  vector_basis(p3, e3);
  vector_basis(p4, e4);
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      cplx sum(0, 0);
      for (int a = 0; a < 4; ++a)
        for (int b = 0; b < 4; ++b) sum += e3[i][a] * e4[j][b] * M[a][b];
      out[3 * i + j] = sum;
    }
  return 9;
}

// Bare amplitude of the configured process.
cplx bare_amp(const Setup &S, const Event &ev);
int  bare_amps(const Setup &S, const Event &ev, cplx *A);

// Linear interpolation on the kt^2 screening table (IArray1D::Interpolate1D,
// src/MEikonal.cc:489-512).
cplx msa_interp(const Setup &S, real a) {
  const int    N    = S.n_kt2;
  const real step = (MAX_KT2 - MIN_KT2) / N;
  if (a < MIN_KT2) a = MIN_KT2;
  int i = static_cast<int>(std::floor((a - MIN_KT2) / step));
  if (i < 0) i = 0;
  if (i >= N) i = N - 1;
  const double *r0 = S.msa + 3 * i, *r1 = S.msa + 3 * (i + 1);
  const cplx    y0(r0[1], r0[2]), y1(r1[1], r1[2]);
  return y0 + (a - real(r0[0])) * ((y1 - y0) / (real(r1[0]) - real(r0[0])));
}

// Eikonal kt-loop screened |M|^2 (MProcess::S3ScreenedAmp2, src/MProcess.cc:157-288): every
// helicity amplitude is screened on its own and the |.|^2 are summed.
real screened_amp2(const Setup &S, const Event &born, const cplx *A0, int nh) {
  const grn_loop_numerics &L = S.p.loop;
  const real stepKT  = (L.kt_max - L.kt_min) / L.n_kt;
  const real stepPhi = 2.0 * PI / L.n_phi;
  const std::vector<real> U = simpson38_weights(L.n_phi);
  const std::vector<real> V = simpson38_weights(L.n_kt);
  cplx sum[9];
  Event lev;
  for (int i = 0; i <= L.n_phi; ++i) {
    const real phi = i * stepPhi;
    for (int j = 0; j <= L.n_kt; ++j) {
      const real kt   = L.kt_min + j * stepKT;
      const cplx   Aeik = msa_interp(S, kt * kt);
      const real kx = kt * std::cos(phi), ky = kt * std::sin(phi);
      if (!loop_kinematics(S, born, born.pf[1].x - kx, born.pf[1].y - ky, born.pf[2].x + kx,
                           born.pf[2].y + ky, lev))
        continue;
      cplx A[9];
      bare_amps(S, lev, A);
      for (int h = 0; h < nh; ++h) sum[h] += (U[i] * V[j]) * (Aeik * A[h] * kt);
    }
  }
  const cplx norm = cplx(0, 1) / (8.0 * PI * PI * S.s);
  real amp2 = 0;
  for (int h = 0; h < nh; ++h)
    amp2 += std::norm(A0[h] + norm * sum[h] * (9.0 * stepPhi * stepKT / 64.0));
  return amp2;
}

// ---------------------------------------------------------------------------
// Regge resonances (PP[RES], PP[RES+CON]; MRegge::ME3, src/MRegge.cc:677-712, with
// spin::ProdAmp / DecayAmp, src/MSpin.cc:280-480, and CBW, src/MForm.cc:743-830), restated
// with explicit (2J+1)-dimensional matrices: per resonance
//   A_r = 2 P(s1,t1) FF_A CBW RFF P(s2,t2) FF_B (1/m^2)^omega [g NORM sqrt(Re Tr f0 R f0^+)]
//         [g_decay NORM sqrt(Re Tr f R f^+)],  R = D^+ rho D,  NORM = sqrt(2J+1),
// f0 (f) the row D^J_{0M}(theta, phi) of q1 (of the first daughter) boosted to the X rest
// frame, D_{MM'} = D^J_{MM'}(theta_R, phi_R) of the frame; J = 0: both brackets g, g_decay.
real fact(int n) { real f = 1; for (int i = 2; i <= n; ++i) f *= i; return f; }
// Wigner small-d by its closed sum over k (as MSpin.cc:927-961 writes it), integer J.
real wigner_small_d(real theta, int m, int mp, int J) {
  real s = 0;
  for (int k = 0; k <= 2 * J; ++k) {
    if (J - mp - k < 0 || J + m - k < 0 || k + mp - m < 0) continue;
    s += std::pow(-1.0, mp - m + k) /
         (fact(J - mp - k) * fact(J + m - k) * fact(k + mp - m) * fact(k)) *
         std::pow(std::cos(theta / 2), 2 * J + m - mp - 2 * k) *
         std::pow(std::sin(theta / 2), mp - m + 2 * k);
  }
  return std::sqrt(fact(J + m) * fact(J - m) * fact(J + mp) * fact(J - mp)) * s;
}
cplx wigner_D(real theta, real phi, int m, int mp, int J) {
  return wigner_small_d(theta, m, mp, J) * std::exp(cplx(0, 1) * real(mp) * phi);
}
// p in the rest frame of X (kinematics::LorentzBoost with sign -1, MKinematics.h:384-401).
V4 to_rest(const V4 &X, const V4 &p) {
  const real M = X.m(), g = X.e / M;
  const real bx = -X.x / X.e, by = -X.y / X.e, bz = -X.z / X.e;
  const real k1 = bx * p.x + by * p.y + bz * p.z;
  const real k2 = g * (g * k1 / (1.0 + g) + p.e);
  return V4(p.x + k2 * bx, p.y + k2 * by, p.z + k2 * bz, g * (p.e + k1));
}
real theta_of(const V4 &v) {
  return (v.x == 0 && v.y == 0 && v.z == 0) ? 0.0 : std::atan2(v.pt(), v.z);
}
real phi_of(const V4 &v) { return (v.x == 0 && v.y == 0) ? 0.0 : std::atan2(v.y, v.x); }

real spin_weight(const std::vector<std::vector<cplx>> &R, real theta, real phi, int J) {
  const int n = 2 * J + 1;
  std::vector<cplx> f(n);
  for (int j = 0; j < n; ++j) f[j] = wigner_D(theta, phi, 0, j - J, J);
  cplx t = 0;
  for (int j = 0; j < n; ++j)
    for (int l = 0; l < n; ++l) t += f[j] * R[j][l] * std::conj(f[l]);
  return std::real(t);
}

cplx regge_res(const Setup &S, const Event &ev) {
  const grn_process_params &p = S.p;
  const V4 &X = ev.pf[0];
  const real m2 = ev.m2;
  // frame rotation angles (spin::GetRhoRotation, MSpin.cc:544-600)
  real thR = 0, phR = 0;
  if (p.spin_frame == GRN_FRAME_HX) {
    thR = theta_of(X);
    phR = phi_of(X);
  } else if (p.spin_frame == GRN_FRAME_CS) {
    const V4 a = to_rest(X, S.pb1), b = to_rest(X, S.pb2);
    const real na = a.p3(), nb = b.p3();
    V4 z(a.x / na - b.x / nb, a.y / na - b.y / nb, a.z / na - b.z / nb, 0);
    const real nz = z.p3();
    z = V4(z.x / nz, z.y / nz, z.z / nz, 0);
    thR = theta_of(z);
    phR = phi_of(z);
  }
  const V4 q1  = to_rest(X, S.pb1 - ev.pf[1]);
  const V4 dau = to_rest(X, ev.pf[3]);
  const real FFA = p.soft.gN_P * proton_ff(p.soft, ev.t1);
  const real FFB = p.soft.gN_P * proton_ff(p.soft, ev.t2);
  const cplx   prop = regge_prop(p.regge, ev.ss[1][0], ev.t1) * FFA *
                    regge_prop(p.regge, ev.ss[2][0], ev.t2) * FFB;
  cplx sum = 0;
  for (int r = 0; r < p.n_res; ++r) {
    const grn_resonance &R = p.res[r];
    const int    J = R.J;
    const real M0 = R.M, W = R.W;
    cplx den(m2 - M0 * M0, M0 * W), num = 1.0;
    if (R.bw == 2) den = cplx(m2 - M0 * M0, std::sqrt(m2) * W);
    if (R.bw == 3) {
      const real ma = p.m_central[0], mb = p.m_central[1];
      const real u = msqrt((m2 - sq(ma + mb)) * (m2 - sq(ma - mb))) / (2 * std::sqrt(m2));
      const real d = msqrt((M0 * M0 - sq(ma + mb)) * (M0 * M0 - sq(ma - mb))) / (2 * M0);
      den = cplx(m2 - M0 * M0, W * M0 * M0 / std::sqrt(m2) * std::pow(u / d, 2 * J + 1));
    }
    if (R.bw == 4 && J == 2)
      num = 7.0 / 6.0 - (4.0 / 3.0) * (m2 / (M0 * M0)) + (2.0 / 3.0) * sq(m2) / sq(sq(M0));
    const cplx   cbw = -num / den;
    const real rff = std::exp(-sq(m2 - M0 * M0) / sq(sq(R.g_ff)));
    const real V   = std::pow(1.0 / m2, p.omega);
    cplx prod = cplx(R.g_regge[0], R.g_regge[1]);
    real dec = R.g_decay;
    if (J == 2) {
      const int n = 5;
      std::vector<std::vector<cplx>> D(n, std::vector<cplx>(n)), rho = D, Rr = D;
      for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j) {
          D[i][j]   = wigner_D(thR, phR, i - 2, j - 2, 2);
          rho[i][j] = cplx(R.rho[0][5 * i + j], R.rho[1][5 * i + j]);
        }
      for (int i = 0; i < n; ++i)
        for (int k = 0; k < n; ++k) {
          cplx t = 0;
          for (int j = 0; j < n; ++j)
            for (int l = 0; l < n; ++l) t += std::conj(D[j][i]) * rho[j][l] * D[l][k];
          Rr[i][k] = t;
        }
      if (p.spin_gen) prod *= std::sqrt(5.0) * msqrt(spin_weight(Rr, theta_of(q1), phi_of(q1), 2));
      if (p.spin_dec) dec *= std::sqrt(5.0) * msqrt(spin_weight(Rr, theta_of(dau), phi_of(dau), 2));
    }
    sum += 2.0 * cbw * rff * V * prod * dec;
  }
  return prop * sum;
}

// ---------------------------------------------------------------------------
// Observables of the on-the-fly histograms (MUserHistograms::FillHistograms,
// src/MUserHistograms.cc:60-125, frames of kinematics::LorentzFrame, MKinematics.h:952-1011):
// order M, Y, Pt, |dphi_pp|, pT1, m(first central), y3, y4, then (cos theta, phi) of the first
// central particle in CS, HX, AH, PG (beam 2), CM and the lab.
void observables(const Setup &S, const Event &ev, real *o) {
  const V4 &X = ev.pf[0];
  o[0] = X.m();
  o[1] = X.rap();
  o[2] = X.pt();
  real D = std::atan2(ev.pf[1].y, ev.pf[1].x) - std::atan2(ev.pf[2].y, ev.pf[2].x);
  while (D >= PI) D -= 2 * PI;
  while (D < -PI) D += 2 * PI;
  o[3] = std::fabs(D);
  o[4] = ev.pf[1].pt();
  o[5] = ev.pf[3].m();
  o[6] = ev.pf[3].rap();
  o[7] = ev.pf[4].rap();
  const V4 p = to_rest(X, ev.pf[3]), b1 = to_rest(X, S.pb1), b2 = to_rest(X, S.pb2);
  using A3 = std::array<real, 3>;
  auto unit = [](A3 v) {
    const real n = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    return A3{v[0] / n, v[1] / n, v[2] / n};
  };
  auto cross = [](const A3 &u, const A3 &v) {
    return A3{u[1] * v[2] - u[2] * v[1], u[2] * v[0] - u[0] * v[2], u[0] * v[1] - u[1] * v[0]};
  };
  const A3 P3 = {p.x, p.y, p.z}, B1 = {b1.x, b1.y, b1.z}, B2 = {b2.x, b2.y, b2.z};
  const A3 u1 = unit(B1), u2 = unit(B2);
  const A3 zs[5] = {unit({u1[0] - u2[0], u1[1] - u2[1], u1[2] - u2[2]}),
                    unit({-(B1[0] + B2[0]), -(B1[1] + B2[1]), -(B1[2] + B2[2])}),
                    unit({u1[0] + u2[0], u1[1] + u2[1], u1[2] + u2[2]}), u2, A3{0, 0, 1}};
  for (int f = 0; f < 5; ++f) {
    const A3 y = f == 4 ? A3{0, 1, 0} : unit(cross(u1, u2));
    const A3 x = unit(cross(y, zs[f]));
    const real qx = x[0] * P3[0] + x[1] * P3[1] + x[2] * P3[2];
    const real qy = y[0] * P3[0] + y[1] * P3[1] + y[2] * P3[2];
    const real qz = zs[f][0] * P3[0] + zs[f][1] * P3[1] + zs[f][2] * P3[2];
    o[8 + 2 * f] = std::cos(std::atan2(std::sqrt(qx * qx + qy * qy), qz));
    o[9 + 2 * f] = (qx == 0 && qy == 0) ? 0.0 : std::atan2(qy, qx);
  }
  const V4 &l = ev.pf[3];
  o[18] = std::cos(std::atan2(l.pt(), l.z));
  o[19] = (l.x == 0 && l.y == 0) ? 0.0 : std::atan2(l.y, l.x);
}

// RES+CONTENSOR (MSubProc.h:319-351): the continuum's and the resonances' helicity amplitudes
// are added per proton configuration; with the high-energy proton vertex all four are equal,
// so the sum of one configuration carries |M|^2.
cplx bare_amp(const Setup &S, const Event &ev) {
  if (S.p.n_central == 4) return regge_me6(S, ev);
  if (S.p.n_central == 6) return regge_me8(S, ev);
  if (S.p.process == GRN_PROC_TENSOR_RES) return tensor_me3(S, ev);
  if (S.p.process == GRN_PROC_TENSOR_RESCON)
    return tensor_me4_2xs(S, ev) + (S.p.n_res > 0 ? tensor_me3(S, ev) : cplx(0.0));
  if (S.p.process == GRN_PROC_REGGE_RES) return regge_res(S, ev);
  if (S.p.process == GRN_PROC_REGGE_RESCON) return regge_me4(S, ev) + regge_res(S, ev);
  return S.p.process == GRN_PROC_TENSOR_CON ? tensor_me4_2xs(S, ev) : regge_me4(S, ev);
}

// All helicity amplitudes of one proton helicity configuration (the high-energy proton
// vertex makes the four proton configurations equal, so |M|^2 = sum over these).
int bare_amps(const Setup &S, const Event &ev, cplx *A) {
  if (S.p.process == GRN_PROC_TENSOR_CON && S.p.central_spin == 1)
    return tensor_me4_2xv(S, ev, A);
  A[0] = bare_amp(S, ev);
  return 1;
}

// ForwardVolume's excitation factor (src/MProcess.cc:1399-1413): per excited leg the
// log-change Jacobian M^2 times the log range of M^2.
real forward_mass_volume(const Setup &S, const Event &ev) {
  if (!S.p.excitation) return 1.0;
  const real range = std::log(S.p.xi_max * S.s) - std::log(sq(1.09));
  real v = 1.0;
  if (ev.ex1) v *= ev.pf[1].m2() * range;
  if (ev.ex2) v *= ev.pf[2].m2() * range;
  return v;
}

// Phase-space weight and integration volume (MContinuum.cc:619-656; ForwardVolume
// MProcess.cc:1390-1415).
real ps_factor(const Setup &S, const Event &ev) {
  const grn_gencuts &g = S.p.gcuts;
  const real J = 1.0 / std::fabs(ev.pf[1].z / ev.pf[1].e - ev.pf[2].z / ev.pf[2].e);
  if (S.p.phase_space == GRN_PS_FACTORIZED) {
    // C_space = dPhi2/(2 pi), B51PhaseSpaceWeight x B51IntegralVolume (MFactorized.cc:160-183,
    // 418-450)
    const real m3 = S.p.m_central[0], m4 = S.p.m_central[1];
    (void)m3;
    (void)m4;
    const real psw  = 0.5 * (1.0 / std::pow(2.0 * PI, 5)) * (ev.pf[1].pt() / (2.0 * ev.pf[1].e)) *
                       (ev.pf[2].pt() / (2.0 * ev.pf[2].e)) * J;
    const real fwd = sq(2.0 * PI) * ev.pf[1].pt() * ev.pf[2].pt() *
                       sq(std::log(g.fpt_max) - std::log(g.fpt_min + ZERO_EPS)) *
                       forward_mass_volume(S, ev);
    const real vol = (ev.m2hi - ev.m2lo) * (g.Y_max - g.Y_min) * fwd;
    return (ev.dw / (2.0 * PI)) * psw * vol;
  }
  const int Kf = S.p.n_central, Nf = Kf + 2;
  real prod = ev.q.pt();
  if (Kf >= 4) {
    prod = 1.0;
    for (int i = 0; i < Kf - 1; ++i) prod *= ev.kq[i].pt();
  }
  const real psw = (1.0 / std::pow(2.0, 2 * (Nf - 2))) * (1.0 / std::pow(2.0 * PI, 3 * Nf - 4)) *
                     (ev.pf[1].pt() / (2.0 * ev.pf[1].e)) * (ev.pf[2].pt() / (2.0 * ev.pf[2].e)) *
                     J * prod;
  const real fwd = sq(2.0 * PI) * ev.pf[1].pt() * ev.pf[2].pt() *
                     sq(std::log(g.fpt_max) - std::log(g.fpt_min + ZERO_EPS)) *
                     forward_mass_volume(S, ev);
  const real vol = std::pow(g.kt_max - g.kt_min, Kf - 1) * std::pow(2.0 * PI, Kf - 1) *
                     std::pow(g.rap_max - g.rap_min, Kf) * fwd;
  return psw * vol;
}

// Fiducial cuts (MProcess::CommonCuts + FindDecayCuts, MProcess.cc:1085-1154).
bool fiducial(const Setup &S, const Event &ev) {
  const grn_fidcuts &f = S.p.fcuts;
  if (!f.active) return true;
  const real at1 = std::fabs(ev.t1), at2 = std::fabs(ev.t2);
  if (!(at1 >= f.ft_min && at1 <= f.ft_max && at2 >= f.ft_min && at2 <= f.ft_max)) return false;
  // excited forward systems: their mass window (CommonCuts, src/MProcess.cc:1105-1119)
  if (ev.ex1 && !(ev.pf[1].m() >= f.fM_min && ev.pf[1].m() <= f.fM_max)) return false;
  if (ev.ex2 && !(ev.pf[2].m() >= f.fM_min && ev.pf[2].m() <= f.fM_max)) return false;
  const real M = msqrt(ev.m2);
  if (!(M >= f.M_min && M <= f.M_max && ev.Y >= f.Y_min && ev.Y <= f.Y_max && ev.Pt >= f.Pt_min &&
        ev.Pt <= f.Pt_max))
    return false;
  bool ok = true;
  // final-state particles: the central pair, or the leaves of its decays (FindDecayCuts)
  const bool casc = S.p.n_decay == 2;
  const int  np   = casc ? 4 : S.p.n_central;
  for (int k = 0; k < np; ++k) {
    const V4 &p = casc ? ev.leaf[k] : ev.pf[3 + k];
    const real pt = p.pt(), et = p.mt(), eta = p.eta(), rap = p.rap();
    if (!(pt >= f.pt_min && pt <= f.pt_max && et >= f.Et_min && et <= f.Et_max &&
          eta >= f.eta_min && eta <= f.eta_max && rap >= f.rap_min && rap <= f.rap_max))
      ok = false;
  }
  return ok;
}

// Veto cuts (MProcess::VetoCuts + FindVetoCuts, MProcess.cc:1069-1082, 1157-1175): false when
// a final-state particle of the central system lies in a veto domain (elastic forward
// protons have no fragments to test).
bool veto_cuts(const Setup &S, const Event &ev) {
  if (!S.p.veto_active) return true;
  const bool leaves = S.p.n_decay == 2 || S.p.n_central >= 4;
  const int  np     = S.p.n_decay == 2 ? 4 : S.p.n_central;
  for (int k = 0; k < np; ++k) {
    const V4 &p = leaves ? ev.leaf[k] : ev.pf[3 + k];
    const real pt = p.pt(), eta = p.eta();
    for (int d = 0; d < S.p.n_veto; ++d)
      if (pt >= S.p.veto_pt_min[d] && pt <= S.p.veto_pt_max[d] && eta >= S.p.veto_eta_min[d] &&
          eta <= S.p.veto_eta_max[d])
        return false;
  }
  return true;
}

// One event weight (MContinuum::EventWeight, src/MContinuum.cc:164-193).
real event_weight(const Setup &S, const real *u, uint8_t &flags, Event &ev) {
  real W = 0.0;
  const bool kin = S.p.phase_space == GRN_PS_FACTORIZED ? build_kinematics_F(S, u, ev)
                                                        : build_kinematics(S, u, ev);
  const bool fid = kin && fiducial(S, ev);
  const bool veto = !kin || veto_cuts(S, ev);
  if (kin && fid && veto) {
    cplx A0[9];
    const int nh = bare_amps(S, ev, A0);
    real amp2 = 0;
    if (S.p.screening) {
      amp2 = screened_amp2(S, ev, A0, nh);
    } else {
      for (int h = 0; h < nh; ++h) amp2 += std::norm(A0[h]);
    }
    W = (1.0 / S.p.s_factor) * ps_factor(S, ev) * amp2 * GEV2BARN / (2.0 * S.s);
  }
  bool amp_ok = true;
  if (std::isnan(W) || std::isinf(W)) {
    W      = 0.0;
    amp_ok = false;
  }
  flags = (kin ? GRN_FLAG_KINEMATICS_OK : 0) | (fid ? GRN_FLAG_FIDCUTS_OK : 0) |
          (veto ? GRN_FLAG_VETOCUTS_OK : 0) | (amp_ok ? GRN_FLAG_AMPLITUDE_OK : 0);
  return W;
}

Setup make_setup(const grn_process_params *p, const double *msa, int n_kt2) {
  Setup S;
  S.p      = *p;
  S.sqrt_s = p->sqrt_s;
  S.s      = p->sqrt_s * p->sqrt_s;
  const real E  = p->sqrt_s / 2.0;
  const real pz = msqrt(E * E - sq(p->m_beam));
  S.pb1 = V4(0, 0, pz, E);
  S.pb2 = V4(0, 0, -pz, E);
  S.msa   = msa;
  S.n_kt2 = n_kt2;
  return S;
}

template <typename F>
void parallel_for(int64_t n, int nthreads, F &&fn) {
  if (nthreads <= 1 || n < 64) {
    fn(0, n);
    return;
  }
  std::vector<std::thread> th;
  const int64_t chunk = (n + nthreads - 1) / nthreads;
  for (int t = 0; t < nthreads; ++t) {
    const int64_t a = t * chunk, b = std::min<int64_t>(n, a + chunk);
    if (a >= b) break;
    th.emplace_back([&fn, a, b] { fn(a, b); });
  }
  for (auto &t : th) t.join();
}

// ---------------------------------------------------------------------------
// Eikonal tables.

// Linear interpolation of the density table (IArray1D::Interpolate1D).
cplx table_interp(const double *tab, int N, real xmin, real xmax, real a) {
  const real step = (xmax - xmin) / N;
  if (a < xmin) a = xmin;
  int i = static_cast<int>(std::floor((a - xmin) / step));
  if (i < 0) i = 0;
  if (i >= N) i = N - 1;
  const double *r0 = tab + 3 * i, *r1 = tab + 3 * (i + 1);
  const cplx y0(r0[1], r0[2]), y1(r1[1], r1[2]);
  return y0 + (a - real(r0[0])) * ((y1 - y0) / (real(r1[0]) - real(r0[0])));
}

}  // namespace orc

// ===========================================================================
// C interface used by the tests (ctypes) and by the benchmark's CPU legs.
extern "C" {

// Weights for n points (u point-major, dim = 8). msa may be NULL when the
// process has no screening. rec (may be NULL) receives per point
// t1, t2, m2 and the 4-vectors pfinal[1..4] (19 doubles).
int orc_weights(const grn_process_params *p, const double *u, int64_t n, int32_t dim, double *w,
                uint8_t *flags, double *rec, const double *msa, int32_t n_kt2, int32_t nthreads) {
  const int32_t want = p ? orc::point_dim(*p) : 8;
  if (!p || !u || !w || dim != want ||
      (p->n_central != 2 && p->n_central != 4 && p->n_central != 6))
    return GRN_ERR_INVALID;
  if (p->n_central >= 4 && p->process != GRN_PROC_REGGE_CON) return GRN_ERR_INVALID;
  if (p->screening && (!msa || n_kt2 < 2)) return GRN_ERR_STATE;
  const orc::Setup S = orc::make_setup(p, msa, n_kt2);
  orc::parallel_for(n, nthreads, [&](int64_t a, int64_t b) {
    orc::Event ev;
    for (int64_t i = a; i < b; ++i) {
      uint8_t f = 0;
      ev        = orc::Event();
      orc::real ur[24];
      for (int d = 0; d < dim; ++d) ur[d] = u[i * dim + d];
      w[i]      = double(orc::event_weight(S, ur, f, ev));
      if (flags) flags[i] = f;
      if (rec) {
        double *r = rec + i * 35;
        r[0] = ev.t1;
        r[1] = ev.t2;
        r[2] = ev.m2;
        for (int k = 0; k < 8; ++k) {
          const orc::V4 &v = k < 4 ? ev.pf[k + 1] : ev.leaf[k - 4];
          r[3 + 4 * k + 0] = v.x;
          r[3 + 4 * k + 1] = v.y;
          r[3 + 4 * k + 2] = v.z;
          r[3 + 4 * k + 3] = v.e;
        }
      }
    }
  });
  return GRN_OK;
}

// Histogram observables (20 per point, see orc::observables) of the points that pass the
// kinematics (ok[i] = 1), from the tree-level event.
int orc_observables(const grn_process_params *p, const double *u, int64_t n, int32_t dim,
                    double *obs, uint8_t *ok, int32_t nthreads) {
  const int32_t want = p ? orc::point_dim(*p) : 8;
  if (!p || !u || !obs || dim != want ||
      (p->n_central != 2 && p->n_central != 4 && p->n_central != 6))
    return GRN_ERR_INVALID;
  grn_process_params q = *p;
  q.screening = 0;
  const orc::Setup S = orc::make_setup(&q, nullptr, 0);
  orc::parallel_for(n, nthreads, [&](int64_t a, int64_t b) {
    for (int64_t i = a; i < b; ++i) {
      uint8_t    f  = 0;
      orc::Event ev = orc::Event();
      orc::real ur[24], ob[20];
      for (int d = 0; d < dim; ++d) ur[d] = u[i * dim + d];
      orc::event_weight(S, ur, f, ev);
      ok[i] = (f & GRN_FLAG_KINEMATICS_OK) ? 1 : 0;
      if (ok[i]) {
        orc::observables(S, ev, ob);
        for (int k = 0; k < 20; ++k) obs[i * 20 + k] = double(ob[k]);
      }
    }
  });
  return GRN_OK;
}

// Eikonal tables and cross sections (MEikonal::S3Constructor, S3Density,
// S3Screening, S3CalcXS; src/MEikonal.cc:46-376). mbt: (n_bt+1) x 3,
// msa: (n_kt2+1) x 3 rows of (x, Re, Im); xs: sigma_tot, sigma_el, sigma_inel [barn].
int orc_eikonal(const grn_process_params *p, int32_t n_bt, int32_t n_kt2, double *mbt, double *msa,
                double *xs, int32_t nthreads) {
  using namespace orc;
  if (!p || n_bt < 2 || n_kt2 < 2 || !mbt) return GRN_ERR_INVALID;
  const double s = p->sqrt_s * p->sqrt_s;

  // Density: (1 / 2 pi s) * int dkt A(s, -kt^2) J0(b kt) kt.
  std::vector<cplx> amp(FB_N + 1);
  const double kstep = (FB_MAX_KT - FB_MIN_KT) / FB_N;
  for (int k = 0; k <= FB_N; ++k) {
    const double kt = FB_MIN_KT + k * kstep;
    amp[k]          = elastic_amp(p->soft, s, -kt * kt) * kt;
  }
  const double bstep = (MAX_BT - MIN_BT) / n_bt;
  parallel_for(n_bt + 1, nthreads, [&](int64_t a, int64_t b) {
    std::vector<cplx> f(FB_N + 1);
    for (int64_t i = a; i < b; ++i) {
      const double bt = MIN_BT + i * bstep;
      for (int k = 0; k <= FB_N; ++k) f[k] = amp[k] * bessel_j0(bt * (FB_MIN_KT + k * kstep));
      const cplx v = simpson13(f, kstep) * (1.0 / (2.0 * PI * s));
      mbt[3 * i + 0] = bt;
      mbt[3 * i + 1] = v.real();
      mbt[3 * i + 2] = v.imag();
    }
  });

  // Cross sections, single channel (S3CalcXS).
  if (xs) {
    const int    N    = 6000;
    const double step = (MAX_BT - MIN_BT) / N;
    std::vector<double> ft(N + 1), fe(N + 1), fi(N + 1);
    for (int i = 0; i <= N; ++i) {
      const double bt = MIN_BT + i * step;
      const cplx   Om = table_interp(mbt, n_bt, MIN_BT, MAX_BT, bt);
      const cplx   Ael = cplx(0, 1) * (1.0 - std::exp(cplx(0, 1) * Om / 2.0));
      ft[i] = 2.0 * Ael.imag() * bt;
      fe[i] = std::norm(Ael) * bt;
      fi[i] = (2.0 * Ael.imag() - std::norm(Ael)) * bt;
    }
    xs[0] = 2.0 * PI * simpson13(ft, step) * GEV2BARN;
    xs[1] = 2.0 * PI * simpson13(fe, step) * GEV2BARN;
    xs[2] = 2.0 * PI * simpson13(fi, step) * GEV2BARN;
  }

  // Screening amplitude: 2s * 2pi * int db i(1 - exp(i Omega/2)) J0(b kt) b.
  if (msa) {
    const double step = (MAX_BT - MIN_BT) / FB_N;
    std::vector<cplx> g(FB_N + 1);
    for (int k = 0; k <= FB_N; ++k) {
      const double bt = MIN_BT + k * step;
      const cplx   Om = table_interp(mbt, n_bt, MIN_BT, MAX_BT, bt);
      g[k] = cplx(0, 1) * (1.0 - std::exp(cplx(0, 1) * Om / 2.0)) * bt;
    }
    const double kstep2 = (MAX_KT2 - MIN_KT2) / n_kt2;
    parallel_for(n_kt2 + 1, nthreads, [&](int64_t a, int64_t b) {
      std::vector<cplx> f(FB_N + 1);
      for (int64_t i = a; i < b; ++i) {
        const double kt2 = MIN_KT2 + i * kstep2;
        const double kt  = msqrt(kt2);
        for (int k = 0; k <= FB_N; ++k) f[k] = g[k] * bessel_j0((MIN_BT + k * step) * kt);
        const cplx v = (2.0 * s) * (2.0 * PI) * simpson13(f, step);
        msa[3 * i + 0] = kt2;
        msa[3 * i + 1] = v.real();
        msa[3 * i + 2] = v.imag();
      }
    });
  }
  return GRN_OK;
}

// Bessel J0 as used by the tables (for unit tests).
double orc_bessel_j0(double x) { return orc::bessel_j0(x); }

// ---------------------------------------------------------------------------
// VEGAS (include/Graniitti/MVEGAS.h:87-142; MGraniitti.cc:1357-1375).

// Rebin: redistribute the bin edges of dimension j so that each new bin holds an
// equal share ac of the importance r (MVEGAS.h:87-104).
static void vegas_rebin(int bins, int dim, int j, double ac, const double *r, double *xmat) {
  std::vector<double> xnew(bins);
  int    k  = 0;
  double dr = 0.0, zn = 0.0, zo = 0.0;
  for (int i = 0; i < bins - 1; ++i) {
    while (ac > dr) dr += r[(++k) - 1];
    if (k > 1) zo = xmat[(k - 2) * dim + j];
    zn = xmat[(k - 1) * dim + j];
    dr -= ac;
    xnew[i] = zn - (zn - zo) * dr / r[k - 1];
  }
  for (int i = 0; i < bins - 1; ++i) xmat[i * dim + j] = xnew[i];
  xmat[(bins - 1) * dim + j] = 1.0;
}

// Fresh uniform grid: xmat[0][j] = 1 then a rebin from one bin
// (VEGASData::ClearAll + InitGridDependent, MVEGAS.h:72-84, 163-187).
void orc_vegas_grid_init(int32_t bins, int32_t dim, double *xmat) {
  std::vector<double> r(bins, 1.0);
  for (int i = 0; i < bins * dim; ++i) xmat[i] = 0.0;
  for (int j = 0; j < dim; ++j) xmat[j] = 1.0;
  for (int j = 0; j < dim; ++j) vegas_rebin(bins, dim, j, 1.0 / bins, r.data(), xmat);
}

// Smooth the f^2 histogram and rebin (VEGASData::OptimizeGrid, MVEGAS.h:107-142).
// f2mat is bins x dim and is modified in place as in the reference.
void orc_vegas_refine(int32_t bins, int32_t dim, double lambda, double *xmat, double *f2mat) {
  const double EPS = 1.0e-30;
  std::vector<double> d(dim), r(bins);
  for (int j = 0; j < dim; ++j) {
    double zo = f2mat[0 * dim + j], zn = f2mat[1 * dim + j];
    f2mat[0 * dim + j] = (zo + zn) / 2.0;
    d[j]               = f2mat[0 * dim + j];
    for (int i = 2; i < bins; ++i) {
      const double ac          = zo + zn;
      zo                       = zn;
      zn                       = f2mat[i * dim + j];
      f2mat[(i - 1) * dim + j] = (ac + zn) / 3.0;
      d[j] += f2mat[(i - 1) * dim + j];
    }
    f2mat[(bins - 1) * dim + j] = (zo + zn) / 2.0;
    d[j] += f2mat[(bins - 1) * dim + j];
  }
  for (int j = 0; j < dim; ++j) {
    double ac = 0.0;
    for (int i = 0; i < bins; ++i) {
      double &v = f2mat[i * dim + j];
      if (v < EPS) v = EPS;
      r[i] = std::pow((1.0 - v / d[j]) / (std::log(d[j]) - std::log(v) + EPS), lambda);
      if (std::isnan(r[i]) || std::isinf(r[i])) r[i] = EPS;
      ac += r[i];
    }
    vegas_rebin(bins, dim, j, ac / bins, r.data(), xmat);
  }
}

// Map uniforms r (n x dim) through the grid: x, VEGAS weight and 1-based bins
// (MGraniitti.cc:1357-1375).
void orc_vegas_map(int32_t bins, int32_t dim, const double *xmat, const double *r, int64_t n,
                   double *x, double *vw, int32_t *bin) {
  for (int64_t k = 0; k < n; ++k) {
    double w = 1.0;
    for (int j = 0; j < dim; ++j) {
      const double zn = r[k * dim + j] * bins + 1.0;
      int          ind = static_cast<int>(static_cast<unsigned>(zn));
      ind = std::max(1, std::min(ind, bins));
      double zo, ac;
      if (ind > 1) {
        zo = xmat[(ind - 1) * dim + j] - xmat[(ind - 2) * dim + j];
        ac = xmat[(ind - 2) * dim + j] + (zn - ind) * zo;
      } else {
        zo = xmat[(ind - 1) * dim + j];
        ac = (zn - ind) * zo;
      }
      x[k * dim + j] = ac;
      w *= zo * bins;
      if (bin) bin[k * dim + j] = ind;
    }
    vw[k] = w;
  }
}

// ---------------------------------------------------------------------------
// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11), written from the paper.
static inline void philox_round(uint32_t c[4], const uint32_t k[2]) {
  const uint64_t p0 = static_cast<uint64_t>(0xD2511F53u) * c[0];
  const uint64_t p1 = static_cast<uint64_t>(0xCD9E8D57u) * c[2];
  const uint32_t hi0 = static_cast<uint32_t>(p0 >> 32), lo0 = static_cast<uint32_t>(p0);
  const uint32_t hi1 = static_cast<uint32_t>(p1 >> 32), lo1 = static_cast<uint32_t>(p1);
  const uint32_t n0 = hi1 ^ c[1] ^ k[0];
  const uint32_t n2 = hi0 ^ c[3] ^ k[1];
  c[0] = n0;
  c[1] = lo1;
  c[2] = n2;
  c[3] = lo0;
}

void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
  uint32_t c[4] = {ctr[0], ctr[1], ctr[2], ctr[3]};
  uint32_t k[2] = {key[0], key[1]};
  for (int r = 0; r < 10; ++r) {
    philox_round(c, k);
    if (r < 9) {
      k[0] += 0x9E3779B9u;
      k[1] += 0xBB67AE85u;
    }
  }
  for (int i = 0; i < 4; ++i) out[i] = c[i];
}

// Uniforms of points first..first+n-1: counter = (index lo, index hi, dimension
// block, stream), key = seed; each block gives two doubles (53-bit, [0,1)).
void orc_uniforms(uint64_t seed, uint32_t stream, int64_t first, int64_t n, int32_t dim,
                  double *out) {
  const uint32_t key[2] = {static_cast<uint32_t>(seed), static_cast<uint32_t>(seed >> 32)};
  for (int64_t i = 0; i < n; ++i) {
    const uint64_t idx = static_cast<uint64_t>(first + i);
    for (int blk = 0; 2 * blk < dim; ++blk) {
      const uint32_t ctr[4] = {static_cast<uint32_t>(idx), static_cast<uint32_t>(idx >> 32),
                               static_cast<uint32_t>(blk), stream};
      uint32_t o[4];
      orc_philox4x32_10(ctr, key, o);
      const uint64_t a = (static_cast<uint64_t>(o[1]) << 32) | o[0];
      const uint64_t b = (static_cast<uint64_t>(o[3]) << 32) | o[2];
      out[i * dim + 2 * blk] = static_cast<double>(a >> 11) * 0x1.0p-53;
      if (2 * blk + 1 < dim) out[i * dim + 2 * blk + 1] = static_cast<double>(b >> 11) * 0x1.0p-53;
    }
  }
}

}  // extern "C"
