// grn_physics.cuh — device physics of the event-weight path.
//
// Formulation: light-cone components p+- = E +- pz throughout. For the elastic
// forward legs the momentum-fraction losses x1, x2 follow from longitudinal
// momentum conservation as a rapidly convergent fixed point, and every invariant
// (t1, t2, s13 ..., t_hat, u_hat) is a sum of same-sign terms. No quantity of order
// sqrt(s) is subtracted from another, which is what lets the kt-loop run in FP32.
// Reference quantities are the ones of the GRANIITTI generator: file:line cited
// per function.
#pragma once

#include <cstdint>
#include <cmath>

#include "graniitti_gb300.h"

#ifdef __CUDACC__
#define GRN_HD __host__ __device__ __forceinline__
// Rarely taken paths (cascade decays, vector-pair amplitudes) stay out of line so that they
// do not raise the register count of the kernels that inline the common path.
#define GRN_HD_COLD static __host__ __device__ __noinline__
#else
#define GRN_HD inline
#define GRN_HD_COLD static inline
#endif

namespace grn {

constexpr double kPi = 3.14159265358979323846264338327950288;

// hbar*c in GeV m; GeV^-2 -> barn (include/Graniitti/MPDG.h:63-78).
constexpr double kHbar     = 6.582119514E-25;
constexpr double kCLight   = 2.99792458E8;
constexpr double kGeV2m    = kHbar * kCLight;
constexpr double kGeV2fm   = kGeV2m * 1E15;
constexpr double kGeV2barn = (kGeV2m * kGeV2m) / 1E-28;
constexpr double kMpiSoft  = 0.13957018;  // pion mass of the pomeron pion loop (MPDG.h:56)
constexpr double kZeroEps  = 1e-12;       // log(pt_min + ZERO_EPS) (MProcess.h)

// Eikonal numerics (include/Graniitti/MEikonal.h:27-40).
constexpr double kMinKT2  = 1E-6;
constexpr double kMaxKT2  = 25.0;
constexpr double kMinBT   = 1E-6;
constexpr double kMaxBT   = 10.0 / kGeV2fm;
constexpr double kFBMinKT = 1E-9;
constexpr double kFBMaxKT = 30.0;
constexpr int    kFBN     = 10000;

template <typename T>
struct cx {
  T re, im;
};
template <typename T>
GRN_HD cx<T> cmul(cx<T> a, cx<T> b) {
  return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re};
}
template <typename T>
GRN_HD cx<T> cscale(cx<T> a, T s) {
  return {a.re * s, a.im * s};
}
template <typename T>
GRN_HD cx<T> cadd(cx<T> a, cx<T> b) {
  return {a.re + b.re, a.im + b.im};
}

// Per-engine constants derived once on the host from grn_process_params.
struct Consts {
  // fiducial windows as monotone images (comparisons without transcendentals): the system
  // mass^2 and pT^2, exp(2 Y) of the system rapidity, sinh(eta) of the particles' eta
  double cut_m2lo, cut_m2hi, cut_pt2lo, cut_pt2hi, cut_e2ylo, cut_e2yhi, cut_sheta_lo,
      cut_sheta_hi;
  double s, sqrt_s;
  double L, eps;            // beam light-cone: pb1+ = pb2- = L, pb1- = pb2+ = eps = m^2/L
  double invL, invL2;       // 1 / L, 1 / L^2
  double ifc1, ifc2;        // 1 / fc1, 1 / fc2 of the proton form factor
  double mp2;               // forward-leg mass^2 (elastic)
  double m3, m4, m3sq, m4sq;
  double lnpt_lo, lnpt_hi;  // log(fpt_min + ZERO_EPS), log(fpt_max)
  double w_const;           // every u-independent factor of the weight
  double M2min, M2max;      // <F>: central-system mass^2 window (B51RandomKin)
  double offshell;          // cascades: widths of the Breit-Wigner mass draws (OFFSHELL)
  double lnM2f_lo, lnM2f_hi;  // excitation: log of the excited masses^2 range [1.09^2, xi s]
  double gin;               // excitation: sqrt(g3P gN_P), the inelastic vertex coupling
  int    dec0;              // cascades: first decay coordinate (10; 8 with OFFSHELL = 0)
  double M2prop;            // off-shell propagator nominal mass^2 (ME4: first central mass)
  double M2propB;           // ME6: mass^2 of the third central particle (second propagator)
  double g2;                // (c0 / gN_P)^2
  double gN2;               // gN_P^2
  double eta0_re[3], eta0_im[3];  // ReggeEta(a0_k, sgn_k)
  double lns0;              // log(s0)
  int    n_active;          // number of active trajectories
  int    active[3];
  // PP[RESTENSOR] resonances: spin, M0^2, M0 W and the real prefactors of the collapsed
  // contractions (tensor_me3)
  int    n_res;
  int    res_J[GRN_MAX_RESONANCES];
  int    res_smask;         // J = 2 coupling structures in use (bit j: g_j != 0)
  double res_M2[GRN_MAX_RESONANCES], res_MW[GRN_MAX_RESONANCES];
  double res_c0[GRN_MAX_RESONANCES], res_c1[GRN_MAX_RESONANCES];
  double res_g[GRN_MAX_RESONANCES][7];  // J = 2 couplings g_Tensor[0..6]
  // PP[RES], PP[RES+CON] (Regge resonances, regge_res_*): count, and per resonance the
  // Breit-Wigner form, M0, width, 1 / S0^4 of the form factor, g_regge x g_decay
  int    rr_n;
  int    rr_J[GRN_MAX_RESONANCES], rr_bw[GRN_MAX_RESONANCES];
  double rr_M[GRN_MAX_RESONANCES], rr_W[GRN_MAX_RESONANCES], rr_iff4[GRN_MAX_RESONANCES];
  double rr_g_re[GRN_MAX_RESONANCES], rr_g_im[GRN_MAX_RESONANCES];
};

// sin(pi x), cos(pi x) without rounding pi x first.
GRN_HD void sincos_pi(double x, double &s, double &c) {
#ifdef __CUDA_ARCH__
  sincospi(x, &s, &c);
#else
  s = std::sin(kPi * x);
  c = std::cos(kPi * x);
#endif
}
// sin(pi x), cos(pi x) in FP32 arithmetic only: x = n + r with n = rint(x), |r| <= 1/2 (r
// exact), then the Taylor series of sin(pi r) / r and cos(pi r) in r^2 through the r^14 term,
// evaluated by Horner's rule (truncation below 1e-9 at |r| = 1/2), and the sign (-1)^n. About
// 2 ulp; relative accuracy kept for small r (the leading term is pi r).
GRN_HD void sincos_pi_poly(float x, float &s, float &c) {
  const float n  = rintf(x);
  const float r  = x - n;
  const float r2 = r * r;
  float ps = 4.6630280576761255e-4f;  // pi^13 / 13!
  ps = fmaf(ps, r2, -7.3704309457143508e-3f);
  ps = fmaf(ps, r2, 8.2145886611128228e-2f);
  ps = fmaf(ps, r2, -5.9926452932079208e-1f);
  ps = fmaf(ps, r2, 2.5501640398773455f);
  ps = fmaf(ps, r2, -5.1677127800499703f);
  ps = fmaf(ps, r2, 3.1415926535897932f);
  float pc = -1.0463810492484570e-4f;  // -pi^14 / 14!
  pc = fmaf(pc, r2, 1.9295743094039231e-3f);
  pc = fmaf(pc, r2, -2.5806891390014061e-2f);
  pc = fmaf(pc, r2, 2.3533063035889320e-1f);
  pc = fmaf(pc, r2, -1.3352627688545894f);
  pc = fmaf(pc, r2, 4.0587121264167683f);
  pc = fmaf(pc, r2, -4.9348022005446793f);
  pc = fmaf(pc, r2, 1.0f);
  const bool odd = (static_cast<int>(n) & 1) != 0;
  s = odd ? -(r * ps) : r * ps;
  c = odd ? -pc : pc;
}
GRN_HD void sincos_pi(float x, float &s, float &c) { sincos_pi_poly(x, s, c); }

// ---------------------------------------------------------------------------
// Model functions, arithmetic type T.

// Double-pole proton form factor (src/MForm.cc:433-435).
template <typename T>
GRN_HD T proton_ff(T fc1, T fc2, T t) {
  return T(1) / ((T(1) - t / fc1) * (T(1) - t / fc2));
}

// Off-shell meson form factor (src/MRegge.cc:1155-1174).
template <typename T>
GRN_HD T meson_ff(const grn_regge_params &rp, T that, T M2) {
  const T tp = that - M2;
  if (rp.offshellFF == 0) return exp(-T(rp.b_EXP) * fabs(tp));
  if (rp.offshellFF == 1)
    return exp(-T(rp.b_OREAR) * sqrt(fabs(tp) + T(rp.a_OREAR) * T(rp.a_OREAR)) +
               T(rp.a_OREAR) * T(rp.b_OREAR));
  return T(1) / (T(1) - tp / T(rp.b_POW));
}

// Inelastic proton vertex of an excited forward leg of mass^2 M2 (S3FINEL, src/MForm.cc:
// 443-449): (|t| / (M2 (|t| + a)))^((1 + Delta_P) / 2), Delta_P = 0.0808, a = 0.5616 GeV^2.
template <typename T>
GRN_HD T proton_ff_inel(T t, T M2) {
  const T at = fabs(t);
  return exp(T(0.5 * (1.0 + 0.0808)) * log(at / (M2 * (at + T(0.5616)))));
}
// Pomeron-proton vertex of forward leg i (MRegge::PomPomProtonVertex, src/MRegge.cc:637-644):
// gN_P F(t) elastic, sqrt(g3P gN_P) S3FINEL(t, M^2) excited (bit i of exc).
template <typename T>
GRN_HD T leg_vertex(const grn_process_params &P, const Consts &K, int exc, int i, T t, T M2) {
  if (exc & (1 << i)) return T(K.gin) * proton_ff_inel<T>(t, M2);
  return T(P.soft.gN_P) * proton_ff<T>(T(P.soft.fc1), T(P.soft.fc2), t);
}

// Regge propagator sum over active trajectories:
//   sum_k ReggeEta(a0_k,sgn_k) exp(-i pi/2 ap_k t) (s/s0)^(a0_k + ap_k t)
// (src/MRegge.cc:888-906 with src/MForm.cc:382-396), from ln s.
template <typename T>
GRN_HD cx<T> regge_prop(const Consts &K, const grn_regge_params &rp, T lns, T t, T off = T(0)) {
  cx<T> M{T(0), T(0)};
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    if (!K.active[k]) continue;
    const T mag = exp((T(rp.a0[k]) + T(rp.ap[k]) * t) * (lns - T(K.lns0)) - off);
    T sn, cs;
    sincos_pi(-T(0.5) * T(rp.ap[k]) * t, sn, cs);
    const cx<T> ph{cs * mag, sn * mag};
    M = cadd(M, cmul(cx<T>{T(K.eta0_re[k]), T(K.eta0_im[k])}, ph));
  }
  return M;
}

// ---------------------------------------------------------------------------
// Tensor-pomeron continuum of two pseudoscalars (MTensorPomeron::ME4 "2xS",
// src/MTensorPomeron.cc:572-898). With the high-energy proton vertex
// -3i gPNN F1(t) P_mu P_nu (P = p' + p, MTensorPomeron.cc:1388), the pomeron
// propagator 1/(4s) (-i s ap)^(alpha(t)-1) (g g + g g - g g / 2) (2288) and the
// traceless pomeron-pseudoscalar vertex -2i g FM(q^2) (Q_a Q_b - g_ab Q^2/4) (2203),
// each exchange contracts to
//   c(s, t) (-6 gPNN g F1(t) FM(t)) (2 (P.Q)^2 - P^2 Q^2 / 2).
// Light-cone dot products a.b = (a+ b- + a- b+)/2 - aT.bT; every large product pairs
// a sqrt(s)-size component with a cancellation-free one.
constexpr double kMpPDG = 0.938272081;  // PDG::mp used by the form factors

// Dirac form factor F1(Q^2) = (GE + tau GM) / (1 + tau) as numerator / denominator (no
// division): Kelly's parameterisation of GE, GM or the dipole.
template <typename T>
GRN_HD void dirac_f1_nd(T Q2, int kelly, T &num, T &den) {
  Q2 = fabs(Q2);
  const T tau = Q2 * T(1.0 / (4.0 * kMpPDG * kMpPDG));
  const T mu  = T(2.792847337);
  if (kelly) {
    const T nE = T(1) - T(0.24) * tau;
    const T dE = T(1) + tau * (T(10.98) + tau * (T(12.82) + tau * T(21.97)));
    const T nM = mu * (T(1) + T(0.12) * tau);
    const T dM = T(1) + tau * (T(10.97) + tau * (T(18.86) + tau * T(6.55)));
    num = nE * dM + tau * nM * dE;
    den = dE * dM * (tau + T(1));
  } else {
    const T d = T(1) + Q2 * T(1.0 / 0.71);
    num = T(1) + tau * mu;
    den = d * d * (tau + T(1));
  }
}

template <typename T>
GRN_HD T dirac_f1(T Q2, int kelly) {
  T n, d;
  dirac_f1_nd<T>(Q2, kelly, n, d);
  return n / d;
}

// Light-cone kinematics of one (tree-level or loop) point.
template <typename T>
struct LCKin {
  T p1p, p1m, p1x, p1y, p2p, p2m, p2x, p2y;  // forward legs
  T p3p, p3m, p3x, p3y, p4p, p4m, p4x, p4y;  // central pair
  T L, eps, mp2;                             // beams: pa = (L, eps, 0), pb = (eps, L, 0)
  T t1, t2, s13, s14, s23, s24, that, uhat;  // invariants
  T q1p, q1m, q2p, q2m;                      // light-cone parts of q1 = pa - p1, q2 = pb - p2
};

// q1+ = x1 L and q1- = -(pT1^2 + x1 mp^2) / ((1 - x1) L), both free of cancellation
// (and likewise for q2 with + and - exchanged).
template <typename T>
GRN_HD void q_lightcone(T x, T ptsq, T mp2, T L, T &big, T &small) {
  big   = x * L;
  small = -(ptsq + x * mp2) / ((T(1) - x) * L);
}

template <typename T>
GRN_HD T lc_dot(T ap, T am, T ax, T ay, T bp, T bm, T bx, T by) {
  return T(0.5) * (ap * bm + am * bp) - (ax * bx + ay * by);
}

// Proton legs of a tensor-pomeron amplitude: F1(t1) FM(t1) F1(t2) FM(t2) with FM(t) =
// 1 / (1 - t / 0.5), as numerator / denominator.
template <typename T>
GRN_HD void proton_legs_nd(const grn_tensor_params &tp, T t1, T t2, T &num, T &den) {
  T n1, d1, n2, d2;
  dirac_f1_nd<T>(t1, tp.em_kelly, n1, d1);
  dirac_f1_nd<T>(t2, tp.em_kelly, n2, d2);
  num = n1 * n2;
  den = d1 * d2 * ((T(1) - T(2) * t1) * (T(1) - T(2) * t2));
}

// Off-shell meson form factor squared over the propagator denominator,
// ff(p^2)^2 / (p^2 - M2), as numerator / denominator (meson_ff).
template <typename T>
GRN_HD void meson_prop_nd(const grn_regge_params &rp, T p2, T M2, T &num, T &den) {
  const T tp = p2 - M2;
  if (rp.offshellFF == 2) {  // (1 / (1 - tp / b))^2 = b^2 / (b - tp)^2
    const T b = T(rp.b_POW), d = b - tp;
    num = b * b;
    den = d * d * tp;
  } else {
    const T f = meson_ff<T>(rp, p2, M2);
    num = f * f;
    den = tp;
  }
}

// Tensor-pomeron continuum of two pseudoscalars (MTensorPomeron::ME4 "2xS"): per exchange
// c(s, t) (-6 gPNN g F1(t) FM(t)) (2 (P.Q)^2 - P^2 Q^2 / 2), c(s, t) = (1/4s) (s ap)^x
// e^{-i pi x / 2}, x = alpha(t) - 1. The t and u channels share t1 and t2, hence the phase
// e^{-i pi (x1 + x2) / 2} and the proton legs F1 FM of both; per channel remains the real
// (ap s)^x1 (ap s')^x2 / (16 s s') with its meson propagator:
//   M = e^{-i pi (x1 + x2)/2} (6 gPNN g)^2 F1 FM F1 FM [w_t v13 v24 R_t + w_u v14 v23 R_u].
template <typename T>
GRN_HD cx<T> tensor_me4_2xs(const grn_process_params &P, const Consts &K, const LCKin<T> &k) {
  const T eps = k.eps, L = k.L;
  // P1 = p1 + pa, P2 = p2 + pb
  const T P1p = k.p1p + L, P1m = k.p1m + eps, P2p = k.p2p + eps, P2m = k.p2m + L;
  const T P1sq = T(2) * k.mp2 + k.p1p * eps + k.p1m * L;
  const T P2sq = T(2) * k.mp2 + k.p2m * eps + k.p2p * L;
  // t-channel meson pt = pa - p1 - p3 (pt+ from conservation: p4+ - eps + p2+)
  const T ptp = k.p4p - eps + k.p2p, ptm = eps - k.p1m - k.p3m;
  const T ptx = -(k.p1x + k.p3x), pty = -(k.p1y + k.p3y);
  // u-channel meson pu = p4 - pa + p1 (pu+ = -(p3+ - eps + p2+))
  const T pup = -(k.p3p - eps + k.p2p), pum = k.p4m - eps + k.p1m;
  const T pux = k.p4x + k.p1x, puy = k.p4y + k.p1y;
  auto vtx = [&](T Pp, T Pm, T Px, T Py, T Psq, T Qp, T Qm, T Qx, T Qy) {
    const T d  = lc_dot<T>(Pp, Pm, Px, Py, Qp, Qm, Qx, Qy);
    const T Q2 = Qp * Qm - (Qx * Qx + Qy * Qy);
    return T(2) * d * d - T(0.5) * Psq * Q2;
  };
  // t channel: Q13 = pt - p3, Q24 = p4 + pt; u channel: Q14 = p4 + pu, Q23 = pu - p3
  const T v13 = vtx(P1p, P1m, k.p1x, k.p1y, P1sq, ptp - k.p3p, ptm - k.p3m, ptx - k.p3x,
                    pty - k.p3y);
  const T v24 = vtx(P2p, P2m, k.p2x, k.p2y, P2sq, k.p4p + ptp, k.p4m + ptm, k.p4x + ptx,
                    k.p4y + pty);
  const T v14 = vtx(P1p, P1m, k.p1x, k.p1y, P1sq, k.p4p + pup, k.p4m + pum, k.p4x + pux,
                    k.p4y + puy);
  const T v23 = vtx(P2p, P2m, k.p2x, k.p2y, P2sq, pup - k.p3p, pum - k.p3m, pux - k.p3x,
                    puy - k.p3y);
  const grn_tensor_params &tp = P.tensor;
  const T M2 = T(K.M2prop), ap = T(tp.ap_P);
  const T x1 = T(tp.delta_P) + ap * k.t1, x2 = T(tp.delta_P) + ap * k.t2;
  T wtn, wtd, wun, wud, ln, ld;
  meson_prop_nd<T>(P.regge, k.that, M2, wtn, wtd);
  meson_prop_nd<T>(P.regge, k.uhat, M2, wun, wud);
  proton_legs_nd<T>(tp, k.t1, k.t2, ln, ld);
  const T Rt = exp(x1 * log(ap * k.s13) + x2 * log(ap * k.s24));
  const T Ru = exp(x1 * log(ap * k.s14) + x2 * log(ap * k.s23));
  // M = -i (i wt v13 v24 At + i wu v14 v23 Au) = wt v13 v24 At + wu v14 v23 Au
  const T B = (wtn * v13 * v24 * Rt) / (T(16) * wtd * k.s13 * k.s24) +
              (wun * v14 * v23 * Ru) / (T(16) * wud * k.s14 * k.s23);
  const T g6 = T(6.0 * tp.gPNN * tp.gPps);
  const T mag = g6 * g6 * B * ln / ld;
  T sn, cs;
  sincos_pi(T(-0.5) * (x1 + x2), sn, cs);
  return {mag * cs, mag * sn};
}

// ---------------------------------------------------------------------------
// Tensor-pomeron resonances decaying to two pseudoscalars, coherent sum
// (MTensorPomeron::ME3, src/MTensorPomeron.cc:164-565, PROC_11). The proton vertex
// -3i gPNN F1(t) P_mu P_nu (P = p' + p, :1388) through the pomeron propagator
// 1/(4s) (-i s ap)^(alpha(t)-1) (g g + g g - g g / 2) (:2288), with s_i = (p_i + X)^2
// (MProcess.cc:1533), gives per leg c(s_i,t_i) (-3i gPNN F1(t_i)) W_i with the traceless
//   W_i = 2 P_i P_i - P_i^2 g / 2.
// Contracted with traceless tensors the vertex structures collapse:
//  J = 2, iG_PPT_total (:1646-1692) with the tensor propagator iD_TMES (:2422-2446) and the
//    decay vertex iG_f2psps (:2121-2137): D = Delta (g_d / 2) F Pi, Pi = kh kh + kh^2 ghat / 3,
//    ghat = -g + X X / m^2, kh = ghat.(p3 - p4), and
//      A = -(9/2) gPNN^2 g_d C F^2 Delta sum_j g_j gamma_j
//    over the seven coupling structures (iG_PPT_00, _12 modes 1 and 2, _03, _04, _05, _06):
//      gamma_0 = 2 tr(W1 W2 Pi),  tr(W1 W2 Pi) = 4 a Pi(P2,P1) - b2 Pi(P1,P1) - b1 Pi(P2,P2),
//      gamma_1 = -2 [4 a M(q1,P1;q2,P2) + 2 beta M(q1,P1;q2,P1) + 2 alpha M(q1,P2;q2,P2)
//                    + 2 alpha beta Pi(q1,q2)],  alpha = -b1/2, beta = -b2/2,
//      gamma_2 = -2 [q1.q2 tr(W1 W2 Pi) + q2 W1 W2 Pi q1 + q1 W2 W1 Pi q2 + tr(W1 W2) Pi(q1,q2)],
//      gamma_3 = -2 Pi(W1 q2, W2 q1),  gamma_4 = -4 E' Pi(q1,q2),
//      gamma_5 = Pi(W1 q2, q2) q1W2q1 + Pi(W2 q1, q1) q2W1q2,
//      gamma_6 = -2 (q2W1q2)(q1W2q1) Pi(q1,q2),
//    with M(a,b;c,d) = (a.c) Pi(b,d) - (a.d) Pi(b,c) - (b.c) Pi(a,d) + (b.d) Pi(a,c) the
//    contraction of the bivectors a^b and c^d (its four products cancel at leading order in
//    s: structure 1 is the difference of structures T2/T3 and T1/R R, (l,s) = (2,0) - (2,2));
//  J = 0, iG_PPS_0 + iG_PPS_1 (:1536-1571) with iD_MES (:2383) and iG_f0ss (:2028):
//      A = 18 gPNN^2 g_d C F^2 Delta [g0 (4 a^2 - b1 b2) + g1 E'],  E' = 4 a E + 5/4 b1 b2 q1.q2;
// C = c(s1,t1) c(s2,t2) F1(t1) F1(t2) FM(t1) FM(t2), FM(q^2) = 1/(1 - q^2), F = exp(-(m^2 -
// M0^2)^2) (the production and the decay form factor), Delta = 1/(m^2 - M0^2 + i M0 W),
// a = P1.P2, b_i = P_i^2 = 4 mp^2 - t_i, q_i = p_beam,i - p_i (P_i.q_i = 0),
// tr(W1 W2) = 4 a^2 - b1 b2, and E = (P1.q2)(P2.q1) - a q1.q2 = M-type bivector contraction of
// P1^q1 and q2^P2 with the metric. The resonance prefactors are Consts::res_c0 (-(9/2) gPNN^2
// g_d for J = 2; 18 gPNN^2 g_d g0 for J = 0), res_c1 (18 gPNN^2 g_d g1, J = 0), res_g.
template <typename T>
GRN_HD T lc_bivector_dot(T ap, T am, T ax, T ay, T bp, T bm, T bx, T by,   // B = a ^ b
                         T cp, T cm, T cx_, T cy, T dp, T dm, T dx, T dy) {  // C = c ^ d
  const T Bpm = ap * bm - am * bp, Cpm = cp * dm - cm * dp;
  const T Bmx = am * bx - ax * bm, Cpx = cp * dx - cx_ * dp;
  const T Bmy = am * by - ay * bm, Cpy = cp * dy - cy * dp;
  const T Bpx = ap * bx - ax * bp, Cmx = cm * dx - cx_ * dm;
  const T Bpy = ap * by - ay * bp, Cmy = cm * dy - cy * dm;
  const T Bxy = ax * by - ay * bx, Cxy = cx_ * dy - cy * dx;
  return T(-0.25) * Bpm * Cpm - T(0.5) * (Bmx * Cpx + Bmy * Cpy + Bpx * Cmx + Bpy * Cmy) +
         Bxy * Cxy;
}

// Pi_ab = Pi(e_a, e_b) on the light-cone basis e+, e-, ex, ey (v = v+ e+ + v- e- + vx ex +
// vy ey), symmetric: ++ +- +x +y -- -x -y xx xy yy. It depends on the central system only,
// which the kt-loop leaves unchanged, so it comes from the tree-level point in FP64 and every
// Pi(v, w) of a loop point is a sum of products of accurate factors: with P1 ~ 2L e+ and
// P2 ~ 2L e- the leading 4 L^2 Pi_+- of Pi(P2,P1) would otherwise cancel, near the zero of the
// d-wave decay distribution, between terms 10^4 times larger than itself.
template <typename T>
struct PiMat {
  T pp, pm, px, py, mm, mx, my, xx, xy, yy;
};

template <typename T>
GRN_HD T pi_form(const PiMat<T> &M, T ap, T am, T ax, T ay, T bp, T bm, T bx, T by) {
  return ap * bp * M.pp + (ap * bm + am * bp) * M.pm + (ap * bx + ax * bp) * M.px +
         (ap * by + ay * bp) * M.py + am * bm * M.mm + (am * bx + ax * bm) * M.mx +
         (am * by + ay * bm) * M.my + ax * bx * M.xx + (ax * by + ay * bx) * M.xy + ay * by * M.yy;
}

// M(a,b;c,d) = sum B^{mu nu} g_{mu rho} C^{rho sigma} Pi_{nu sigma}, B = a^b, C = c^d, metric
// g_{+-} = 1/2, g_xx = g_yy = -1 on the light-cone basis.
template <typename T>
GRN_HD T pi_bivector(const PiMat<T> &M, const T a[4], const T b[4], const T c[4], const T d[4]) {
  // components above the diagonal only: the diagonal is zero exactly (a contracted
  // a[i] b[i] - a[i] b[i] would leave the rounding error of one product), below it antisymmetric
  T B[4][4], C[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    B[i][i] = C[i][i] = T(0);
#pragma unroll
    for (int j = i + 1; j < 4; ++j) {
      B[i][j] = a[i] * b[j] - a[j] * b[i];
      C[i][j] = c[i] * d[j] - c[j] * d[i];
      B[j][i] = -B[i][j];
      C[j][i] = -C[i][j];
    }
  }
  const T Pi[4][4] = {{M.pp, M.pm, M.px, M.py},
                      {M.pm, M.mm, M.mx, M.my},
                      {M.px, M.mx, M.xx, M.xy},
                      {M.py, M.my, M.xy, M.yy}};
  T out = T(0);
#pragma unroll
  for (int nu = 0; nu < 4; ++nu)
#pragma unroll
    for (int sg = 0; sg < 4; ++sg) {
      const T Y = T(0.5) * (B[0][nu] * C[1][sg] + B[1][nu] * C[0][sg]) - B[2][nu] * C[2][sg] -
                  B[3][nu] * C[3][sg];
      out += Y * Pi[nu][sg];
    }
  return out;
}

// Resonance sums of the tree-level central mass: Rs[j] = sum_{J=2} res_c0 g_j F^2 Delta,
// R0 = sum_{J=0} res_c0 F^2 Delta, R1 = sum_{J=0} res_c1 F^2 Delta; and Pi on the basis.
template <typename T>
struct ResSums {
  cx<T>    Rs[7], R0, R1;
  PiMat<T> pi;
};

// Resonance-side vectors: X = p3 + p4, kh = ghat.(p3 - p4) and kh^2 (kh^2 = (p3 - p4)^2 -
// (X.k)^2 / m^2 with X.k = m3^2 - m4^2).
template <typename T>
struct ResVec {
  T Xp, Xm, Xx, Xy, m2, khp, khm, khx, khy, kh2;
};

template <typename T>
GRN_HD ResVec<T> res_vectors(const Consts &K, T p3p, T p3m, T p3x, T p3y, T p4p, T p4m, T p4x,
                             T p4y) {
  ResVec<T> v;
  v.Xp = p3p + p4p; v.Xm = p3m + p4m; v.Xx = p3x + p4x; v.Xy = p3y + p4y;
  v.m2 = v.Xp * v.Xm - (v.Xx * v.Xx + v.Xy * v.Xy);
  const T pk = T(K.m3sq - K.m4sq);
  const T c  = pk / v.m2;
  v.khp = -(p3p - p4p) + c * v.Xp;
  v.khm = -(p3m - p4m) + c * v.Xm;
  v.khx = -(p3x - p4x) + c * v.Xx;
  v.khy = -(p3y - p4y) + c * v.Xy;
  v.kh2 = T(2) * T(K.m3sq + K.m4sq) - v.m2 - pk * c;
  return v;
}

// Pi_ab = kappa_a kappa_b + kh^2/3 (xi_a xi_b / m^2 - g_ab) with kappa_a = kh.e_a,
// xi_a = X.e_a (e+.v = v-/2, e-.v = v+/2, ex.v = -vx, ey.v = -vy).
GRN_HD PiMat<double> pi_matrix(const ResVec<double> &v) {
  const double k[4] = {0.5 * v.khm, 0.5 * v.khp, -v.khx, -v.khy};
  const double x[4] = {0.5 * v.Xm, 0.5 * v.Xp, -v.Xx, -v.Xy};
  const double t = v.kh2 / 3.0, im2 = 1.0 / v.m2;
  auto e = [&](int i, int j, double g) { return k[i] * k[j] + t * (x[i] * x[j] * im2 - g); };
  return {e(0, 0, 0.0), e(0, 1, 0.5), e(0, 2, 0.0), e(0, 3, 0.0), e(1, 1, 0.0),
          e(1, 2, 0.0), e(1, 3, 0.0), e(2, 2, -1.0), e(2, 3, 0.0), e(3, 3, -1.0)};
}

GRN_HD ResSums<double> resonance_sums(const Consts &K, double m2, const ResVec<double> &v) {
  ResSums<double> R;
  for (int j = 0; j < 7; ++j) R.Rs[j] = {0, 0};
  R.R0 = R.R1 = {0, 0};
  for (int r = 0; r < K.n_res; ++r) {
    const double dm = m2 - K.res_M2[r], mw = K.res_MW[r];
    const double f2 = exp(-2.0 * dm * dm) / (dm * dm + mw * mw);  // F^2 / |m^2 - M0^2 + i M0 W|^2
    const cx<double> D{dm * f2, -mw * f2};
    if (K.res_J[r] == 2) {
      for (int j = 0; j < 7; ++j)
        R.Rs[j] = cadd(R.Rs[j], cscale(D, K.res_c0[r] * K.res_g[r][j]));
    } else {
      R.R0 = cadd(R.R0, cscale(D, K.res_c0[r]));
      R.R1 = cadd(R.R1, cscale(D, K.res_c1[r]));
    }
  }
  R.pi = pi_matrix(v);
  return R;
}

template <typename T>
GRN_HD cx<T> tensor_me3(const grn_process_params &P, const Consts &K, const LCKin<T> &k,
                        const ResSums<T> &R) {
  const T L = k.L, eps = k.eps;
  const T P1p = k.p1p + L, P1m = k.p1m + eps, P2p = k.p2p + eps, P2m = k.p2m + L;
  const T b1 = T(4) * k.mp2 - k.t1, b2 = T(4) * k.mp2 - k.t2;
  const T a  = lc_dot<T>(P1p, P1m, k.p1x, k.p1y, P2p, P2m, k.p2x, k.p2y);
  const T Xp = k.p3p + k.p4p, Xm = k.p3m + k.p4m, Xx = k.p3x + k.p4x, Xy = k.p3y + k.p4y;
  const T m2 = Xp * Xm - (Xx * Xx + Xy * Xy);
  const T s1 = k.mp2 + m2 + k.p1p * Xm + k.p1m * Xp - T(2) * (k.p1x * Xx + k.p1y * Xy);
  const T s2 = k.mp2 + m2 + k.p2p * Xm + k.p2m * Xp - T(2) * (k.p2x * Xx + k.p2y * Xy);
  // P_i and q_i = p_beam,i - p_i = (q+, q-, -p_iT)
  const T P1[4] = {P1p, P1m, k.p1x, k.p1y}, P2[4] = {P2p, P2m, k.p2x, k.p2y};
  const T q1[4] = {k.q1p, k.q1m, -k.p1x, -k.p1y}, q2[4] = {k.q2p, k.q2m, -k.p2x, -k.p2y};
  auto pif = [&](const T *u, const T *w) {
    return pi_form<T>(R.pi, u[0], u[1], u[2], u[3], w[0], w[1], w[2], w[3]);
  };
  auto dot = [&](const T *u, const T *w) {
    return lc_dot<T>(u[0], u[1], u[2], u[3], w[0], w[1], w[2], w[3]);
  };
  const int mask = K.res_smask;
  cx<T> G{T(0), T(0)};
  const bool j0 = R.R0.re != T(0) || R.R0.im != T(0) || R.R1.re != T(0) || R.R1.im != T(0);
  T q1q2 = T(0), Ep = T(0);
  if (j0 || (mask & 0x16)) {  // E' for J = 0 and structure 4; q1.q2 for structures 1, 2, 4
    q1q2 = dot(q1, q2);
    const T E = lc_bivector_dot<T>(P1p, P1m, k.p1x, k.p1y, q1[0], q1[1], q1[2], q1[3], q2[0],
                                   q2[1], q2[2], q2[3], P2p, P2m, k.p2x, k.p2y);
    Ep = T(4) * a * E + T(1.25) * b1 * b2 * q1q2;
  }
  if (mask) {
    const T Pi21 = pif(P2, P1), Pi11 = pif(P1, P1), Pi22 = pif(P2, P2);
    const T Tr   = T(4) * a * Pi21 - b2 * Pi11 - b1 * Pi22;
    G = cadd(G, cscale(R.Rs[0], T(2) * Tr));
    if (mask & ~1) {
      const T trW  = T(4) * a * a - b1 * b2;
      const T P1q2 = dot(P1, q2), P2q1 = dot(P2, q1);
      const T Pq12 = pif(q1, q2);
      const T al = T(-0.5) * b1, be = T(-0.5) * b2;
      if (mask & 2) {  // (l,s) = (2,0) - (2,2): bivector form
        const T F1 = T(4) * a * pi_bivector<T>(R.pi, q1, P1, q2, P2) +
                     T(2) * be * pi_bivector<T>(R.pi, q1, P1, q2, P1) +
                     T(2) * al * pi_bivector<T>(R.pi, q1, P2, q2, P2) + T(2) * al * be * Pq12;
        G = cadd(G, cscale(R.Rs[1], T(-2) * F1));
      }
      const T PP1q1 = pif(P1, q1), PP2q2 = pif(P2, q2);
      if (mask & 4) {  // (l,s) = (2,0) + (2,2)
        const T Pu1q1 = T(2) * P1q2 * PP1q1 - T(0.5) * b1 * Pq12;
        const T Pu2q2 = T(2) * P2q1 * PP2q2 - T(0.5) * b2 * Pq12;
        const T c12   = T(4) * a * P1q2 * pif(P2, q1) - T(0.5) * b2 * Pu1q1;
        const T c21   = T(4) * a * P2q1 * pif(P1, q2) - T(0.5) * b1 * Pu2q2;
        G = cadd(G, cscale(R.Rs[2], T(-2) * (q1q2 * Tr + c12 + c21 + trW * Pq12)));
      }
      if (mask & 8) {  // (l,s) = (2,4): Pi(W1 q2, W2 q1)
        const T Pu1u2 = T(4) * P1q2 * P2q1 * Pi21 - b2 * P1q2 * PP1q1 - b1 * P2q1 * PP2q2 +
                        T(0.25) * b1 * b2 * Pq12;
        G = cadd(G, cscale(R.Rs[3], T(-2) * Pu1u2));
      }
      if (mask & 16)  // (l,s) = (4,2)
        G = cadd(G, cscale(R.Rs[4], T(-4) * Ep * Pq12));
      if (mask & 0x60) {
        const T X1 = T(2) * P1q2 * P1q2 - T(0.5) * b1 * k.t2;  // q2 W1 q2
        const T X2 = T(2) * P2q1 * P2q1 - T(0.5) * b2 * k.t1;  // q1 W2 q1
        if (mask & 32) {  // (l,s) = (4,4)
          const T Pu1q2 = T(2) * P1q2 * pif(P1, q2) - T(0.5) * b1 * pif(q2, q2);
          const T Pu2q1 = T(2) * P2q1 * pif(P2, q1) - T(0.5) * b2 * pif(q1, q1);
          G = cadd(G, cscale(R.Rs[5], Pu1q2 * X2 + Pu2q1 * X1));
        }
        if (mask & 64)  // (l,s) = (6,4)
          G = cadd(G, cscale(R.Rs[6], T(-2) * X1 * X2 * Pq12));
      }
    }
  }
  if (j0) {
    const T S0 = T(4) * a * a - b1 * b2;
    G = cadd(G, cadd(cscale(R.R0, S0), cscale(R.R1, Ep)));
  }
  // C = c(s1,t1) c(s2,t2) F1 F1 FM FM with c(s,t) = (s ap)^x e^{-i pi x/2} / (4s), x = alpha(t)-1
  const grn_tensor_params &tp = P.tensor;
  const T x1 = T(tp.delta_P) + T(tp.ap_P) * k.t1, x2 = T(tp.delta_P) + T(tp.ap_P) * k.t2;
  const T mag = exp(x1 * log(s1 * T(tp.ap_P)) + x2 * log(s2 * T(tp.ap_P))) / (T(16) * s1 * s2) *
                dirac_f1<T>(k.t1, tp.em_kelly) * dirac_f1<T>(k.t2, tp.em_kelly) /
                ((T(1) - k.t1) * (T(1) - k.t2));
  T sn, cs;
  sincos_pi(T(-0.5) * (x1 + x2), sn, cs);
  return cmul(G, cx<T>{mag * cs, mag * sn});
}

// ---------------------------------------------------------------------------
// Tensor-pomeron continuum of two vector mesons, "2xV" (MTensorPomeron::ME4,
// src/MTensorPomeron.cc:808-888). Each pomeron-vector-vector vertex iG_Pvv (:2224-2237,
// i FM(q^2, 0.5) (2 g1 Gamma0 - g2 Gamma2), :2500-2529) is contracted with its pomeron leg
// W = 2 P P - P^2 g / 2 (proton vertex through the pomeron propagator, as for 2xS) and with
// the polarization vector e of its external vector meson (e.x = 0). With x the external and
// y the other meson momentum of the vertex (Gamma(k1, k2) with {k1, k2} = {y, x}):
//   vertex . W . e = ce e + cx x + cP P,
//   ce = 4 g1 (yWx)(x.y) + g2 (b x.y - 2 yWx),
//   cx = -4 g1 (yWx)(y.e) - g2 (b y.e - 2 eWy),
//   cP = -4 g2 ((x.y)(P.e) - (y.e)(P.x)),
// so that the two vertices of a channel meet through the vector propagator iD_V (:2353-2369)
// as one Minkowski product of two vectors. The nine amplitudes e3_i.M.e4_j of a real
// polarization basis give the reference's sum over the helicity states (MassiveSpin1PolSum,
// :1243-1263) of |amplitude|^2.
template <typename T>
struct LV {
  T p, m, x, y;  // light-cone components (+, -) and transverse
};
template <typename T>
GRN_HD T ldot(const LV<T> &a, const LV<T> &b) {
  return lc_dot<T>(a.p, a.m, a.x, a.y, b.p, b.m, b.x, b.y);
}

template <typename T>
GRN_HD LV<T> vv_vertex(const LV<T> &e, const LV<T> &x, const LV<T> &y, const LV<T> &P, T b, T g1,
                       T g2) {
  const T xy = ldot(x, y), Px = ldot(P, x), Py = ldot(P, y), Pe = ldot(P, e), ye = ldot(y, e);
  const T yWx = T(2) * Py * Px - T(0.5) * b * xy;
  const T eWy = T(2) * Pe * Py - T(0.5) * b * ye;
  const T ce  = T(4) * g1 * yWx * xy + g2 * (b * xy - T(2) * yWx);
  const T cx_ = -T(4) * g1 * yWx * ye - g2 * (b * ye - T(2) * eWy);
  const T cP  = -T(4) * g2 * (xy * Pe - ye * Px);
  return {ce * e.p + cx_ * x.p + cP * P.p, ce * e.m + cx_ * x.m + cP * P.m,
          ce * e.x + cx_ * x.x + cP * P.x, ce * e.y + cx_ * x.y + cP * P.y};
}

// Real polarization basis of a massive vector (light-cone momentum): two transverse unit
// vectors (z x p^, p^ x t1; x x p^ near the z axis) and the longitudinal (|p|/m, E p^/m).
template <typename T>
GRN_HD void vector_basis(T pp, T pm, T px, T py, LV<T> e[3]) {
  const T E = T(0.5) * (pp + pm), pz = T(0.5) * (pp - pm);
  const T m = sqrt(pp * pm - (px * px + py * py));
  const T P = sqrt(px * px + py * py + pz * pz);
  T n[3] = {T(0), T(0), T(1)};
  if (P > T(1e-12)) { n[0] = px / P; n[1] = py / P; n[2] = pz / P; }
  T a[3] = {T(0), T(0), T(1)};
  if (fabs(n[2]) > T(0.9)) { a[0] = T(1); a[2] = T(0); }
  T t1[3] = {a[1] * n[2] - a[2] * n[1], a[2] * n[0] - a[0] * n[2], a[0] * n[1] - a[1] * n[0]};
  const T nt = sqrt(t1[0] * t1[0] + t1[1] * t1[1] + t1[2] * t1[2]);
  t1[0] /= nt; t1[1] /= nt; t1[2] /= nt;
  const T t2[3] = {n[1] * t1[2] - n[2] * t1[1], n[2] * t1[0] - n[0] * t1[2],
                   n[0] * t1[1] - n[1] * t1[0]};
  e[0] = {t1[2], -t1[2], t1[0], t1[1]};
  e[1] = {t2[2], -t2[2], t2[0], t2[1]};
  const T l0 = P / m, ls = E / m;
  e[2] = {l0 + ls * n[2], l0 - ls * n[2], ls * n[0], ls * n[1]};
}

// Reggeized vector propagator iD_V (:2353-2369): -(e^{i phi} s34 / (4 M0^2))^(alpha - 1) /
// (p^2 - M0^2), alpha = 0.5 + 0.9 p^2, phi = pi/2 exp((4 M0^2 - s34) / (4 M0^2)) - pi/2. Its
// s34-dependent factors are constants of an event (the central pair does not change in the
// loop): lns = ln(s34 / (4 M0^2)) and phi / pi.
template <typename T>
struct VProp {
  T lns, ph;
};
template <typename T>
GRN_HD VProp<T> vector_prop_consts(T M0sq, T s34) {
  const T sth = T(4) * M0sq;
  return {log(s34 / sth), T(0.5) * (exp((sth - s34) / sth) - T(1))};
}

// The nine amplitudes A[3 i + j] = e3_i . M . e4_j of one proton helicity configuration. Both
// channels share t1 and t2, hence the pomeron phase e^{-i pi (x1 + x2) / 2} and the proton
// legs; per channel remain the pomeron magnitudes (ap s)^x1 (ap s')^x2 / (16 s s'), the vector
// propagator and the off-shell form factors, with one exponential and one phase each.
template <typename T>
GRN_HD void tensor_me4_2xv(const grn_process_params &P, const Consts &K, const LCKin<T> &k,
                           const VProp<T> &vp, const LV<T> e3[3], const LV<T> e4[3], cx<T> A[9]) {
  const grn_tensor_params &tp = P.tensor;
  const T L = k.L, eps = k.eps;
  const LV<T> P1{k.p1p + L, k.p1m + eps, k.p1x, k.p1y};
  const LV<T> P2{k.p2p + eps, k.p2m + L, k.p2x, k.p2y};
  const T b1 = T(4) * k.mp2 - k.t1, b2 = T(4) * k.mp2 - k.t2;
  const LV<T> p3{k.p3p, k.p3m, k.p3x, k.p3y}, p4{k.p4p, k.p4m, k.p4x, k.p4y};
  // pt = q1 - p3, pu = p4 - q1 (q1 = pa - p1 = (q1+, q1-, -p1T))
  const LV<T> pt{k.q1p - k.p3p, k.q1m - k.p3m, -k.p1x - k.p3x, -k.p1y - k.p3y};
  const LV<T> mpt{-pt.p, -pt.m, -pt.x, -pt.y};
  const LV<T> pu{k.p4p - k.q1p, k.p4m - k.q1m, k.p4x + k.p1x, k.p4y + k.p1y};
  const LV<T> mpu{-pu.p, -pu.m, -pu.x, -pu.y};
  const T g1 = T(tp.gPvv[0]), g2 = T(tp.gPvv[1]);
  // channel constants (-3i gPNN F1)^2 (i FM)^2 c c ff^2 D_V = 9 gPNN^2 F1 F1 FM FM c c ff^2 D_V
  const T M0sq = T(K.M2prop), ap = T(tp.ap_P);
  const T x1 = T(tp.delta_P) + ap * k.t1, x2 = T(tp.delta_P) + ap * k.t2;
  T ln, ld, wtn, wtd, wun, wud;
  proton_legs_nd<T>(tp, k.t1, k.t2, ln, ld);
  meson_prop_nd<T>(P.regge, k.that, M0sq, wtn, wtd);  // ff^2 / (p^2 - M0^2)
  meson_prop_nd<T>(P.regge, k.uhat, M0sq, wun, wud);
  const T at = T(-0.5) + T(0.9) * k.that, au = T(-0.5) + T(0.9) * k.uhat;  // alpha - 1
  const T com = T(-9.0 * tp.gPNN * tp.gPNN / 16.0) * ln / ld;
  const T mt = com * wtn * exp(x1 * log(ap * k.s13) + x2 * log(ap * k.s24) + at * vp.lns) /
               (wtd * k.s13 * k.s24);
  const T mu = com * wun * exp(x1 * log(ap * k.s14) + x2 * log(ap * k.s23) + au * vp.lns) /
               (wud * k.s14 * k.s23);
  const T ph0 = T(-0.5) * (x1 + x2);
  T snt, cst, snu, csu;
  sincos_pi(ph0 + at * vp.ph, snt, cst);
  sincos_pi(ph0 + au * vp.ph, snu, csu);
  const cx<T> Ct{mt * cst, mt * snt}, Cu{mu * csu, mu * snu};
  LV<T> a_t[3], b_t[3], a_u[3], b_u[3];
  for (int i = 0; i < 3; ++i) {
    a_t[i] = vv_vertex<T>(e3[i], p3, pt, P1, b1, g1, g2);   // upper, t channel
    b_t[i] = vv_vertex<T>(e4[i], p4, mpt, P2, b2, g1, g2);  // lower, t channel
    a_u[i] = vv_vertex<T>(e4[i], p4, mpu, P1, b1, g1, g2);  // upper, u channel
    b_u[i] = vv_vertex<T>(e3[i], p3, pu, P2, b2, g1, g2);   // lower, u channel
  }
  // M = -i (M_t + M_u)
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      const T dt = ldot(a_t[i], b_t[j]), du = ldot(a_u[j], b_u[i]);
      const T re = Ct.re * dt + Cu.re * du, im = Ct.im * dt + Cu.im * du;
      A[3 * i + j] = {im, -re};
    }
}

// ---------------------------------------------------------------------------
// Born (tree-level) kinematics of p p -> p (a b) p in the <C> class, FP64.
struct Born {
  // forward legs
  double p1x, p1y, p2x, p2y;   // transverse momenta
  double pt1sq, pt2sq;
  double x1, x2;               // light-cone momentum-fraction losses
  double p1p, p1m, p2p, p2m;   // light-cone components (+, -)
  // central pair
  double p3x, p3y, p4x, p4y;
  double p3p, p3m, p4p, p4m;
  double mt3, mt4, y3, y4;
  double jx;                   // class-specific Jacobian factor: kt (<C>),
                               // p*/M_X x (M_max^2 - M_min^2) (<F>)
  double m3sq, m4sq;           // central masses^2 (off-shell ones for cascades)
  int    leafok;               // cascades: all four daughters pass the particle cuts
  // forward legs: masses^2 (mp^2, or an excited N* mass^2), excitation bits (1: leg 1, 2:
  // leg 2) and the forward-mass volume factor of the weight (1 when elastic)
  double mf1sq, mf2sq, jf;
  int    exc;
  // invariants
  double t1, t2, s13, s14, s23, s24, that, uhat, m2;
};

// Forward-leg light-cone solution given the central pair's P+, P- and the two forward
// transverse masses^2: longitudinal conservation
//   x1 = a1 + c2 / (1 - x2),  x2 = a2 + c1 / (1 - x1),  a = (P+- - eps) / L, c = mT^2 / L^2.
// Eliminating x2 gives for d = x1 - a1 the quadratic b2 d^2 - (b1 b2 - c1 + c2) d + b1 c2 = 0
// (b = 1 - a), whose small root d = 2 b1 c2 / (B + sqrt(B^2 - 4 b1 b2 c2)), B = b1 b2 - c1 + c2,
// is free of cancellation for elastic legs (c ~ 1e-8) and excited ones (c up to M^2 / s).
// Same physical root as kinematics::SolvePz (include/Graniitti/MKinematics.h:220) picks
// (forward-going legs, MContinuum.cc:375-380).
template <typename T>
GRN_HD bool solve_x(T a1, T a2, T c1, T c2, T &x1, T &x2) {
  const T b1 = T(1) - a1, b2 = T(1) - a2;
  const T B  = b1 * b2 - c1 + c2;
  const T D  = B * B - T(4) * b1 * b2 * c2;
  if (!(B > T(0) && D >= T(0))) return false;
  x1 = a1 + T(2) * b1 * c2 / (B + sqrt(D));
  x2 = a2 + c1 / (T(1) - x1);
  return (x1 > T(0)) && (x2 > T(0)) && (x1 < T(1)) && (x2 < T(1));
}

// BNRandomKin + BNBuildKin + GetLorentzScalars for Kf = 2
// (src/MContinuum.cc:276-435, src/MProcess.cc:1499-1584).
GRN_HD bool born_invariants(const Consts &K, Born &b);

GRN_HD void cascade_masses(const grn_process_params &P, const Consts &K, const double *u,
                           double &m3, double &m4);
GRN_HD_COLD int cascade_cuts(const grn_process_params &P, int dec0, double p3x, double p3y,
                             double p3z, double E3, double m3, double p4x, double p4y, double p4z,
                             double E4, double m4, const double *u);

// Forward legs' masses (MProcess::SampleForwardMasses, src/MProcess.cc:1317-1365): elastic,
// or excited N* masses^2 log-uniform in [1.09^2, xi_max s] from u_m0 (and u_m1 for double
// excitation); single excitation takes the side from u_side (< 0.5: leg 1). The weight gains
// M^2 x (log range) per excited leg (ForwardVolume, src/MProcess.cc:1399-1413).
GRN_HD void forward_masses(const grn_process_params &P, const Consts &K, double u_m0,
                           double u_m1, double u_side, Born &b) {
  b.mf1sq = b.mf2sq = K.mp2;
  b.exc   = 0;
  b.jf    = 1.0;
  if (!P.excitation) return;
  const double range = K.lnM2f_hi - K.lnM2f_lo;
  if (P.excitation == 1) {
    const double M2 = exp(K.lnM2f_lo + range * u_m0);
    if (u_side < 0.5) {
      b.mf1sq = M2;
      b.exc   = 1;
    } else {
      b.mf2sq = M2;
      b.exc   = 2;
    }
    b.jf = M2 * range;
  } else {
    b.mf1sq = exp(K.lnM2f_lo + range * u_m0);
    b.mf2sq = exp(K.lnM2f_lo + range * u_m1);
    b.exc   = 3;
    b.jf    = b.mf1sq * range * b.mf2sq * range;
  }
}

// CASC: the instantiation serves two-body cascades of the central particles (their masses
// from cascade_masses, the daughters from the decay coordinates, particle cuts on them).
template <bool CASC>
GRN_HD bool born_kinematics_C(const grn_process_params &P, const Consts &K, const double *u,
                              Born &b) {
  const grn_gencuts &g = P.gcuts;
  const double pt1 = exp(K.lnpt_lo + (K.lnpt_hi - K.lnpt_lo) * u[0]);
  const double pt2 = exp(K.lnpt_lo + (K.lnpt_hi - K.lnpt_lo) * u[1]);
  double s1, c1, s2, c2, sk, ck;
  sincos_pi(2.0 * u[2], s1, c1);
  sincos_pi(2.0 * u[3], s2, c2);
  const double kt = g.kt_min + (g.kt_max - g.kt_min) * u[4];
  sincos_pi(2.0 * u[5], sk, ck);
  b.y3 = g.rap_min + (g.rap_max - g.rap_min) * u[6];
  b.y4 = g.rap_min + (g.rap_max - g.rap_min) * u[7];
  b.jx = kt;

  b.p1x = pt1 * c1;
  b.p1y = pt1 * s1;
  b.p2x = pt2 * c2;
  b.p2y = pt2 * s2;
  b.pt1sq = b.p1x * b.p1x + b.p1y * b.p1y;
  b.pt2sq = b.p2x * b.p2x + b.p2y * b.p2y;
  // Central pair transverse momenta from the linear system (MContinuum.cc:438-550).
  const double wx = b.p1x + b.p2x, wy = b.p1y + b.p2y;
  const double qx = kt * ck, qy = kt * sk;
  b.p3x = 0.5 * (qx - wx);
  b.p3y = 0.5 * (qy - wy);
  b.p4x = 0.5 * (-qx - wx);
  b.p4y = 0.5 * (-qy - wy);
  double m3 = K.m3, m4 = K.m4;
  b.m3sq = K.m3sq;
  b.m4sq = K.m4sq;
  if (CASC && P.n_decay == 2) {
    cascade_masses(P, K, u, m3, m4);  // BNRandomKin: GetOffShellMass of each central particle
    b.m3sq = m3 * m3;
    b.m4sq = m4 * m4;
  }
  b.leafok = 1;
  b.mt3 = sqrt(b.m3sq + b.p3x * b.p3x + b.p3y * b.p3y);
  b.mt4 = sqrt(b.m4sq + b.p4x * b.p4x + b.p4y * b.p4y);
  const double e3 = exp(b.y3), e4 = exp(b.y4);
  b.p3p = b.mt3 * e3;
  b.p3m = b.mt3 / e3;
  b.p4p = b.mt4 * e4;
  b.p4m = b.mt4 / e4;
  const double Pp = b.p3p + b.p4p, Pm = b.p3m + b.p4m;
  if (0.5 * (Pp + Pm) > K.sqrt_s) return false;  // crude energy check (MContinuum.cc:373)
  // forward masses: u[8] (and u[9] for double excitation; the side draw u[9] for single).
  // Excited processes have 10 coordinates, so they run the 16-dimensional instantiation;
  // the 8-dimensional one never reads past u[7].
  if (CASC)
    forward_masses(P, K, u[8], u[9], u[9], b);
  else
    forward_masses(P, K, 0.0, 0.0, 0.0, b);
  if (CASC && P.n_decay == 2) {
    // isotropic decays of the two central particles (ConstructDecayKinematics); the particle
    // cuts act on the four daughters (FindDecayCuts, src/MProcess.cc:1140-1154)
    b.leafok = cascade_cuts(P, K.dec0, b.p3x, b.p3y, b.mt3 * sinh(b.y3), b.mt3 * cosh(b.y3), m3,
                            b.p4x, b.p4y, b.mt4 * sinh(b.y4), b.mt4 * cosh(b.y4), m4, u);
  }
  return born_invariants(K, b);
}

// Forward legs (light-cone closure) and Lorentz scalars of the tree-level event from
// the central pair (p3, p4 transverse and light-cone components) and the forward
// transverse momenta already in b (MContinuum.cc:372-384, MFactorized.cc:327-343,
// MProcess.cc:1499-1584).
GRN_HD bool born_invariants(const Consts &K, Born &b) {
  const double Pp = b.p3p + b.p4p, Pm = b.p3m + b.p4m;
  const double mT1sq = b.mf1sq + b.pt1sq, mT2sq = b.mf2sq + b.pt2sq;
  if (!solve_x((Pp - K.eps) * K.invL, (Pm - K.eps) * K.invL, mT1sq * K.invL2, mT2sq * K.invL2,
               b.x1, b.x2))
    return false;
  // 1 / (1 - x) of each leg, shared by its minus (plus) component and its t
  const double r1 = 1.0 / (1.0 - b.x1), r2 = 1.0 / (1.0 - b.x2);
  b.p1p = (1.0 - b.x1) * K.L;
  b.p1m = mT1sq * r1 * K.invL;
  b.p2m = (1.0 - b.x2) * K.L;
  b.p2p = mT2sq * r2 * K.invL;

  // Invariants: (pa + pb)^2 = ma^2 + mb^2 + pa+ pb- + pa- pb+ - 2 paT.pbT
  // t = (pb - p)^2 = -(pT^2 + x (m_f^2 - mp^2) + x^2 mp^2) / (1 - x): same-sign terms (m_f >= mp)
  b.t1  = -(b.pt1sq + b.x1 * (b.mf1sq - K.mp2) + b.x1 * b.x1 * K.mp2) * r1;
  b.t2  = -(b.pt2sq + b.x2 * (b.mf2sq - K.mp2) + b.x2 * b.x2 * K.mp2) * r2;
  b.s13 = b.mf1sq + b.m3sq + b.p1p * b.p3m + b.p1m * b.p3p - 2.0 * (b.p1x * b.p3x + b.p1y * b.p3y);
  b.s14 = b.mf1sq + b.m4sq + b.p1p * b.p4m + b.p1m * b.p4p - 2.0 * (b.p1x * b.p4x + b.p1y * b.p4y);
  b.s23 = b.mf2sq + b.m3sq + b.p2p * b.p3m + b.p2m * b.p3p - 2.0 * (b.p2x * b.p3x + b.p2y * b.p3y);
  b.s24 = b.mf2sq + b.m4sq + b.p2p * b.p4m + b.p2m * b.p4p - 2.0 * (b.p2x * b.p4x + b.p2y * b.p4y);
  b.m2  = b.m3sq + b.m4sq + b.p3p * b.p4m + b.p3m * b.p4p - 2.0 * (b.p3x * b.p4x + b.p3y * b.p4y);
  // t_hat = (q1 - p3)^2 with q1 = pb1 - p1: (q1+ - p3+) = p4+ - eps + p2+ by conservation.
  {
    const double dp = b.p4p - K.eps + b.p2p;
    const double dm = K.eps - b.p1m - b.p3m;
    const double tx = b.p1x + b.p3x, ty = b.p1y + b.p3y;
    b.that = dp * dm - (tx * tx + ty * ty);
  }
  {
    const double dp = b.p3p - K.eps + b.p2p;
    const double dm = K.eps - b.p1m - b.p4m;
    const double tx = b.p1x + b.p4x, ty = b.p1y + b.p4y;
    b.uhat = dp * dm - (tx * tx + ty * ty);
  }
  return true;
}


// Relativistic Breit-Wigner mass by inverse CDF in m^2 on [max(M_MIN, m0 - n W)^2,
// (m0 + n W)^2], n = OFFSHELL widths (MRandom::RelativisticBWRandom, src/MRandom.cc:82-104;
// include/Graniitti/MProcess.h:363) from the uniform R; n = 0 gives the pole mass.
GRN_HD double bw_mass(double m0, double W, double n, double M_MIN, double R) {
  if (W < 1e-40) return m0;
  const double m2    = m0 * m0;
  const double m2max = (m0 + n * W) * (m0 + n * W);
  const double m2min = fmax(fmax(0.0, M_MIN * M_MIN), (m0 - n * W) * (m0 - n * W));
  const double a = atan2(m2min - m2, m0 * W), c = atan2(m2max - m2, m0 * W);
  const double v = m2 + m0 * W * tan(a + R * (c - a));
  return fmax(M_MIN, sqrt(fmax(0.0, v)));
}

// Off-shell masses of the two central particles of a cascade (GetOffShellMass: the
// daughters' mass sum + 1e-5 GeV bounds the Breit-Wigner from below) from u[8], u[9]; the
// pole masses when OFFSHELL = 0 (no mass coordinates).
GRN_HD void cascade_masses(const grn_process_params &P, const Consts &K, const double *u,
                           double &m3, double &m4) {
  m3 = P.m_central[0];
  m4 = P.m_central[1];
  if (K.offshell > 0.0) {
    m3 = bw_mass(m3, P.width[0], K.offshell, P.m_daughter[0] + P.m_daughter[1] + 1e-5, u[8]);
    m4 = bw_mass(m4, P.width[1], K.offshell, P.m_daughter[2] + P.m_daughter[3] + 1e-5, u[9]);
  }
}

// Two-body decay of a mother (px, py, pz, E; mass M) into masses ma, mb with (cos theta,
// phi) in its rest frame, boosted to the lab (TwoBodyPhaseSpace, LorentzBoost,
// include/Graniitti/MKinematics.h:384-459); out: (px, py, pz, E) of a and b.
GRN_HD void decay2(double px, double py, double pz, double E, double M, double ma, double mb,
                   double ct, double phi_frac, double a[4], double bb[4]) {
  const double ms = ma + mb, md = ma - mb;
  const double pn = sqrt(fmax(0.0, (M - ms) * (M + ms) * (M + md) * (M - md))) / (2.0 * M);
  const double st = sqrt(fmax(0.0, 1.0 - ct * ct));
  double sp, cp;
  sincos_pi(2.0 * phi_frac, sp, cp);
  const double kx = pn * st * cp, ky = pn * st * sp, kz = pn * ct;
  const double Ea = sqrt(ma * ma + pn * pn), Eb = sqrt(mb * mb + pn * pn);
  const double bx = px / E, by = py / E, bz = pz / E, gam = E / M;
  const double k1 = bx * kx + by * ky + bz * kz;
  const double ca = gam * (gam * k1 / (1.0 + gam) + Ea);
  const double cb = gam * (-gam * k1 / (1.0 + gam) + Eb);
  a[0] = kx + ca * bx;  a[1] = ky + ca * by;  a[2] = kz + ca * bz;  a[3] = gam * (Ea + k1);
  bb[0] = -kx + cb * bx; bb[1] = -ky + cb * by; bb[2] = -kz + cb * bz; bb[3] = gam * (Eb - k1);
}

// The four daughters of the two central particles, decay angles from u[dec0..dec0 + 3].
GRN_HD_COLD void cascade_daughters(const grn_process_params &P, int dec0, double p3x, double p3y,
                                   double p3z, double E3, double m3, double p4x, double p4y,
                                   double p4z, double E4, double m4, const double *u,
                                   double d[4][4]) {
  const double *v = u + dec0;
  decay2(p3x, p3y, p3z, E3, m3, P.m_daughter[0], P.m_daughter[1], 2.0 * v[0] - 1.0, v[1], d[0],
         d[1]);
  decay2(p4x, p4y, p4z, E4, m4, P.m_daughter[2], P.m_daughter[3], 2.0 * v[2] - 1.0, v[3], d[2],
         d[3]);
}

// Particle cuts of one final-state particle (px, py, pz, E) (FIDCUT PARTICLE block).
GRN_HD bool particle_cuts(const grn_process_params &P, const double *p) {
  const grn_fidcuts &f = P.fcuts;
  const double ptsq = p[0] * p[0] + p[1] * p[1];
  const double pt   = sqrt(ptsq);
  const double mt   = sqrt(fmax(0.0, p[3] * p[3] - p[2] * p[2]));
  const double pa   = sqrt(ptsq + p[2] * p[2]);
  const double eta  = 0.5 * log((pa + p[2]) / (pa - p[2]));
  const double y    = 0.5 * log((p[3] + p[2]) / (p[3] - p[2]));
  return pt >= f.pt_min && pt <= f.pt_max && mt >= f.Et_min && mt <= f.Et_max &&
         eta >= f.eta_min && eta <= f.eta_max && y >= f.rap_min && y <= f.rap_max;
}

// All four cascade daughters pass the particle cuts.
// Veto cuts (MProcess::FindVetoCuts, src/MProcess.cc:1157-1175): true when a final-state
// particle (px, py, pz) lies in one of the veto domains.
GRN_HD bool veto_hit(const grn_process_params &P, double px, double py, double pz) {
  const double pt = sqrt(px * px + py * py), eta = asinh(pz / pt);
  bool hit = false;
  for (int k = 0; k < P.n_veto; ++k)
    hit |= pt >= P.veto_pt_min[k] && pt <= P.veto_pt_max[k] && eta >= P.veto_eta_min[k] &&
           eta <= P.veto_eta_max[k];
  return hit;
}

// bit 0: the four daughters pass the particle cuts; bit 1: one of them hits a veto domain.
GRN_HD_COLD int cascade_cuts(const grn_process_params &P, int dec0, double p3x, double p3y,
                             double p3z, double E3, double m3, double p4x, double p4y, double p4z,
                             double E4, double m4, const double *u) {
  double d[4][4];
  cascade_daughters(P, dec0, p3x, p3y, p3z, E3, m3, p4x, p4y, p4z, E4, m4, u, d);
  int ok = 1, veto = 0;
  for (int k = 0; k < 4; ++k) {
    ok &= particle_cuts(P, d[k]) ? 1 : 0;
    if (P.veto_active) veto |= veto_hit(P, d[k][0], d[k][1], d[k][2]) ? 2 : 0;
  }
  return ok | veto;
}

// B51RandomKin + B51BuildKin for a 2-body central system, the isotropic decay
// angles lifted into u[6] (cos theta = 2 u6 - 1) and u[7] (phi = 2 pi u7), the
// draws TwoBodyPhaseSpace makes (src/MFactorized.cc:245-412;
// include/Graniitti/MKinematics.h:405-459).
// CASC: the instantiation serves two-body cascades (14-dimensional points); the 8-dimensional
// one leaves the cascade code out.
template <bool CASC>
GRN_HD bool born_kinematics_F(const grn_process_params &P, const Consts &K, const double *u,
                              Born &b) {
  const grn_gencuts &g = P.gcuts;
  const double pt1 = exp(K.lnpt_lo + (K.lnpt_hi - K.lnpt_lo) * u[0]);
  const double pt2 = exp(K.lnpt_lo + (K.lnpt_hi - K.lnpt_lo) * u[1]);
  double s1, c1, s2, c2;
  sincos_pi(2.0 * u[2], s1, c1);
  sincos_pi(2.0 * u[3], s2, c2);
  const double yX  = g.Y_min + (g.Y_max - g.Y_min) * u[4];
  double m3 = K.m3, m4 = K.m4, M2lo = K.M2min, M2hi = K.M2max;
  if (CASC && P.n_decay == 2) {
    // off-shell central masses and the mass window they leave (B51RandomKin)
    cascade_masses(P, K, u, m3, m4);
    const double Mmin = fmax(m3 + m4 + 1e-4, g.M_min);
    if (!(Mmin * Mmin < M2hi)) return false;
    M2lo = Mmin * Mmin;
  }
  b.m3sq = m3 * m3;
  b.m4sq = m4 * m4;
  b.leafok = 1;
  const double m2X = M2lo + (M2hi - M2lo) * u[5];
  b.p1x = pt1 * c1;
  b.p1y = pt1 * s1;
  b.p2x = pt2 * c2;
  b.p2y = pt2 * s2;
  b.pt1sq = b.p1x * b.p1x + b.p1y * b.p1y;
  b.pt2sq = b.p2x * b.p2x + b.p2y * b.p2y;
  const double Xx = -(b.p1x + b.p2x), Xy = -(b.p1y + b.p2y);
  const double mTX = sqrt(m2X + Xx * Xx + Xy * Xy);
  const double eY  = exp(yX);
  const double XP = mTX * eY, XM = mTX / eY;
  const double EX = 0.5 * (XP + XM), ZX = 0.5 * (XP - XM);
  // forward masses: u[6] (and u[7] for double excitation; the side draw u[7] for single)
  forward_masses(P, K, u[6], u[7], u[7], b);
  if (EX > K.sqrt_s - (sqrt(b.mf1sq) + sqrt(b.mf2sq))) return false;  // MFactorized.cc:321
  // isotropic decay in the central-system rest frame, boosted to the lab
  const double MX = sqrt(m2X);
  const double ms = m3 + m4, md = m3 - m4;
  const double ps = sqrt(fmax(0.0, (MX - ms) * (MX + ms) * (MX + md) * (MX - md))) / (2.0 * MX);
  // decay angles: the draws after the forward masses (u[6], u[7]; u[8], u[9] when excited)
  const int    da = (CASC && P.excitation) ? 8 : 6;
  const double ct = 2.0 * u[da] - 1.0;
  const double st = sqrt(fmax(0.0, 1.0 - ct * ct));
  double sp, cp;
  sincos_pi(2.0 * u[da + 1], sp, cp);
  const double kx = ps * st * cp, ky = ps * st * sp, kz = ps * ct;
  const double E3s = sqrt(b.m3sq + ps * ps), E4s = sqrt(b.m4sq + ps * ps);
  const double bx = Xx / EX, by = Xy / EX, bz = ZX / EX, gam = EX / MX;
  const double k1 = bx * kx + by * ky + bz * kz;
  const double a3 = gam * (gam * k1 / (1.0 + gam) + E3s);
  const double a4 = gam * (-gam * k1 / (1.0 + gam) + E4s);
  b.p3x = kx + a3 * bx;
  b.p3y = ky + a3 * by;
  const double p3z = kz + a3 * bz, E3 = gam * (E3s + k1);
  b.p4x = -kx + a4 * bx;
  b.p4y = -ky + a4 * by;
  const double p4z = -kz + a4 * bz, E4 = gam * (E4s - k1);
  b.mt3 = sqrt(b.m3sq + b.p3x * b.p3x + b.p3y * b.p3y);
  b.mt4 = sqrt(b.m4sq + b.p4x * b.p4x + b.p4y * b.p4y);
  // light-cone components; the smaller one from mT^2 / larger (exact, no cancellation)
  if (p3z >= 0) { b.p3p = E3 + p3z; b.p3m = b.mt3 * b.mt3 / b.p3p; }
  else          { b.p3m = E3 - p3z; b.p3p = b.mt3 * b.mt3 / b.p3m; }
  if (p4z >= 0) { b.p4p = E4 + p4z; b.p4m = b.mt4 * b.mt4 / b.p4p; }
  else          { b.p4m = E4 - p4z; b.p4p = b.mt4 * b.mt4 / b.p4m; }
  b.y3 = 0.5 * log(b.p3p / b.p3m);
  b.y4 = 0.5 * log(b.p4p / b.p4m);
  b.jx = ps / MX * (M2hi - M2lo);
  if (CASC && P.n_decay == 2) {
    // isotropic decays of the two central particles (ConstructDecayKinematics); the particle
    // cuts act on the four daughters (FindDecayCuts, src/MProcess.cc:1140-1154)
    b.leafok =
        cascade_cuts(P, K.dec0, b.p3x, b.p3y, p3z, E3, m3, b.p4x, b.p4y, p4z, E4, m4, u);
  }
  return born_invariants(K, b);
}

template <bool CASC = false>
GRN_HD bool born_kinematics(const grn_process_params &P, const Consts &K, const double *u,
                            Born &b) {
  if (P.phase_space == GRN_PS_FACTORIZED) return born_kinematics_F<CASC>(P, K, u, b);
  return born_kinematics_C<CASC>(P, K, u, b);
}

// Fiducial cuts (MProcess::CommonCuts + FindDecayCuts, src/MProcess.cc:1085-1154).
GRN_HD bool fiducial_cuts(const grn_process_params &P, const Consts &K, const Born &b) {
  const grn_fidcuts &f = P.fcuts;
  if (!f.active) return true;
  const double at1 = fabs(b.t1), at2 = fabs(b.t2);
  if (!(at1 >= f.ft_min && at1 <= f.ft_max && at2 >= f.ft_min && at2 <= f.ft_max)) return false;
  // excited forward systems: their mass window (CommonCuts, src/MProcess.cc:1105-1119)
  if (b.exc) {
    const double mf1 = sqrt(b.mf1sq), mf2 = sqrt(b.mf2sq);
    if ((b.exc & 1) && !(mf1 >= f.fM_min && mf1 <= f.fM_max)) return false;
    if ((b.exc & 2) && !(mf2 >= f.fM_min && mf2 <= f.fM_max)) return false;
  }
  // M = sqrt(m2), Y = log(P+ / P-) / 2, Pt and each particle's eta = asinh(pz / pT) are
  // compared through monotone images of the windows (Consts::cut_*), without transcendentals
  const double m2 = fmax(b.m2, 0.0);
  const double Pp = b.p3p + b.p4p, Pm = b.p3m + b.p4m;
  const double sx = b.p3x + b.p4x, sy = b.p3y + b.p4y;
  const double pt2 = sx * sx + sy * sy;
  if (!(m2 >= K.cut_m2lo && m2 <= K.cut_m2hi && Pp >= Pm * K.cut_e2ylo &&
        Pp <= Pm * K.cut_e2yhi && pt2 >= K.cut_pt2lo && pt2 <= K.cut_pt2hi))
    return false;
  if (P.n_decay == 2) return (b.leafok & 1) != 0;
  bool ok = true;
  const double px[2] = {b.p3x, b.p4x}, py[2] = {b.p3y, b.p4y};
  const double mt[2] = {b.mt3, b.mt4}, y[2] = {b.y3, b.y4};
  const double pz[2] = {0.5 * (b.p3p - b.p3m), 0.5 * (b.p4p - b.p4m)};
#pragma unroll
  for (int k = 0; k < 2; ++k) {
    const double pt = sqrt(px[k] * px[k] + py[k] * py[k]);
    if (!(pt >= f.pt_min && pt <= f.pt_max && mt[k] >= f.Et_min && mt[k] <= f.Et_max &&
          pz[k] >= pt * K.cut_sheta_lo && pz[k] <= pt * K.cut_sheta_hi &&
          y[k] >= f.rap_min && y[k] <= f.rap_max))
      ok = false;
  }
  return ok;
}

// Veto cuts on the final-state leaves (MProcess::VetoCuts, src/MProcess.cc:1069-1082): true
// when the event is not vetoed.
GRN_HD bool veto_cuts(const grn_process_params &P, const Born &b) {
  if (!P.veto_active) return true;
  if (P.n_decay == 2) return (b.leafok & 2) == 0;
  return !veto_hit(P, b.p3x, b.p3y, 0.5 * (b.p3p - b.p3m)) &&
         !veto_hit(P, b.p4x, b.p4y, 0.5 * (b.p4p - b.p4m));
}

// Regge continuum amplitude of a 2-body central state, sign +1
// (MRegge::ME4, src/MRegge.cc:394-438; PomPomProtonVertex 637-644), from the
// invariants. Used for the FP64 Born amplitude and, with T = float, per loop point.
template <typename T>
GRN_HD cx<T> regge_me4(const grn_process_params &P, const Consts &K, T t1, T t2, T lns13, T lns14,
                       T lns23, T lns24, T that, T uhat, int exc = 0, T mf1sq = T(0),
                       T mf2sq = T(0), T lnsc = T(0)) {
  const grn_regge_params &rp = P.regge;
  const T M2  = T(K.M2prop);
  const T ffa = meson_ff<T>(rp, that, M2);
  const T ffb = meson_ff<T>(rp, uhat, M2);
  const T Xt  = ffa * ffa / (that - M2);
  const T Xu  = ffb * ffb / (uhat - M2);
  const T vtx = exc ? leg_vertex<T>(P, K, exc, 0, t1, mf1sq) *
                          leg_vertex<T>(P, K, exc, 1, t2, mf2sq) * T(K.g2)
                    : T(K.gN2) * proton_ff<T>(T(P.soft.fc1), T(P.soft.fc2), t1) *
                          proton_ff<T>(T(P.soft.fc1), T(P.soft.fc2), t2) * T(K.g2);
  if (K.n_active == 1) {
    // One trajectory: both channels share the phase exp(-i pi ap (t1+t2)/2).
    const int k  = K.active[0] ? 0 : (K.active[1] ? 1 : 2);
    const T   a1 = T(rp.a0[k]) + T(rp.ap[k]) * t1;
    const T   a2 = T(rp.a0[k]) + T(rp.ap[k]) * t2;
    const T   l0 = T(K.lns0);
    const T   mt = exp(a1 * (lns13 - l0) + a2 * (lns24 - l0) - lnsc) * Xt +
                 exp(a1 * (lns14 - l0) + a2 * (lns23 - l0) - lnsc) * Xu;
    T sn, cs;
    sincos_pi(-T(0.5) * T(rp.ap[k]) * (t1 + t2), sn, cs);
    const cx<T> e0{T(K.eta0_re[k]), T(K.eta0_im[k])};
    const cx<T> e2 = cmul(e0, e0);
    return cscale(cmul(e2, cx<T>{cs, sn}), vtx * mt);
  }
  const T     ho = T(0.5) * lnsc;
  const cx<T> At = cscale(cmul(regge_prop<T>(K, rp, lns13, t1, ho),
                               regge_prop<T>(K, rp, lns24, t2, ho)),
                          Xt);
  const cx<T> Au = cscale(cmul(regge_prop<T>(K, rp, lns14, t1, ho),
                               regge_prop<T>(K, rp, lns23, t2, ho)),
                          Xu);
  return cscale(cadd(At, Au), vtx);
}

// ---------------------------------------------------------------------------
// Regge resonances (PP[RES], PP[RES+CON]; MRegge::ME3, src/MRegge.cc:677-712, with
// spin::ProdAmp / DecayAmp, src/MSpin.cc:280-480, and the Breit-Wigner forms of
// src/MForm.cc:743-830). Per resonance r
//   A_r = 2 P(s1,t1) P(s2,t2) gN^2 F(t1) F(t2) CBW_r(m^2) exp(-(m^2 - M_r^2)^2 / S0^4)
//         (1/m^2)^omega g_r g_decay,r S^prod_r S^dec_r
// with P(s,t) the Regge propagator sum and F the proton form factor as in the continuum,
// s_i = (p_i + X)^2. For J = 2 the spin factors (SPINGEN / SPINDEC) are
//   S = sqrt(5) sqrt(Re f rho_rot f^+),  f_M = d^2_{0M}(theta) e^{i M phi},  M = -2..2,
// with (theta, phi) the direction of the momentum transfer q1 (production) or of the first
// daughter (decay) in the X rest frame reached by a pure boost, and rho_rot = D^+ rho D the
// resonance's density matrix rotated by D_{MM'} = d^2_{MM'}(theta_R) e^{i M' phi_R} to the
// chosen frame (CM: none; HX: X's lab direction; CS: the beams' bisector in the X frame).
// J = 0: S = 1 (and the decay T-matrix element of two pseudoscalars is 1).

// Wigner small-d d^2_{m m'}(theta) from c = cos(theta/2), s = sin(theta/2) (sum over k of the
// standard closed formula, in the sign convention of MSpin.cc:927-961).
GRN_HD double wigner_d2(int m, int mp, double c, double s) {
  const double f[5] = {1.0, 1.0, 2.0, 6.0, 24.0};
  double sum = 0.0;
  for (int k = 0; k <= 4; ++k) {
    if (2 - mp - k < 0 || 2 + m - k < 0 || k + mp - m < 0) continue;
    double v = (((mp - m + k) & 1) ? -1.0 : 1.0) / (f[2 - mp - k] * f[2 + m - k] * f[k + mp - m] * f[k]);
    for (int e = 0; e < 4 + m - mp - 2 * k; ++e) v *= c;
    for (int e = 0; e < mp - m + 2 * k; ++e) v *= s;
    sum += v;
  }
  return sqrt(f[2 + m] * f[2 - m] * f[2 + mp] * f[2 - mp]) * sum;
}

// Direction of (x, y, z): cos(theta), sin(theta), e^{i phi} (phi = 0 on the z axis).
template <typename T>
GRN_HD void direction(T x, T y, T z, T &ct, T &st, T &cp, T &sp) {
  const T rt = sqrt(x * x + y * y), r = sqrt(rt * rt + z * z);
  ct = r > T(0) ? z / r : T(1);
  st = r > T(0) ? rt / r : T(0);
  cp = rt > T(0) ? x / rt : T(1);
  sp = rt > T(0) ? y / rt : T(0);
}

// Re(f rho f^+) for f_M = d^2_{0M}(theta) e^{i M phi}; rho Hermitian packed as its 5 diagonal
// entries, then the real and the imaginary parts of the 10 entries above it (row-major).
template <typename T>
GRN_HD T spin2_form(const T *rho, T ct, T st, T cp, T sp) {
  const T a = T(0.6123724356957945) * st * st;  // sqrt(3/8) sin^2
  const T b = T(1.224744871391589) * st * ct;   // sqrt(3/2) sin cos
  const T d[5] = {a, b, T(1.5) * ct * ct - T(0.5), -b, a};  // d^2_{0M}, M = -2..2
  // e^{i k phi}, k = 1..4 (the phase of entry (j, l) is e^{i (M_j - M_l) phi})
  T c[5], sn[5];
  c[0] = T(1); sn[0] = T(0);
  for (int k = 1; k < 5; ++k) {
    c[k]  = c[k - 1] * cp - sn[k - 1] * sp;
    sn[k] = sn[k - 1] * cp + c[k - 1] * sp;
  }
  T q = T(0);
  for (int j = 0; j < 5; ++j) q += d[j] * d[j] * rho[j];
  int u = 0;
  for (int j = 0; j < 5; ++j)
    for (int l = j + 1; l < 5; ++l, ++u) {
      // 2 Re(rho_jl e^{i (M_j - M_l) phi}), M_j - M_l = j - l < 0
      const int k = l - j;
      q += T(2) * d[j] * d[l] * (rho[5 + u] * c[k] + rho[15 + u] * sn[k]);
    }
  return q;
}

// Per-event data of the Regge resonances: the loop-invariant factor of each resonance, the
// rotated density matrices (packed as in spin2_form) of the J = 2 resonances (SPINGEN), and
// X for the boost of q1 into its rest frame.
template <typename T>
struct RegRes {
  cx<T> C[GRN_MAX_RESONANCES];
  T     rho[GRN_MAX_RESONANCES][25];
  T     Xe, Xx, Xy, Xz, M;
};

// q = (E, x, y, z) into the rest frame of X (MKinematics.h:384-401 with sign -1): spatial part.
template <typename T>
GRN_HD void boost_to_rest(T Xe, T Xx, T Xy, T Xz, T M, T E, T &x, T &y, T &z) {
  const T k = (Xx * x + Xy * y + Xz * z) / (M * (Xe + M)) - E / M;
  x += k * Xx;
  y += k * Xy;
  z += k * Xz;
}

GRN_HD_COLD void regge_res_event(const grn_process_params &P, const Consts &K, double p3p,
                                 double p3m, double p3x, double p3y, double p4p, double p4m,
                                 double p4x, double p4y, RegRes<double> &R) {
  const double Xp = p3p + p4p, Xm = p3m + p4m;
  R.Xe = 0.5 * (Xp + Xm);
  R.Xz = 0.5 * (Xp - Xm);
  R.Xx = p3x + p4x;
  R.Xy = p3y + p4y;
  const double m2 = Xp * Xm - (R.Xx * R.Xx + R.Xy * R.Xy);
  R.M = sqrt(m2);
  // frame rotation (theta_R, phi_R) as half-angle cos / sin and e^{i phi_R}
  double ct = 1.0, st = 0.0, cp = 1.0, sp = 0.0;
  if (P.spin_frame == GRN_FRAME_HX) {
    direction<double>(R.Xx, R.Xy, R.Xz, ct, st, cp, sp);
  } else if (P.spin_frame == GRN_FRAME_CS) {
    const double E = 0.5 * K.sqrt_s, pz = 0.5 * (K.L - K.eps);
    double ax = 0, ay = 0, az = pz, bx = 0, by = 0, bz = -pz;
    boost_to_rest(R.Xe, R.Xx, R.Xy, R.Xz, R.M, E, ax, ay, az);
    boost_to_rest(R.Xe, R.Xx, R.Xy, R.Xz, R.M, E, bx, by, bz);
    const double na = sqrt(ax * ax + ay * ay + az * az), nb = sqrt(bx * bx + by * by + bz * bz);
    direction<double>(ax / na - bx / nb, ay / na - by / nb, az / na - bz / nb, ct, st, cp, sp);
  }
  // half-angle cosine and sine; the smaller one from sin theta_R = 2 hc hs (the form
  // sqrt((1 - cos) / 2) would keep few digits for theta_R -> 0, the frame of a central
  // system with vanishing transverse momentum)
  double hc, hs;
  if (ct >= 0.0) {
    hc = sqrt(0.5 * (1.0 + ct));
    hs = 0.5 * st / hc;
  } else {
    hs = sqrt(0.5 * (1.0 - ct));
    hc = 0.5 * st / hs;
  }
  // D_{ij} = d^2_{M_i M_j}(theta_R) e^{i M_j phi_R}
  double Dr[5][5], Di[5][5];
  for (int j = 0; j < 5; ++j) {
    // e^{i M_j phi_R}, M_j = j - 2
    double er = 1.0, ei = 0.0;
    const int mj = j - 2;
    for (int k = 0; k < (mj < 0 ? -mj : mj); ++k) {
      const double t = er * cp - ei * sp * (mj < 0 ? -1.0 : 1.0);
      ei = ei * cp + er * sp * (mj < 0 ? -1.0 : 1.0);
      er = t;
    }
    for (int i = 0; i < 5; ++i) {
      const double d = wigner_d2(i - 2, mj, hc, hs);
      Dr[i][j] = d * er;
      Di[i][j] = d * ei;
    }
  }
  // daughter direction in the X rest frame
  double dx = p3x, dy = p3y, dz = 0.5 * (p3p - p3m);
  boost_to_rest(R.Xe, R.Xx, R.Xy, R.Xz, R.M, 0.5 * (p3p + p3m), dx, dy, dz);
  double dct, dst, dcp, dsp;
  direction<double>(dx, dy, dz, dct, dst, dcp, dsp);
  const double lm2 = log(m2);
  for (int r = 0; r < K.rr_n; ++r) {
    const double M0 = K.rr_M[r], W = K.rr_W[r], M02 = M0 * M0, dm = m2 - M02;
    // complex Breit-Wigner -1/den (times a numerator for form 4)
    double dre = dm, dim = M0 * W, num = 1.0;
    if (K.rr_bw[r] == 2) {
      dim = sqrt(m2) * W;
    } else if (K.rr_bw[r] == 3) {
      const double ma = sqrt(K.m3sq), mb = sqrt(K.m4sq);
      const double u = sqrt(fmax(0.0, (m2 - (ma + mb) * (ma + mb)) * (m2 - (ma - mb) * (ma - mb)))) /
                       (2.0 * sqrt(m2));
      const double v = sqrt(fmax(0.0, (M02 - (ma + mb) * (ma + mb)) * (M02 - (ma - mb) * (ma - mb)))) /
                       (2.0 * M0);
      dim = W * M02 / sqrt(m2) * pow(u / v, 2.0 * K.rr_J[r] + 1.0);
    } else if (K.rr_bw[r] == 4 && K.rr_J[r] == 2) {
      const double x = m2 / M02;
      num = 7.0 / 6.0 - (4.0 / 3.0) * x + (2.0 / 3.0) * x * x;
    }
    const double id = -num / (dre * dre + dim * dim);
    const cx<double> bw{dre * id, -dim * id};
    // form factor, flux, 2, and g_regge g_decay
    double f = 2.0 * exp(-dm * dm * K.rr_iff4[r] - P.omega * lm2);
    if (K.rr_J[r] == 2) {
      // rho_rot = D^+ rho D, packed
      const double *rr = P.res[r].rho[0], *ri = P.res[r].rho[1];
      double Rr[5][5], Ri[5][5];
      for (int i = 0; i < 5; ++i)
        for (int k = 0; k < 5; ++k) {
          double sr = 0.0, si = 0.0;
          for (int j = 0; j < 5; ++j)
            for (int l = 0; l < 5; ++l) {
              // conj(D_ji) rho_jl D_lk
              const double ar = Dr[j][i], ai = -Di[j][i];
              const double br = rr[5 * j + l], bi = ri[5 * j + l];
              const double cr = ar * br - ai * bi, ci = ar * bi + ai * br;
              sr += cr * Dr[l][k] - ci * Di[l][k];
              si += cr * Di[l][k] + ci * Dr[l][k];
            }
          Rr[i][k] = sr;
          Ri[i][k] = si;
        }
      double pk[25];
      int    u = 0;
      for (int j = 0; j < 5; ++j) pk[j] = Rr[j][j];
      for (int j = 0; j < 5; ++j)
        for (int l = j + 1; l < 5; ++l, ++u) {
          pk[5 + u]  = Rr[j][l];
          pk[15 + u] = Ri[j][l];
        }
      for (int k = 0; k < 25; ++k) R.rho[r][k] = pk[k];
      if (P.spin_dec) f *= sqrt(5.0) * sqrt(fmax(0.0, spin2_form<double>(pk, dct, dst, dcp, dsp)));
    } else {
      for (int k = 0; k < 25; ++k) R.rho[r][k] = 0.0;
    }
    R.C[r] = cscale(cmul(bw, cx<double>{K.rr_g_re[r], K.rr_g_im[r]}), f);
  }
}

// Resonance amplitude at a point: q1 = (qE, qx, qy, qz), s1, s2, t1, t2.
template <typename T>
GRN_HD cx<T> regge_res_amp(const grn_process_params &P, const Consts &K, const RegRes<T> &R, T t1,
                           T t2, T lns1, T lns2, T qE, T qx, T qy, T qz) {
  cx<T> sum{T(0), T(0)};
  T     ct = T(1), st = T(0), cp = T(1), sp = T(0);
  bool  dir = false;
  for (int r = 0; r < K.rr_n; ++r) {
    T s = T(1);
    if (K.rr_J[r] == 2 && P.spin_gen) {
      if (!dir) {
        boost_to_rest<T>(R.Xe, R.Xx, R.Xy, R.Xz, R.M, qE, qx, qy, qz);
        direction<T>(qx, qy, qz, ct, st, cp, sp);
        dir = true;
      }
      s = T(2.23606797749979) * sqrt(fmax(T(0), spin2_form<T>(R.rho[r], ct, st, cp, sp)));
    }
    sum = cadd(sum, cscale(R.C[r], s));
  }
  const grn_regge_params &rp = P.regge;
  const T vtx = T(K.gN2) * proton_ff<T>(T(P.soft.fc1), T(P.soft.fc2), t1) *
                proton_ff<T>(T(P.soft.fc1), T(P.soft.fc2), t2);
  return cscale(cmul(sum, cmul(regge_prop<T>(K, rp, lns1, t1), regge_prop<T>(K, rp, lns2, t2))),
                vtx);
}

// Bare amplitude at one kt-loop point: forward legs p1T - k, p2T + k with the
// tree-level central pair (for Kf = 2 the pair is unchanged because p1T + p2T is
// loop invariant; MContinuum::LoopKinematics, src/MContinuum.cc:94-161).
// Returns false when the point is kinematically invalid (the reference skips it).
template <typename T>
struct LoopEvent {
  T p1x, p1y, p2x, p2y;     // tree-level forward transverse momenta
  T p3x, p3y, p4x, p4y;
  T p3p, p3m, p4p, p4m;
  T a1, a2;                 // (P+ - eps)/L, (P- - eps)/L
  T ia1, ia2;               // 1/(1 - a1), 1/(1 - a2)
  T invL, invL2, L, eps, mp2, m3sq, m4sq;
  T mf1, mf2;               // forward legs' masses^2 (mp2 unless excited)
  int exc;                  // excited forward legs (bit 0: leg 1, bit 1: leg 2)
  // event scale of the FP32 loop: lnsc is subtracted from the Regge exponents (FP32 exp
  // covers only |x| < 87), the resonance sums are stored divided by escale, and the loop sum
  // is multiplied by escale in FP64 (1 and 0 for events inside the FP32 range)
  T      lnsc;
  double escale;
  ResSums<T> res;           // PP[RESTENSOR]: resonance sums of the tree-level central mass
};

// Kinematics of one kt-loop point; false when it is kinematically invalid.
// The light-cone closure x1 = a1 + c2 / (1 - x2), x2 = a2 + c1 / (1 - x1) (solve_x) in two
// steps: the first from the event's 1/(1 - a_i), the second from r_i = 1/(1 - x_i) of the
// first, which then serve as 1/(1 - x_i) of the point (c_i = mT_i^2 / L^2 ~ 1e-8: the second
// step moves x_i by O(c^2) ~ 1e-16 relative, r_i by as little); two reciprocals per point.
template <typename T>
GRN_HD bool loop_point_kin(const LoopEvent<T> &e, T kx, T ky, LCKin<T> &kk) {
  const T q1x = e.p1x - kx, q1y = e.p1y - ky;
  const T q2x = e.p2x + kx, q2y = e.p2y + ky;
  const T pt1sq = q1x * q1x + q1y * q1y;
  const T pt2sq = q2x * q2x + q2y * q2y;
  const T mT1sq = e.mf1 + pt1sq, mT2sq = e.mf2 + pt2sq;
  const T c1 = mT1sq * e.invL2, c2 = mT2sq * e.invL2;
  T r1 = T(1) / (T(1) - (e.a1 + c2 * e.ia2));
  T r2 = T(1) / (T(1) - (e.a2 + c1 * e.ia1));
  T x1 = e.a1 + c2 * r2, x2 = e.a2 + c1 * r1;
  if (e.exc) {  // excited legs: c up to M^2 / s, the closed-form closure (solve_x)
    if (!solve_x<T>(e.a1, e.a2, c1, c2, x1, x2)) return false;
    r1 = T(1) / (T(1) - x1);
    r2 = T(1) / (T(1) - x2);
  }
  if (!((x1 > T(0)) && (x2 > T(0)) && (x1 < T(1)) && (x2 < T(1)))) return false;
  const T p1p = (T(1) - x1) * e.L;
  const T p1m = mT1sq * r1 * e.invL;
  const T p2m = (T(1) - x2) * e.L;
  const T p2p = mT2sq * r2 * e.invL;
  kk.p1p = p1p; kk.p1m = p1m; kk.p1x = q1x; kk.p1y = q1y;
  kk.p2p = p2p; kk.p2m = p2m; kk.p2x = q2x; kk.p2y = q2y;
  kk.p3p = e.p3p; kk.p3m = e.p3m; kk.p3x = e.p3x; kk.p3y = e.p3y;
  kk.p4p = e.p4p; kk.p4m = e.p4m; kk.p4x = e.p4x; kk.p4y = e.p4y;
  kk.L = e.L; kk.eps = e.eps; kk.mp2 = e.mp2;
  kk.t1  = -(pt1sq + x1 * (e.mf1 - e.mp2) + x1 * x1 * e.mp2) * r1;
  kk.t2  = -(pt2sq + x2 * (e.mf2 - e.mp2) + x2 * x2 * e.mp2) * r2;
  kk.s13 = e.mf1 + e.m3sq + p1p * e.p3m + p1m * e.p3p - T(2) * (q1x * e.p3x + q1y * e.p3y);
  kk.s14 = e.mf1 + e.m4sq + p1p * e.p4m + p1m * e.p4p - T(2) * (q1x * e.p4x + q1y * e.p4y);
  kk.s23 = e.mf2 + e.m3sq + p2p * e.p3m + p2m * e.p3p - T(2) * (q2x * e.p3x + q2y * e.p3y);
  kk.s24 = e.mf2 + e.m4sq + p2p * e.p4m + p2m * e.p4p - T(2) * (q2x * e.p4x + q2y * e.p4y);
  {
    const T dp = e.p4p - e.eps + p2p;
    const T dm = e.eps - p1m - e.p3m;
    const T tx = q1x + e.p3x, ty = q1y + e.p3y;
    kk.that    = dp * dm - (tx * tx + ty * ty);
  }
  {
    const T dp = e.p3p - e.eps + p2p;
    const T dm = e.eps - p1m - e.p4m;
    const T tx = q1x + e.p4x, ty = q1y + e.p4y;
    kk.uhat    = dp * dm - (tx * tx + ty * ty);
  }
  // q1 = pa - p1: q1+ = x1 L, q1- = -(pT1^2 + x1 mp^2) / ((1 - x1) L) (q_lightcone)
  kk.q1p = x1 * e.L;
  kk.q1m = -(pt1sq + (e.mf1 - e.mp2) + x1 * e.mp2) * r1 * e.invL;
  kk.q2m = x2 * e.L;
  kk.q2p = -(pt2sq + (e.mf2 - e.mp2) + x2 * e.mp2) * r2 * e.invL;
  return true;
}

template <typename T>
GRN_HD bool loop_point_amp(const grn_process_params &P, const Consts &K, const LoopEvent<T> &e,
                           T kx, T ky, cx<T> &A) {
  LCKin<T> kk;
  if (!loop_point_kin<T>(e, kx, ky, kk)) return false;
  if (P.process == GRN_PROC_TENSOR_CON) {
    A = tensor_me4_2xs<T>(P, K, kk);
  } else if (P.process == GRN_PROC_TENSOR_RES) {
    A = tensor_me3<T>(P, K, kk, e.res);
  } else if (P.process == GRN_PROC_TENSOR_RESCON) {
    A = tensor_me4_2xs<T>(P, K, kk);
    if (K.n_res > 0) A = cadd(A, tensor_me3<T>(P, K, kk, e.res));
  } else {
    A = regge_me4<T>(P, K, kk.t1, kk.t2, log(kk.s13), log(kk.s14), log(kk.s23), log(kk.s24),
                     kk.that, kk.uhat, e.exc, e.mf1, e.mf2, e.lnsc);
  }
  return true;
}

// ---------------------------------------------------------------------------
// Fast FP32 kt-loop point: increments over the tree-level point.
//
// Every loop-point quantity is written as its tree-level value (FP64 per event)
// plus an increment that is an explicit polynomial in the loop momentum k:
//   pT1'^2 - pT1^2 = -2 p1T.k + k^2,   pT2'^2 - pT2^2 = 2 p2T.k + k^2,
//   x1 = a1 + c2 ia2, x2 = a2 + c1 ia1, 1/(1 - x1) = ia1 (1 + c2 ia2 ia1)
// with a_i = (P+- - eps)/L, ia_i = 1/(1 - a_i), c_i = mT_i^2/L^2 ~ 1e-8 (the
// fixed point of solve_x closes after one step; truncation ~ (c ia)^2 ~ 1e-16),
// and s13' = s13 + ds13, ..., so that ln s13' = ln s13 + ln(1 + ds13/s13). The
// Regge exponent is then the Born exponent (kept in FP64, applied after the loop
// sum) plus an O(1) increment, and every FP32 operand is an O(1) quantity: the
// MUFU fast log2/exp2 paths keep ~1e-7 absolute accuracy on the exponent. The
// off-shell form factors and proton form factors share the point's one division.

GRN_HD float fast_log(float x) {
#ifdef __CUDA_ARCH__
  return __logf(x);
#else
  return std::log(x);
#endif
}
GRN_HD float fast_exp(float x) {
#ifdef __CUDA_ARCH__
  return __expf(x);
#else
  return std::exp(x);
#endif
}
// Base-2 forms (one MUFU instruction each on the device): the fast loop keeps its
// logarithms and exponents in log2 units, so no ln 2 scalings are executed.
GRN_HD float fast_log2(float x) {
#ifdef __CUDA_ARCH__
  float y;
  asm("lg2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));  // the SFU's log2 (normal x)
  return y;
#else
  return std::log2(x);
#endif
}
GRN_HD float fast_exp2(float x) {
#ifdef __CUDA_ARCH__
  float y;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));  // the SFU's 2^x (~2 ulp)
  return y;
#else
  return std::exp2(x);
#endif
}
// a / b through the reciprocal unit (about 2 ulp); b in the normal range.
GRN_HD float fast_div(float a, float b) {
#ifdef __CUDA_ARCH__
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(b));  // the SFU's 1/b (normal b)
  return a * r;
#else
  return a / b;
#endif
}
// The SFU's sine and cosine of an argument in [-pi, pi] (absolute error ~5e-7).
GRN_HD void sfu_sincos(float a, float &s, float &c) {
#ifdef __CUDA_ARCH__
  asm("sin.approx.ftz.f32 %0, %1;" : "=f"(s) : "f"(a));
  asm("cos.approx.ftz.f32 %0, %1;" : "=f"(c) : "f"(a));
#else
  s = std::sin(a);
  c = std::cos(a);
#endif
}
// sin(pi x), cos(pi x) for the loop phase: x reduced by its period 2 to [-1, 1], then
// the hardware sine / cosine of pi r (absolute error ~5e-7, |pi r| <= pi).
GRN_HD void fast_sincos_pi(float x, float &s, float &c) {
#ifdef __CUDA_ARCH__
  const float r = fmaf(-2.f, rintf(0.5f * x), x);
  sfu_sincos(float(kPi) * r, s, c);
#else
  s = std::sin(float(kPi) * x);
  c = std::cos(float(kPi) * x);
#endif
}
constexpr double kLog2e = 1.4426950408889634074;

// Per-event fields of the fast loop (stored between the two kernel stages).
#define GRN_LOOP_EVENT_FIELDS(X)                                                              \
  X(p1x) X(p1y) X(p2x) X(p2y) X(p3x) X(p3y) X(p4x) X(p4y) X(p3p) X(p3m) X(p4p) X(p4m) X(ia1) \
  X(ia2) X(q1c) X(q2c) X(x10) X(x20) X(r10) X(r20) X(mT1s0) X(mT2s0) X(T1n0) X(T2n0) X(t10)   \
  X(t20) X(is13) X(is14) X(is23) X(is24) X(L13) X(L14) X(L23) X(L24) X(a10) X(a20) X(dpa0)    \
  X(dma0) X(dpb0) X(dmb0) X(c3x) X(c3y) X(c4x) X(c4y) X(fa0) X(fb0) X(rho_t) X(rho_u)         \
  X(pre_re) X(pre_im)
#define GRN_COUNT_FIELD(f) +1
constexpr int kLoopEventFields = 0 GRN_LOOP_EVENT_FIELDS(GRN_COUNT_FIELD);

template <typename T>
struct LoopEventF {
  // tree-level transverse momenta
  T p1x, p1y, p2x, p2y, p3x, p3y, p4x, p4y;
  T p3p, p3m, p4p, p4m;
  T ia1, ia2, q1c, q2c;      // 1/(1-a), ia1^2 ia2, ia2^2 ia1
  T L, invL, invL2, mp2, M2;
  T x10, x20, r10, r20;      // tree-level x and 1/(1-x) (linear closure)
  T mT1s0, mT2s0, T1n0, T2n0;  // mT^2 and pT^2 + x^2 mp^2 at k = 0
  T t10, t20;
  T is13, is14, is23, is24;  // 1/s at k = 0
  T L13, L14, L23, L24;      // log2(s/s0) at k = 0
  T a10, a20, ap;            // trajectory at t1, t2 (k = 0) and slope
  T dpa0, dma0, dpb0, dmb0;  // light-cone factors of t_hat, u_hat at k = 0
  T c3x, c3y, c4x, c4y;      // p1T + p3T, p1T + p4T
  T ifc1, ifc2;
  T ff_b, ff_a2, ff_ab;
  T fa0, fb0;                // 2 log2 ff(t_hat), 2 log2 ff(u_hat) at k = 0 (exponential kinds)
  T rho_t, rho_u;            // exp(E_t0 - Emax), exp(E_u0 - Emax)
  T pre_re, pre_im;          // couplings x ReggeEta^2 x tree-level phase [x b_POW^2]
  double escale;             // exp(Emax), applied in FP64 after the loop sum
  int ffmode;
};

// Per-engine constants of the fast loop.
template <typename T>
GRN_HD void make_loop_consts_fast(const grn_process_params &P, const Consts &K,
                                  LoopEventF<T> &e) {
  const int k = K.active[0] ? 0 : (K.active[1] ? 1 : 2);
  e.L = T(K.L); e.invL = T(K.invL); e.invL2 = T(K.invL2);
  e.mp2 = T(K.mp2); e.M2 = T(K.M2prop);
  e.ap = T(P.regge.ap[k]);
  e.ifc1 = T(1.0 / P.soft.fc1); e.ifc2 = T(1.0 / P.soft.fc2);
  e.ffmode = P.regge.offshellFF;
  e.ff_a2 = T(P.regge.a_OREAR * P.regge.a_OREAR);
  e.ff_ab = T(P.regge.a_OREAR * P.regge.b_OREAR);
  e.ff_b = T(e.ffmode == 2 ? P.regge.b_POW : (e.ffmode == 0 ? P.regge.b_EXP : P.regge.b_OREAR));
}

// Per-event part of the fast loop from the tree-level event (FP64 here), and the
// tree-level amplitude A0 from the same quantities (A0 = the fast loop point at
// k = 0, evaluated in FP64 and multiplied by exp(Emax)).
template <typename T>
GRN_HD void make_loop_event_fast(const grn_process_params &P, const Consts &K, const Born &b,
                                 LoopEventF<T> &e, double *A0re = nullptr,
                                 double *A0im = nullptr) {
  make_loop_consts_fast<T>(P, K, e);
  e.p1x = T(b.p1x); e.p1y = T(b.p1y); e.p2x = T(b.p2x); e.p2y = T(b.p2y);
  e.p3x = T(b.p3x); e.p3y = T(b.p3y); e.p4x = T(b.p4x); e.p4y = T(b.p4y);
  e.p3p = T(b.p3p); e.p3m = T(b.p3m); e.p4p = T(b.p4p); e.p4m = T(b.p4m);
  const double a1 = (b.p3p + b.p4p - K.eps) * K.invL, a2 = (b.p3m + b.p4m - K.eps) * K.invL;
  const double ia1 = 1.0 / (1.0 - a1), ia2 = 1.0 / (1.0 - a2);
  e.ia1 = T(ia1); e.ia2 = T(ia2); e.q1c = T(ia1 * ia1 * ia2); e.q2c = T(ia2 * ia2 * ia1);
  const double L = K.L, invL = K.invL, invL2 = K.invL2, mp2 = K.mp2;
  // k = 0 values of the linear closure (same formulas as the loop point, in FP64)
  const double mT1s = mp2 + b.pt1sq, mT2s = mp2 + b.pt2sq;
  const double c1 = mT1s * invL2, c2 = mT2s * invL2;
  const double x1 = a1 + c2 * ia2, x2 = a2 + c1 * ia1;
  const double r1 = ia1 + ia1 * ia1 * ia2 * c2, r2 = ia2 + ia2 * ia2 * ia1 * c1;
  const double p1p = (1.0 - x1) * L, p1m = mT1s * invL * r1;
  const double p2m = (1.0 - x2) * L, p2p = mT2s * invL * r2;
  const double T1n = b.pt1sq + x1 * x1 * mp2, T2n = b.pt2sq + x2 * x2 * mp2;
  const double t1 = -T1n * r1, t2 = -T2n * r2;
  e.x10 = T(x1); e.x20 = T(x2); e.r10 = T(r1); e.r20 = T(r2);
  e.mT1s0 = T(mT1s); e.mT2s0 = T(mT2s); e.T1n0 = T(T1n); e.T2n0 = T(T2n);
  e.t10 = T(t1); e.t20 = T(t2);
  auto sinv = [&](double pp, double pm, double mq, double qp, double qm, double mr, double dot) {
    return mq + mr + pp * qm + pm * qp - 2.0 * dot;
  };
  const double s13 = sinv(p1p, p1m, mp2, b.p3p, b.p3m, b.m3sq, b.p1x * b.p3x + b.p1y * b.p3y);
  const double s14 = sinv(p1p, p1m, mp2, b.p4p, b.p4m, b.m4sq, b.p1x * b.p4x + b.p1y * b.p4y);
  const double s23 = sinv(p2p, p2m, mp2, b.p3p, b.p3m, b.m3sq, b.p2x * b.p3x + b.p2y * b.p3y);
  const double s24 = sinv(p2p, p2m, mp2, b.p4p, b.p4m, b.m4sq, b.p2x * b.p4x + b.p2y * b.p4y);
  if constexpr (sizeof(T) == sizeof(float)) {
    // FP32 fields: the reciprocal of the rounded value (within 1 ulp of the rounded FP64 one)
    e.is13 = 1.0f / float(s13); e.is14 = 1.0f / float(s14);
    e.is23 = 1.0f / float(s23); e.is24 = 1.0f / float(s24);
  } else {
    e.is13 = T(1.0 / s13); e.is14 = T(1.0 / s14); e.is23 = T(1.0 / s23); e.is24 = T(1.0 / s24);
  }
  const double l0 = log(P.regge.s0);
  const double L13 = log(s13) - l0, L14 = log(s14) - l0, L23 = log(s23) - l0, L24 = log(s24) - l0;
  e.L13 = T(L13 * kLog2e); e.L14 = T(L14 * kLog2e); e.L23 = T(L23 * kLog2e);
  e.L24 = T(L24 * kLog2e);
  const int k = K.active[0] ? 0 : (K.active[1] ? 1 : 2);
  const double a0 = P.regge.a0[k], ap = P.regge.ap[k];
  e.a10 = T(a0 + ap * t1); e.a20 = T(a0 + ap * t2);
  e.dpa0 = T(b.p4p - K.eps + p2p); e.dma0 = T(K.eps - p1m - b.p3m);
  e.dpb0 = T(b.p3p - K.eps + p2p); e.dmb0 = T(K.eps - p1m - b.p4m);
  e.c3x = T(b.p1x + b.p3x); e.c3y = T(b.p1y + b.p3y);
  e.c4x = T(b.p1x + b.p4x); e.c4y = T(b.p1y + b.p4y);
  double pre = K.gN2 * K.g2;
  // tree-level exponents E = a1 L13 + a2 L24 (+ exponential form factors)
  double Et = (a0 + ap * t1) * L13 + (a0 + ap * t2) * L24;
  double Eu = (a0 + ap * t1) * L14 + (a0 + ap * t2) * L23;
  const double ta = (b.p4p - K.eps + p2p) * (K.eps - p1m - b.p3m) -
                    ((b.p1x + b.p3x) * (b.p1x + b.p3x) + (b.p1y + b.p3y) * (b.p1y + b.p3y)) - K.M2prop;
  const double tb = (b.p3p - K.eps + p2p) * (K.eps - p1m - b.p4m) -
                    ((b.p1x + b.p4x) * (b.p1x + b.p4x) + (b.p1y + b.p4y) * (b.p1y + b.p4y)) - K.M2prop;
  double fa = 0, fb = 0;
  if (e.ffmode == 2) {
    pre *= P.regge.b_POW * P.regge.b_POW;
  } else if (e.ffmode == 0) {
    fa = -2.0 * P.regge.b_EXP * fabs(ta);
    fb = -2.0 * P.regge.b_EXP * fabs(tb);
  } else {
    fa = 2.0 * (P.regge.a_OREAR * P.regge.b_OREAR -
                P.regge.b_OREAR * sqrt(fabs(ta) + P.regge.a_OREAR * P.regge.a_OREAR));
    fb = 2.0 * (P.regge.a_OREAR * P.regge.b_OREAR -
                P.regge.b_OREAR * sqrt(fabs(tb) + P.regge.a_OREAR * P.regge.a_OREAR));
  }
  e.fa0 = T(fa * kLog2e); e.fb0 = T(fb * kLog2e);
  Et += fa;
  Eu += fb;
  const double Em = Et > Eu ? Et : Eu;
  // exp(Et - Em), exp(Eu - Em): the larger channel's is exactly 1
  const double rx = exp(Et > Eu ? Eu - Et : Et - Eu);
  const double rt = Et > Eu ? 1.0 : rx, ru = Et > Eu ? rx : 1.0;
  e.rho_t = T(rt); e.rho_u = T(ru);
  e.escale = exp(Em);
  // couplings x ReggeEta(a0)^2 x exp(-i pi ap (t1 + t2)/2) at k = 0
  const double er = K.eta0_re[k], ei = K.eta0_im[k];
  const double e2r = er * er - ei * ei, e2i = 2.0 * er * ei;
  double sn, cs;
  sincos_pi(-0.5 * ap * (t1 + t2), sn, cs);
  const double pr = pre * (e2r * cs - e2i * sn), pi = pre * (e2r * sn + e2i * cs);
  e.pre_re = T(pr);
  e.pre_im = T(pi);
  if (A0re) {
    // tree-level amplitude from the same factors (FP64)
    const double i1 = K.ifc1, i2 = K.ifc2;
    const double Pd = (1.0 - t1 * i1) * (1.0 - t1 * i2) * (1.0 - t2 * i1) * (1.0 - t2 * i2);
    double m;
    if (e.ffmode == 2) {
      const double Da = P.regge.b_POW - ta, Db = P.regge.b_POW - tb;
      m = (rt * Db * Db * tb + ru * Da * Da * ta) / (Pd * Da * Da * Db * Db * ta * tb);
    } else {
      m = (rt * tb + ru * ta) / (Pd * ta * tb);
    }
    *A0re = pr * m * e.escale;
    *A0im = pi * m * e.escale;
  }
}

// Bare Regge amplitude at loop momentum k = (kx, ky), k2 = kx^2 + ky^2, relative to
// exp(Emax) of the event (single active trajectory). Same quantity as
// loop_point_amp (src/MContinuum.cc:94-161 kinematics, src/MRegge.cc:394-438).
template <typename T>
GRN_HD bool loop_point_amp_fast(const LoopEventF<T> &e, T kx, T ky, T k2, cx<T> &A) {
  const T kd1 = kx * e.p1x + ky * e.p1y;
  const T kd2 = kx * e.p2x + ky * e.p2y;
  const T dm1 = k2 - T(2) * kd1;  // d(mT1^2) = d(pT1^2)
  const T dm2 = k2 + T(2) * kd2;
  const T dc1 = dm1 * e.invL2, dc2 = dm2 * e.invL2;
  const T dx1 = dc2 * e.ia2, dx2 = dc1 * e.ia1;
  const T dr1 = e.q1c * dc2, dr2 = e.q2c * dc1;
  const T r1 = e.r10 + dr1, r2 = e.r20 + dr2;
  const T dp1m = e.invL * (dm1 * r1 + e.mT1s0 * dr1);
  const T dp2p = e.invL * (dm2 * r2 + e.mT2s0 * dr2);
  const T dp1p = -dx1 * e.L, dp2m = -dx2 * e.L;
  const T k3 = kx * e.p3x + ky * e.p3y, k4 = kx * e.p4x + ky * e.p4y;
  const T ds13 = dp1p * e.p3m + dp1m * e.p3p + T(2) * k3;
  const T ds14 = dp1p * e.p4m + dp1m * e.p4p + T(2) * k4;
  const T ds23 = dp2p * e.p3m + dp2m * e.p3p - T(2) * k3;
  const T ds24 = dp2p * e.p4m + dp2m * e.p4p - T(2) * k4;
  // log2 of the s ratios; exponents below are in log2 units
  const T d13 = fast_log2(T(1) + ds13 * e.is13);
  const T d14 = fast_log2(T(1) + ds14 * e.is14);
  const T d23 = fast_log2(T(1) + ds23 * e.is23);
  const T d24 = fast_log2(T(1) + ds24 * e.is24);
  const T dt1 = -(dm1 + dx1 * (T(2) * e.x10 + dx1) * e.mp2) * r1 - e.T1n0 * dr1;
  const T dt2 = -(dm2 + dx2 * (T(2) * e.x20 + dx2) * e.mp2) * r2 - e.T2n0 * dr2;
  const T t1 = e.t10 + dt1, t2 = e.t20 + dt2;
  T dEt = e.ap * (dt1 * (e.L13 + d13) + dt2 * (e.L24 + d24)) + e.a10 * d13 + e.a20 * d24;
  T dEu = e.ap * (dt1 * (e.L14 + d14) + dt2 * (e.L23 + d23)) + e.a10 * d14 + e.a20 * d23;
  // t_hat - M2 and u_hat - M2
  const T ta = (e.dpa0 + dp2p) * (e.dma0 - dp1m) -
               ((e.c3x - kx) * (e.c3x - kx) + (e.c3y - ky) * (e.c3y - ky)) - e.M2;
  const T tb = (e.dpb0 + dp2p) * (e.dmb0 - dp1m) -
               ((e.c4x - kx) * (e.c4x - kx) + (e.c4y - ky) * (e.c4y - ky)) - e.M2;
  const T Pd = (T(1) - t1 * e.ifc1) * (T(1) - t1 * e.ifc2) * (T(1) - t2 * e.ifc1) *
               (T(1) - t2 * e.ifc2);
  T num, den;
  if (e.ffmode == 2) {
    const T Da = e.ff_b - ta, Db = e.ff_b - tb;
    const T Xt = e.rho_t * fast_exp2(dEt), Xu = e.rho_u * fast_exp2(dEu);
    num = Xt * (Db * Db) * tb + Xu * (Da * Da) * ta;
    den = Pd * (Da * Da) * (Db * Db) * ta * tb;
  } else {
    T fa, fb;  // 2 log2 of the off-shell form factors
    if (e.ffmode == 0) {
      fa = T(-2.0 * kLog2e) * e.ff_b * fabs(ta);
      fb = T(-2.0 * kLog2e) * e.ff_b * fabs(tb);
    } else {
      fa = T(2.0 * kLog2e) * (e.ff_ab - e.ff_b * sqrt(fabs(ta) + e.ff_a2));
      fb = T(2.0 * kLog2e) * (e.ff_ab - e.ff_b * sqrt(fabs(tb) + e.ff_a2));
    }
    const T Xt = e.rho_t * fast_exp2(dEt + (fa - e.fa0));
    const T Xu = e.rho_u * fast_exp2(dEu + (fb - e.fb0));
    num = Xt * tb + Xu * ta;
    den = Pd * ta * tb;
  }
  T sn, cs;
  fast_sincos_pi(T(-0.5) * e.ap * (dt1 + dt2), sn, cs);
  const T m = fast_div(num, den);
  A = {(e.pre_re * cs - e.pre_im * sn) * m, (e.pre_re * sn + e.pre_im * cs) * m};
  return (e.x10 + dx1 < T(1)) && (e.x20 + dx2 < T(1));
}

// rescale (the FP32 loop): events whose Regge exponent (Regge continuum) or resonance sums
// (tensor-pomeron resonances alone) fall outside the FP32 range get the event scale of
// LoopEvent (lnsc, escale); the FP64 loop keeps 0 and 1.
template <typename T>
GRN_HD void make_loop_event(const grn_process_params &P, const Consts &K, const Born &b,
                            LoopEvent<T> &e, bool rescale = false) {
  e.p1x = T(b.p1x); e.p1y = T(b.p1y); e.p2x = T(b.p2x); e.p2y = T(b.p2y);
  e.p3x = T(b.p3x); e.p3y = T(b.p3y); e.p4x = T(b.p4x); e.p4y = T(b.p4y);
  e.p3p = T(b.p3p); e.p3m = T(b.p3m); e.p4p = T(b.p4p); e.p4m = T(b.p4m);
  const double a1 = (b.p3p + b.p4p - K.eps) * K.invL, a2 = (b.p3m + b.p4m - K.eps) * K.invL;
  e.a1 = T(a1);
  e.a2 = T(a2);
  e.ia1 = T(1.0 / (1.0 - a1));
  e.ia2 = T(1.0 / (1.0 - a2));
  e.L = T(K.L); e.invL2 = T(K.invL2); e.invL = T(K.invL);
  e.eps = T(K.eps); e.mp2 = T(K.mp2); e.m3sq = T(b.m3sq); e.m4sq = T(b.m4sq);
  e.mf1 = T(b.mf1sq); e.mf2 = T(b.mf2sq); e.exc = b.exc;
  e.lnsc   = T(0);
  e.escale = 1.0;
  if (K.n_res > 0) {
    const ResVec<double> v =
        res_vectors<double>(K, b.p3p, b.p3m, b.p3x, b.p3y, b.p4p, b.p4m, b.p4x, b.p4y);
    const ResSums<double> R = resonance_sums(K, b.m2, v);
    double sc = 1.0;
    if (rescale && P.process == GRN_PROC_TENSOR_RES) {
      // the resonance factors F^2 / |m^2 - M0^2 + i M0 W|^2 reach exp(-2 (m^2 - M0^2)^2)
      double rmax = fmax(fabs(R.R0.re) + fabs(R.R0.im), fabs(R.R1.re) + fabs(R.R1.im));
      for (int j = 0; j < 7; ++j) rmax = fmax(rmax, fabs(R.Rs[j].re) + fabs(R.Rs[j].im));
      if (rmax > 0.0 && (rmax < 1e-25 || rmax > 1e25)) {
        // clamped so that 2^-k stays finite for subnormal factors (their weights are ~0)
        const int k = ilogb(rmax) < -1020 ? -1020 : (ilogb(rmax) > 1020 ? 1020 : ilogb(rmax));
        sc       = ldexp(1.0, -k);
        e.escale = ldexp(1.0, k);
      }
    }
    for (int j = 0; j < 7; ++j) e.res.Rs[j] = {T(R.Rs[j].re * sc), T(R.Rs[j].im * sc)};
    e.res.R0 = {T(R.R0.re * sc), T(R.R0.im * sc)};
    e.res.R1 = {T(R.R1.re * sc), T(R.R1.im * sc)};
    e.res.pi = {T(R.pi.pp), T(R.pi.pm), T(R.pi.px), T(R.pi.py), T(R.pi.mm),
                T(R.pi.mx), T(R.pi.my), T(R.pi.xx), T(R.pi.xy), T(R.pi.yy)};
  } else {
    e.res = ResSums<T>{};
  }
  if (rescale && P.process == GRN_PROC_REGGE_CON) {
    // the tree-level exponent alpha(t1) ln(s1x) + alpha(t2) ln(s2y) of the larger channel and
    // trajectory; beyond +-40 the loop points (within ~20 of it) would leave the FP32 range
    const grn_regge_params &rp = P.regge;
    const double l13 = log(b.s13) - K.lns0, l14 = log(b.s14) - K.lns0;
    const double l23 = log(b.s23) - K.lns0, l24 = log(b.s24) - K.lns0;
    double x0 = -1e300;
    for (int k = 0; k < 3; ++k) {
      if (!K.active[k]) continue;
      const double al1 = rp.a0[k] + rp.ap[k] * b.t1, al2 = rp.a0[k] + rp.ap[k] * b.t2;
      x0 = fmax(x0, fmax(al1 * l13 + al2 * l24, al1 * l14 + al2 * l23));
    }
    if (x0 < -40.0 || (x0 > 40.0 && x0 < 700.0)) {
      e.lnsc   = T(x0);
      e.escale = exp(double(T(x0)));
    }
  }
}

// Observables of a Born point (GRN_OBS_* order), for the on-the-fly histograms.
// Observables from the system X (light-cone Xp, Xm, transverse Xx, Xy, mass^2 m2), the
// forward transverse momenta, and the first two central particles (light-cone, transverse,
// mass^2 of the first).
GRN_HD_COLD void observables_core(const Consts &K, double Xp, double Xm, double Xx, double Xy,
                                  double m2, double p1x, double p1y, double p2x, double p2y,
                                  double p3p, double p3m, double p3x, double p3y, double m3sq,
                                  double y4, double *o) {
  const double Xe = 0.5 * (Xp + Xm), Xz = 0.5 * (Xp - Xm), M = sqrt(fmax(m2, 0.0));
  o[GRN_OBS_M]  = M;
  o[GRN_OBS_Y]  = 0.5 * log(Xp / Xm);
  o[GRN_OBS_PT] = sqrt(Xx * Xx + Xy * Xy);
  double dphi   = atan2(p1y, p1x) - atan2(p2y, p2x);
  while (dphi >= kPi) dphi -= 2.0 * kPi;
  while (dphi < -kPi) dphi += 2.0 * kPi;
  o[GRN_OBS_DPHI_PP] = fabs(dphi);
  o[GRN_OBS_PT1]     = sqrt(p1x * p1x + p1y * p1y);
  o[GRN_OBS_M0]      = sqrt(m3sq);
  o[GRN_OBS_RAP3]    = 0.5 * log(p3p / p3m);
  o[GRN_OBS_RAP4]    = y4;
  // first central particle and the beams in the X rest frame
  double px = p3x, py = p3y, pz = 0.5 * (p3p - p3m);
  const double pe = 0.5 * (p3p + p3m);
  o[GRN_OBS_COSTH_LA] = pz / sqrt(px * px + py * py + pz * pz);
  o[GRN_OBS_PHI_LA]   = atan2(py, px);
  boost_to_rest<double>(Xe, Xx, Xy, Xz, M, pe, px, py, pz);
  const double E = 0.5 * K.sqrt_s, bz = 0.5 * (K.L - K.eps);
  double a[3] = {0.0, 0.0, bz}, c[3] = {0.0, 0.0, -bz};
  boost_to_rest<double>(Xe, Xx, Xy, Xz, M, E, a[0], a[1], a[2]);
  boost_to_rest<double>(Xe, Xx, Xy, Xz, M, E, c[0], c[1], c[2]);
  auto unit = [](double *v) {
    const double n = sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    v[0] /= n; v[1] /= n; v[2] /= n;
  };
  auto cross = [](const double *u, const double *v, double *w) {
    w[0] = u[1] * v[2] - u[2] * v[1];
    w[1] = u[2] * v[0] - u[0] * v[2];
    w[2] = u[0] * v[1] - u[1] * v[0];
  };
  double ua[3] = {a[0], a[1], a[2]}, uc[3] = {c[0], c[1], c[2]};
  unit(ua);
  unit(uc);
  double y[3];
  cross(ua, uc, y);
  unit(y);
  const double pn = sqrt(px * px + py * py + pz * pz);
  for (int f = 0; f < 5; ++f) {  // CS, HX, AH, PG, CM
    double z[3], yy[3] = {y[0], y[1], y[2]};
    if (f == 0) { z[0] = ua[0] - uc[0]; z[1] = ua[1] - uc[1]; z[2] = ua[2] - uc[2]; }
    if (f == 1) { z[0] = -(a[0] + c[0]); z[1] = -(a[1] + c[1]); z[2] = -(a[2] + c[2]); }
    if (f == 2) { z[0] = ua[0] + uc[0]; z[1] = ua[1] + uc[1]; z[2] = ua[2] + uc[2]; }
    if (f == 3) { z[0] = c[0]; z[1] = c[1]; z[2] = c[2]; }
    if (f == 4) { z[0] = 0.0; z[1] = 0.0; z[2] = 1.0; yy[0] = 0.0; yy[1] = 1.0; yy[2] = 0.0; }
    unit(z);
    double x[3];
    cross(yy, z, x);
    unit(x);
    const double qx = px * x[0] + py * x[1] + pz * x[2];
    const double qy = px * yy[0] + py * yy[1] + pz * yy[2];
    const double qz = px * z[0] + py * z[1] + pz * z[2];
    o[GRN_OBS_COSTH_CS + 2 * f] = qz / pn;
    o[GRN_OBS_PHI_CS + 2 * f]   = (qx == 0.0 && qy == 0.0) ? 0.0 : atan2(qy, qx);
  }
}

GRN_HD_COLD void event_observables(const Consts &K, const Born &b, double *o) {
  observables_core(K, b.p3p + b.p4p, b.p3m + b.p4m, b.p3x + b.p4x, b.p3y + b.p4y, b.m2, b.p1x,
                   b.p1y, b.p2x, b.p2y, b.p3p, b.p3m, b.p3x, b.p3y, b.m3sq, b.y4, o);
}

GRN_HD bool is_regge_res(const grn_process_params &P) {
  return P.process == GRN_PROC_REGGE_RES || P.process == GRN_PROC_REGGE_RESCON;
}

// Tree-level Regge resonances (+ continuum for PP[RES+CON]) from the Born kinematics.
GRN_HD_COLD cx<double> regge_res_born(const grn_process_params &P, const Consts &K, const Born &b) {
  RegRes<double> R;
  regge_res_event(P, K, b.p3p, b.p3m, b.p3x, b.p3y, b.p4p, b.p4m, b.p4x, b.p4y, R);
  const double Xp = b.p3p + b.p4p, Xm = b.p3m + b.p4m, Xx = b.p3x + b.p4x, Xy = b.p3y + b.p4y;
  const double s1 = K.mp2 + b.m2 + b.p1p * Xm + b.p1m * Xp - 2.0 * (b.p1x * Xx + b.p1y * Xy);
  const double s2 = K.mp2 + b.m2 + b.p2p * Xm + b.p2m * Xp - 2.0 * (b.p2x * Xx + b.p2y * Xy);
  double q1p, q1m;
  q_lightcone<double>(b.x1, b.pt1sq, K.mp2, K.L, q1p, q1m);
  cx<double> A = regge_res_amp<double>(P, K, R, b.t1, b.t2, log(s1), log(s2), 0.5 * (q1p + q1m),
                                       -b.p1x, -b.p1y, 0.5 * (q1p - q1m));
  if (P.process == GRN_PROC_REGGE_RESCON)
    A = cadd(A, regge_me4<double>(P, K, b.t1, b.t2, log(b.s13), log(b.s14), log(b.s23),
                                  log(b.s24), b.that, b.uhat));
  return A;
}

// Tree-level amplitude of the configured process from the Born kinematics (FP64).
GRN_HD cx<double> born_amp(const grn_process_params &P, const Consts &K, const Born &b) {
  if (is_regge_res(P)) return regge_res_born(P, K, b);
  if (P.process == GRN_PROC_TENSOR_CON || P.process == GRN_PROC_TENSOR_RES ||
      P.process == GRN_PROC_TENSOR_RESCON) {
    LCKin<double> k{b.p1p, b.p1m, b.p1x, b.p1y, b.p2p, b.p2m, b.p2x,  b.p2y, b.p3p,
                    b.p3m, b.p3x, b.p3y, b.p4p, b.p4m, b.p4x, b.p4y,  K.L,   K.eps,
                    K.mp2, b.t1,  b.t2,  b.s13, b.s14, b.s23, b.s24, b.that, b.uhat};
    if (P.process == GRN_PROC_TENSOR_CON) return tensor_me4_2xs<double>(P, K, k);
    // RES+CONTENSOR: the 2xS continuum and the resonances summed coherently (MSubProc.h:319-351;
    // all four non-flip proton helicity amplitudes of each are equal)
    const cx<double> Ac = P.process == GRN_PROC_TENSOR_RESCON ? tensor_me4_2xs<double>(P, K, k)
                                                               : cx<double>{0.0, 0.0};
    if (K.n_res == 0) return Ac;
    q_lightcone<double>(b.x1, b.pt1sq, K.mp2, K.L, k.q1p, k.q1m);
    q_lightcone<double>(b.x2, b.pt2sq, K.mp2, K.L, k.q2m, k.q2p);
    const ResVec<double> v =
        res_vectors<double>(K, b.p3p, b.p3m, b.p3x, b.p3y, b.p4p, b.p4m, b.p4x, b.p4y);
    return cadd(Ac, tensor_me3<double>(P, K, k, resonance_sums(K, b.m2, v)));
  }
  return regge_me4<double>(P, K, b.t1, b.t2, log(b.s13), log(b.s14), log(b.s23), log(b.s24),
                           b.that, b.uhat, b.exc, b.mf1sq, b.mf2sq);
}

// Processes whose |M|^2 is a sum over several helicity amplitudes (vector pairs, "2xV").
GRN_HD bool is_vector_pair(const grn_process_params &P) {
  return P.process == GRN_PROC_TENSOR_CON && P.central_spin == 1;
}

// Tree-level 2xV amplitudes (FP64) in the polarization basis of the central pair.
GRN_HD_COLD void born_amps_2xv(const grn_process_params &P, const Consts &K, const Born &b,
                          cx<double> A[9]) {
  LCKin<double> k{b.p1p, b.p1m, b.p1x, b.p1y, b.p2p, b.p2m, b.p2x,  b.p2y, b.p3p,
                  b.p3m, b.p3x, b.p3y, b.p4p, b.p4m, b.p4x, b.p4y,  K.L,   K.eps,
                  K.mp2, b.t1,  b.t2,  b.s13, b.s14, b.s23, b.s24, b.that, b.uhat};
  q_lightcone<double>(b.x1, b.pt1sq, K.mp2, K.L, k.q1p, k.q1m);
  q_lightcone<double>(b.x2, b.pt2sq, K.mp2, K.L, k.q2m, k.q2p);
  LV<double> e3[3], e4[3];
  vector_basis<double>(b.p3p, b.p3m, b.p3x, b.p3y, e3);
  vector_basis<double>(b.p4p, b.p4m, b.p4x, b.p4y, e4);
  tensor_me4_2xv<double>(P, K, k, vector_prop_consts<double>(K.M2prop, b.m2), e3, e4, A);
}

// Unscreened |M|^2 of the tree-level point (sum over the helicity amplitudes; the four
// proton helicity configurations of the high-energy vertex are equal and averaged).
template <bool VV = false>
GRN_HD double born_amp2(const grn_process_params &P, const Consts &K, const Born &b) {
  if (VV && is_vector_pair(P)) {
    cx<double> A[9];
    born_amps_2xv(P, K, b, A);
    double s = 0.0;
    for (int h = 0; h < 9; ++h) s += A[h].re * A[h].re + A[h].im * A[h].im;
    return s;
  }
  const cx<double> A0 = born_amp(P, K, b);
  return A0.re * A0.re + A0.im * A0.im;
}

// u-independent part of the weight and the u-dependent Jacobians
// (MContinuum::EventWeight, BNPhaseSpaceWeight, BNIntegralVolume and
// ForwardVolume; src/MContinuum.cc:164-193, 619-656; src/MProcess.cc:1390-1415;
// for <F>: MFactorized::EventWeight, B51PhaseSpaceWeight, B51IntegralVolume and the
// 2-body phase-space factor dPhi2/(2 pi), src/MFactorized.cc:142-184, 418-450).
GRN_HD double weight_jacobian(const Consts &K, const Born &b) {
  const double E1 = 0.5 * (b.p1p + b.p1m), pz1 = 0.5 * (b.p1p - b.p1m);
  const double E2 = 0.5 * (b.p2p + b.p2m), pz2 = 0.5 * (b.p2p - b.p2m);
  // (pT1 / 2E1) (pT2 / 2E2) J pT1 pT2 with J = 1 / |pz1/E1 - pz2/E2|
  //   = pT1^2 pT2^2 / (4 |pz1 E2 - pz2 E1|): one division, no square root (pz1 E2 and
  // -pz2 E1 have the same sign for the two forward legs, so nothing cancels)
  const double den = 4.0 * fabs(pz1 * E2 - pz2 * E1);
  return K.w_const * (b.pt1sq * b.pt2sq / den) * b.jx * b.jf;
}

}  // namespace grn
