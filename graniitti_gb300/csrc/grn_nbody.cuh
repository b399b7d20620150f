// Regge continuum of four or six central particles: PP[CON]<F|C> -> a b c d (MRegge::ME6,
// src/MRegge.cc:470-534) and -> a b c d e f (MRegge::ME8, src/MRegge.cc:560-627).
// Factorized class: the central system decayed by the flat N-body
// phase space of MKinematics.h:523-691 (NBodySetup, NBodyPhaseSpace) and the event weight of
// MFactorized::EventWeight (src/MFactorized.cc:142-184). Continuum class: the 14-dimensional
// phase space of MContinuum::BNRandomKin / BNBuildKin (src/MContinuum.cc:276-435).
//
// Factorized hypercube (3 N + 2 coordinates, N central particles): u[0..5] the factorized
// skeleton (log pT of the forward legs, their azimuths, the system rapidity and mass^2),
// u[6..N+3] the N - 2 intermediate-mass draws of NBodySetup (used in ascending order),
// u[N+4+2k], u[N+5+2k] (cos theta = 2 u - 1, phi = 2 pi u) of the k-th decay of the
// recursion (particles N-1, ..., 1 of the decay list in that order). These are the draws the
// reference takes from its random-number generator inside EventWeight, in the same order.
//
// The amplitude is the sum over the 24 orderings (a, b, c, d) of the four particles along
// the ladder:
//   R(s_1a, t1) FF(t1) ff(t_a, MA) / (t_a - MA) ff(t_ab, MA) R(s_bc, t_ab) ff(t_ab, MB)
//   / (t_d - MB) ff(t_d, MB) R(s_2d, t2) FF(t2) g^4
// with t_a = (q1 - p_a)^2, t_ab = (q1 - p_a - p_b)^2, t_d = (q2 - p_d)^2, R the Regge
// propagator sum and ff the off-shell meson form factor; MA, MB the masses of the first and
// third particle of the decay list. Invariants are formed from light-cone components (no
// cancellation against the beam energy). Screened events run the kt-loop in FP64: the
// forward legs take p1T - kT, p2T + kT; in the factorized class the central system and its
// decay products keep their momenta (MFactorized::LoopKinematics, src/MFactorized.cc:84-139),
// in the continuum class the central transverse momenta are re-solved with the tree-level
// difference momenta, rapidities and masses (MContinuum::LoopKinematics).
#pragma once

#include "grn_physics.cuh"

namespace grn {

constexpr int kNb    = 4;  // central particles of the 4-body processes (the FP32 loop's shape)
constexpr int kNbMax = 6;  // the largest central multiplicity (ME8)

GRN_HD bool is_nbody(const grn_process_params &P) { return P.n_central >= kNb; }

// Light-cone 4-vector (p = E + pz, m = E - pz).
struct LC4 {
  double p, m, x, y;
};

GRN_HD double lc_dot(const LC4 &a, const LC4 &b) {
  return 0.5 * (a.p * b.m + a.m * b.p) - a.x * b.x - a.y * b.y;
}

// Lab 4-vector (px, py, pz, E) to light-cone with the smaller component from mT^2.
GRN_HD LC4 lc_from_lab(double px, double py, double pz, double E, double m2) {
  const double mt2 = m2 + px * px + py * py;
  LC4 r;
  r.x = px;
  r.y = py;
  if (pz >= 0) {
    r.p = E + pz;
    r.m = mt2 / r.p;
  } else {
    r.m = E - pz;
    r.p = mt2 / r.m;
  }
  return r;
}

struct NBEvent {
  int    n;                 // central particles (4 or 6)
  LC4    X;                 // central system
  LC4    c[kNbMax];         // central particles in decay-list order
  double m2[kNbMax];        // their masses^2
  double p1x, p1y, p2x, p2y, pt1sq, pt2sq;  // tree-level forward transverse momenta
  double a1, a2;            // (X+ - eps)/L, (X- - eps)/L: forward-leg closure constants
  double dw;                // N-body phase-space weight (NBodySetup volume x momenta)
  double m2w;               // mass^2 window of the system (B51IntegralVolume)
  double sbc[kNbMax][kNbMax];  // (p_b + p_c)^2 of central pairs
  bool   cuts;              // the central particles pass the particle cuts
  bool   veto;              // a central particle hits a veto domain
  double jx;                // per-event phase-space factor: F dPhi_N / (2 pi) x mass^2 window,
                            // C the product of the difference momenta kt_i
  double kx[kNbMax - 1], ky[kNbMax - 1], y[kNbMax];  // C: difference momenta, rapidities
};

// Forward legs at transverse momenta (q1x, q1y), (q2x, q2y): light-cone closure (the
// solution kinematics::SolvePz picks), t1, t2 and q1 = pb1 - p1, q2 = pb2 - p2.
struct NBLegs {
  LC4    p1, p2, q1, q2;
  double t1, t2;
};

GRN_HD bool nbody_legs(const Consts &K, const NBEvent &e, double p1x, double p1y, double p2x,
                       double p2y, NBLegs &g) {
  const double pt1sq = p1x * p1x + p1y * p1y, pt2sq = p2x * p2x + p2y * p2y;
  const double mT1sq = K.mp2 + pt1sq, mT2sq = K.mp2 + pt2sq;
  const double L2 = K.L * K.L;
  double x1, x2;
  if (!solve_x(e.a1, e.a2, mT1sq / L2, mT2sq / L2, x1, x2)) return false;
  g.p1 = {(1.0 - x1) * K.L, 0.0, p1x, p1y};
  g.p1.m = mT1sq / g.p1.p;
  g.p2 = {0.0, (1.0 - x2) * K.L, p2x, p2y};
  g.p2.p = mT2sq / g.p2.m;
  g.t1 = -(pt1sq + x1 * x1 * K.mp2) / (1.0 - x1);
  g.t2 = -(pt2sq + x2 * x2 * K.mp2) / (1.0 - x2);
  q_lightcone<double>(x1, pt1sq, K.mp2, K.L, g.q1.p, g.q1.m);
  q_lightcone<double>(x2, pt2sq, K.mp2, K.L, g.q2.m, g.q2.p);
  g.q1.x = -p1x;
  g.q1.y = -p1y;
  g.q2.x = -p2x;
  g.q2.y = -p2y;
  return true;
}

// Pair invariants and particle cuts of the central particles in e.c (GetLorentzScalars,
// MProcess.cc:1515-1530; CommonCuts, MProcess.cc:1085-1138); false for a negative pair mass^2.
GRN_HD bool nbody_finish(const grn_process_params &P, NBEvent &e) {
  for (int a = 0; a < e.n; ++a)
    for (int b = a + 1; b < e.n; ++b) {
      e.sbc[a][b] = e.m2[a] + e.m2[b] + 2.0 * lc_dot(e.c[a], e.c[b]);
      e.sbc[b][a] = e.sbc[a][b];
      if (e.sbc[a][b] < 0) return false;
    }
  e.veto = false;
  if (P.veto_active)
    for (int a = 0; a < e.n; ++a)
      e.veto |= veto_hit(P, e.c[a].x, e.c[a].y, 0.5 * (e.c[a].p - e.c[a].m));
  const grn_fidcuts &f = P.fcuts;
  e.cuts = true;
  if (f.active) {
    for (int a = 0; a < e.n; ++a) {
      const double pt  = sqrt(e.c[a].x * e.c[a].x + e.c[a].y * e.c[a].y);
      const double mt  = sqrt(e.m2[a] + pt * pt);
      const double y   = 0.5 * log(e.c[a].p / e.c[a].m);
      const double eta = asinh(0.5 * (e.c[a].p - e.c[a].m) / pt);
      if (!(pt >= f.pt_min && pt <= f.pt_max && mt >= f.Et_min && mt <= f.Et_max &&
            eta >= f.eta_min && eta <= f.eta_max && y >= f.rap_min && y <= f.rap_max))
        e.cuts = false;
    }
  }
  return true;
}

// Continuum class (MContinuum::BNBuildKin, src/MContinuum.cc:334-435): central transverse
// momenta from the linear system of MContinuum::BLinearSystem for N = 4 or 6 particles,
//   2 p0 = q0 - w - (p2 + ... + p_{N-1}),  2 p1 = -q0 - w - (p2 + ... + p_{N-1}),
//   2 p_i = -q_{i-1} - w - (the sum of the p_j with j != i, i - 1),  i >= 2,  w = p1T + p2T,
// solved with the inverse of its matrix (exact rationals); rapidities and masses fixed, the
// system X their sum, the forward-leg closure constants from X. Also the loop kinematics of
// the class (MContinuum::LoopKinematics, src/MContinuum.cc:94-161) at new forward transverse
// momenta.
GRN_HD bool nbody_build_C(const Consts &K, NBEvent &e, double p1x, double p1y, double p2x,
                          double p2y) {
  constexpr double A4[4][4] = {{0.875, 0.125, -0.5, -0.25},
                               {0.375, 0.625, -0.5, -0.25},
                               {-0.125, 0.125, 0.5, -0.25},
                               {-0.625, -0.375, 0.5, 0.75}};
  constexpr double A6[6][6] = {
      {4.0 / 3, 1.0 / 2, -2.0 / 3, -1.0 / 2, -1.0 / 3, -1.0 / 6},
      {5.0 / 6, 1.0, -2.0 / 3, -1.0 / 2, -1.0 / 3, -1.0 / 6},
      {1.0 / 3, 1.0 / 2, 1.0 / 3, -1.0 / 2, -1.0 / 3, -1.0 / 6},
      {-1.0 / 6, 0.0, 1.0 / 3, 1.0 / 2, -1.0 / 3, -1.0 / 6},
      {-2.0 / 3, -1.0 / 2, 1.0 / 3, 1.0 / 2, 2.0 / 3, -1.0 / 6},
      {-7.0 / 6, -1.0, 1.0 / 3, 1.0 / 2, 2.0 / 3, 5.0 / 6}};
  const int    N  = e.n;
  const double wx = p1x + p2x, wy = p1y + p2y;
  double bx[kNbMax], by[kNbMax];
  bx[0] = e.kx[0] - wx;
  by[0] = e.ky[0] - wy;
  for (int i = 1; i < N; ++i) {
    bx[i] = -e.kx[i - 1] - wx;
    by[i] = -e.ky[i - 1] - wy;
  }
  LC4    X{0.0, 0.0, 0.0, 0.0};
  double msum = 0.0;
  for (int i = 0; i < N; ++i) {
    double px = 0.0, py = 0.0;
    for (int j = 0; j < N; ++j) {
      const double a = N == 4 ? A4[i][j] : A6[i][j];
      px += a * bx[j];
      py += a * by[j];
    }
    const double mt = sqrt(e.m2[i] + px * px + py * py);
    const double ey = exp(e.y[i]);
    e.c[i] = {mt * ey, mt / ey, px, py};
    X.p += e.c[i].p;
    X.m += e.c[i].m;
    X.x += px;
    X.y += py;
    msum += sqrt(e.m2[i]);
  }
  e.X = X;
  if (0.5 * (X.p + X.m) > K.sqrt_s) return false;  // energy check (MContinuum.cc:373)
  if (!(X.p * X.m - X.x * X.x - X.y * X.y >= msum * msum)) return false;
  e.a1 = (X.p - K.eps) / K.L;
  e.a2 = (X.m - K.eps) / K.L;
  return true;
}

// B51RandomKin / B51BuildKin with the N-body decay of the central system
// (src/MFactorized.cc:245-407): false when the point is kinematically impossible.
GRN_HD bool nbody_kinematics(const grn_process_params &P, const Consts &K, const double *u,
                             NBEvent &e) {
  const grn_gencuts &g = P.gcuts;
  const int          N = P.n_central;
  e.n                  = N;
  if (P.phase_space == GRN_PS_CONTINUUM) {
    // BNRandomKin (src/MContinuum.cc:276-331): forward legs u[0..3], difference momenta kt
    // u[4..N+2] and azimuths u[N+3..2N+1], rapidities u[2N+2..3N+1]
    const double pt1 = exp(K.lnpt_lo + (K.lnpt_hi - K.lnpt_lo) * u[0]);
    const double pt2 = exp(K.lnpt_lo + (K.lnpt_hi - K.lnpt_lo) * u[1]);
    double s1, c1, s2, c2;
    sincos_pi(2.0 * u[2], s1, c1);
    sincos_pi(2.0 * u[3], s2, c2);
    e.p1x = pt1 * c1;
    e.p1y = pt1 * s1;
    e.p2x = pt2 * c2;
    e.p2y = pt2 * s2;
    e.pt1sq = e.p1x * e.p1x + e.p1y * e.p1y;
    e.pt2sq = e.p2x * e.p2x + e.p2y * e.p2y;
    e.jx = 1.0;
    for (int i = 0; i < N - 1; ++i) {
      const double kt = g.kt_min + (g.kt_max - g.kt_min) * u[4 + i];
      double sk, ck;
      sincos_pi(2.0 * u[N + 3 + i], sk, ck);
      e.kx[i] = kt * ck;
      e.ky[i] = kt * sk;
      e.jx *= kt;
    }
    for (int i = 0; i < N; ++i) {
      e.y[i]  = g.rap_min + (g.rap_max - g.rap_min) * u[2 * N + 2 + i];
      e.m2[i] = P.m_central[i] * P.m_central[i];
    }
    if (!nbody_build_C(K, e, e.p1x, e.p1y, e.p2x, e.p2y)) return false;
    double x1, x2;
    if (!solve_x(e.a1, e.a2, (K.mp2 + e.pt1sq) / (K.L * K.L), (K.mp2 + e.pt2sq) / (K.L * K.L),
                 x1, x2))
      return false;
    return nbody_finish(P, e);
  }
  const double pt1 = exp(K.lnpt_lo + (K.lnpt_hi - K.lnpt_lo) * u[0]);
  const double pt2 = exp(K.lnpt_lo + (K.lnpt_hi - K.lnpt_lo) * u[1]);
  double s1, c1, s2, c2;
  sincos_pi(2.0 * u[2], s1, c1);
  sincos_pi(2.0 * u[3], s2, c2);
  const double yX  = g.Y_min + (g.Y_max - g.Y_min) * u[4];
  const double m2X = K.M2min + (K.M2max - K.M2min) * u[5];
  e.m2w = K.M2max - K.M2min;
  e.p1x = pt1 * c1;
  e.p1y = pt1 * s1;
  e.p2x = pt2 * c2;
  e.p2y = pt2 * s2;
  e.pt1sq = e.p1x * e.p1x + e.p1y * e.p1y;
  e.pt2sq = e.p2x * e.p2x + e.p2y * e.p2y;
  const double Xx = -(e.p1x + e.p2x), Xy = -(e.p1y + e.p2y);
  const double mTX = sqrt(m2X + Xx * Xx + Xy * Xy);
  const double eY = exp(yX);
  e.X = {mTX * eY, mTX / eY, Xx, Xy};
  const double EX = 0.5 * (e.X.p + e.X.m), ZX = 0.5 * (e.X.p - e.X.m);
  if (EX > K.sqrt_s - 2.0 * sqrt(K.mp2)) return false;  // energy overflow (MFactorized.cc:323)
  e.a1 = (e.X.p - K.eps) / K.L;
  e.a2 = (e.X.m - K.eps) / K.L;
  double x1, x2;
  if (!solve_x(e.a1, e.a2, (K.mp2 + e.pt1sq) / (K.L * K.L), (K.mp2 + e.pt2sq) / (K.L * K.L),
               x1, x2))
    return false;

  // NBodySetup (MKinematics.h:529-605), weighted: intermediate masses from the ordered draws,
  // decay momenta, volume 1 / (2 (2 pi)^(2N-3)) DELTA^(N-2) / (N-2)! / M0
  const double M0 = sqrt(m2X);
  double m[kNbMax], sum[kNbMax];
  for (int i = 0; i < N; ++i) {
    m[i]   = P.m_central[i];
    sum[i] = (i ? sum[i - 1] : 0.0) + m[i];
    e.m2[i] = m[i] * m[i];
  }
  const double D = M0 - sum[N - 1];
  if (!(D > 0)) return false;
  double r[kNbMax - 2];  // the N - 2 mass draws in ascending order (insertion sort)
  for (int i = 0; i < N - 2; ++i) {
    const double v = u[6 + i];
    int          j = i;
    for (; j > 0 && r[j - 1] > v; --j) r[j] = r[j - 1];
    r[j] = v;
  }
  double Meff[kNbMax];
  Meff[0]     = m[0];
  Meff[N - 1] = M0;
  for (int i = 1; i < N - 1; ++i) Meff[i] = sum[i] + r[i - 1] * D;
  double pn[kNbMax];
  double w = 1.0;
  for (int i = 1; i < N; ++i) {
    const double x = Meff[i], y = Meff[i - 1], z = m[i];
    pn[i] = sqrt(fmax(0.0, (x - y - z) * (x + y + z) * (x + y - z) * (x - y + z))) / (2.0 * x);
    w *= pn[i];
  }
  const double tp = 2.0 * kPi;
  if (N == 4) {
    e.dw = w / (2.0 * (tp * tp * tp * tp * tp)) * (D * D) / 2.0 / M0;
  } else {
    const double tp3 = tp * tp * tp, D2 = D * D;
    e.dw = w / (2.0 * (tp3 * tp3 * tp3)) * (D2 * D2) / 24.0 / M0;
  }
  e.jx = e.m2w * e.dw / (2.0 * kPi);

  // NBodyPhaseSpace (MKinematics.h:643-691): from the last particle down, an isotropic
  // momentum in the rest frame of what is left, boosted to the lab with that system's
  // lab momentum, then subtracted from it; the first particle takes the remainder.
  double kx = Xx, ky = Xy, kz = ZX, kE = EX;
  for (int i = N - 1; i >= 1; --i) {
    const int    j  = N + 4 + 2 * (N - 1 - i);
    const double ct = 2.0 * u[j] - 1.0;
    const double st = sqrt(fmax(0.0, 1.0 - ct * ct));
    double sp, cp;
    sincos_pi(2.0 * u[j + 1], sp, cp);
    const double px = pn[i] * st * cp, py = pn[i] * st * sp, pz = pn[i] * ct;
    const double pE = sqrt(e.m2[i] + pn[i] * pn[i]);
    const double kM = sqrt(fmax(0.0, kE * kE - kx * kx - ky * ky - kz * kz));
    const double bx = kx / kE, by = ky / kE, bz = kz / kE, gam = kE / kM;
    const double k1 = bx * px + by * py + bz * pz;
    const double k2 = gam * (gam * k1 / (1.0 + gam) + pE);
    const double lx = px + k2 * bx, ly = py + k2 * by, lz = pz + k2 * bz, lE = gam * (pE + k1);
    e.c[i] = lc_from_lab(lx, ly, lz, lE, e.m2[i]);
    kx -= lx;
    ky -= ly;
    kz -= lz;
    kE -= lE;
  }
  e.c[0] = lc_from_lab(kx, ky, kz, kE, e.m2[0]);

  return nbody_finish(P, e);
}

// Event-level cuts: forward |t| and the system's mass, rapidity and pT (CommonCuts), plus
// the particle cuts; t from the tree-level legs.
GRN_HD bool nbody_fiducial(const grn_process_params &P, const NBEvent &e, const NBLegs &g) {
  const grn_fidcuts &f = P.fcuts;
  if (!f.active) return true;
  const double at1 = fabs(g.t1), at2 = fabs(g.t2);
  if (!(at1 >= f.ft_min && at1 <= f.ft_max && at2 >= f.ft_min && at2 <= f.ft_max)) return false;
  const double M  = sqrt(fmax(0.0, e.X.p * e.X.m - e.X.x * e.X.x - e.X.y * e.X.y));
  const double Y  = 0.5 * log(e.X.p / e.X.m);
  const double Pt = sqrt(e.X.x * e.X.x + e.X.y * e.X.y);
  if (!(M >= f.M_min && M <= f.M_max && Y >= f.Y_min && Y <= f.Y_max && Pt >= f.Pt_min &&
        Pt <= f.Pt_max))
    return false;
  return e.cuts;
}

GRN_HD_COLD bool nbody_amp6(const grn_process_params &P, const Consts &K, const NBEvent &e,
                            const NBLegs &g, cx<double> &A);

// ME6 (MRegge.cc:470-534) at forward legs g, or ME8 for six central particles; false when an
// invariant check fails (GetLorentzScalars: negative s-type invariants or positive t1, t2).
GRN_HD bool nbody_amp(const grn_process_params &P, const Consts &K, const NBEvent &e,
                      const NBLegs &g, cx<double> &A) {
  if (e.n == kNbMax) return nbody_amp6(P, K, e, g, A);
  const grn_regge_params &rp = P.regge;
  if (g.t1 > 0 || g.t2 > 0) return false;
  double lns1[kNb], lns2[kNb], d1[kNb], f1[kNb], f2[kNb];
  cx<double> R1[kNb], R2[kNb];
  const double MA = K.m3sq, MB = K.M2propB;
  for (int a = 0; a < kNb; ++a) {
    const double s1 = K.mp2 + e.m2[a] + 2.0 * lc_dot(g.p1, e.c[a]);
    const double s2 = K.mp2 + e.m2[a] + 2.0 * lc_dot(g.p2, e.c[a]);
    if (s1 < 0 || s2 < 0) return false;
    lns1[a] = log(s1);
    lns2[a] = log(s2);
    d1[a] = lc_dot(g.q1, e.c[a]);
    const double ta = g.t1 + e.m2[a] - 2.0 * d1[a];
    const double td = g.t2 + e.m2[a] - 2.0 * lc_dot(g.q2, e.c[a]);
    f1[a] = meson_ff<double>(rp, ta, MA) / (ta - MA);
    f2[a] = meson_ff<double>(rp, td, MB) / (td - MB);
    R1[a] = regge_prop<double>(K, rp, lns1[a], g.t1);
    R2[a] = regge_prop<double>(K, rp, lns2[a], g.t2);
  }
  cx<double> S{0.0, 0.0};
  for (int a = 0; a < kNb; ++a)
    for (int b = 0; b < kNb; ++b) {
      if (b == a) continue;
      const double tab = g.t1 + e.sbc[a][b] - 2.0 * (d1[a] + d1[b]);
      const double fab = meson_ff<double>(rp, tab, MA) * meson_ff<double>(rp, tab, MB);
      for (int c = 0; c < kNb; ++c) {
        if (c == a || c == b) continue;
        const int d = 6 - a - b - c;
        const cx<double> Rm = regge_prop<double>(K, rp, log(e.sbc[b][c]), tab);
        const cx<double> t  = cscale(cmul(cmul(R1[a], Rm), R2[d]), f1[a] * fab * f2[d]);
        S = cadd(S, t);
      }
    }
  const double g2 = K.g2;
  const double vtx = K.gN2 * proton_ff<double>(P.soft.fc1, P.soft.fc2, g.t1) *
                     proton_ff<double>(P.soft.fc1, P.soft.fc2, g.t2) * g2 * g2;
  A = cscale(S, vtx);
  return true;
}

// ME8 (MRegge.cc:560-627): the sum over the 720 orderings (a b c d e f) of the six central
// particles along the ladder of
//   R(s_1a, t1) FF_A ff(t_ab, MA) g / (t_ab - MA) ff(t_bc, MA) g R(s_bc, t_bc) ff(t_bc, MB) g
//   / (t_cd - MB) ff(t_de, MB) g R(s_de, t_de) ff(t_de, MC) g / (t_ef - MC) ff(t_ef, MC) g
//   R(s_2f, t2) FF_B
// with the reference's invariants t_ab = (q1 - p_a)^2, t_bc = T_ab, t_cd = T_bc, t_de = T_cd,
// t_ef = (q2 - p_f)^2, where T_xy = (q1 - p_x - p_y)^2 (the scalars it reads from
// LORENTZSCALAR::tt_xy), and MA, MB, MC the masses^2 of the first, third and fifth particle of
// the decay list. The 120 Regge factors R(s_yz, T_xy) of distinct (x, y, z) are formed once;
// each ordering is then a product of five tabulated factors.
GRN_HD_COLD bool nbody_amp6(const grn_process_params &P, const Consts &K, const NBEvent &e,
                            const NBLegs &g, cx<double> &A) {
  constexpr int N = kNbMax;
  const grn_regge_params &rp = P.regge;
  if (g.t1 > 0 || g.t2 > 0) return false;
  const double MA = P.m_central[0] * P.m_central[0], MB = P.m_central[2] * P.m_central[2];
  const double MC = P.m_central[4] * P.m_central[4];
  double     d1[N];
  cx<double> X1[N], X2[N];
  for (int a = 0; a < N; ++a) {
    const double s1 = K.mp2 + e.m2[a] + 2.0 * lc_dot(g.p1, e.c[a]);
    const double s2 = K.mp2 + e.m2[a] + 2.0 * lc_dot(g.p2, e.c[a]);
    if (s1 < 0 || s2 < 0) return false;
    d1[a] = lc_dot(g.q1, e.c[a]);
    const double ta = g.t1 + e.m2[a] - 2.0 * d1[a];
    const double tf = g.t2 + e.m2[a] - 2.0 * lc_dot(g.q2, e.c[a]);
    X1[a] = cscale(regge_prop<double>(K, rp, log(s1), g.t1), meson_ff<double>(rp, ta, MA) / (ta - MA));
    X2[a] = cscale(regge_prop<double>(K, rp, log(s2), g.t2), meson_ff<double>(rp, tf, MC) / (tf - MC));
  }
  double     fAB[N][N], fBC[N][N], pB[N][N], lsb[N][N];
  for (int x = 0; x < N; ++x)
    for (int y = x + 1; y < N; ++y) {
      const double T = g.t1 + e.sbc[x][y] - 2.0 * (d1[x] + d1[y]);
      fAB[x][y] = fAB[y][x] = meson_ff<double>(rp, T, MA) * meson_ff<double>(rp, T, MB);
      fBC[x][y] = fBC[y][x] = meson_ff<double>(rp, T, MB) * meson_ff<double>(rp, T, MC);
      pB[x][y] = pB[y][x] = 1.0 / (T - MB);
      lsb[x][y] = lsb[y][x] = log(e.sbc[x][y]);
    }
  cx<double> Rt[N][N][N];  // R(s_yz, T_xy)
  for (int x = 0; x < N; ++x)
    for (int y = 0; y < N; ++y) {
      if (y == x) continue;
      const int    lo = x < y ? x : y, hi = x < y ? y : x;
      const double T  = g.t1 + e.sbc[lo][hi] - 2.0 * (d1[x] + d1[y]);
      for (int z = 0; z < N; ++z)
        if (z != x && z != y) Rt[x][y][z] = regge_prop<double>(K, rp, lsb[y][z], T);
    }
  cx<double> S{0.0, 0.0};
  for (int a = 0; a < N; ++a)
    for (int b = 0; b < N; ++b) {
      if (b == a) continue;
      for (int c = 0; c < N; ++c) {
        if (c == a || c == b) continue;
        const cx<double> Y = cscale(cmul(X1[a], Rt[a][b][c]), fAB[a][b] * pB[b][c]);
        for (int d = 0; d < N; ++d) {
          if (d == a || d == b || d == c) continue;
          for (int k = 0; k < N; ++k) {  // k = e of the ordering, f the one left
            if (k == a || k == b || k == c || k == d) continue;
            const int f = 15 - a - b - c - d - k;
            S = cadd(S, cmul(cscale(cmul(Y, Rt[c][d][k]), fBC[c][d]), X2[f]));
          }
        }
      }
    }
  const double g2  = K.g2;
  const double vtx = K.gN2 * proton_ff<double>(P.soft.fc1, P.soft.fc2, g.t1) *
                     proton_ff<double>(P.soft.fc1, P.soft.fc2, g.t2) * g2 * g2 * g2;
  A = cscale(S, vtx);
  return true;
}

// Event weight factor without |M|^2: F: C_space = dPhi_N / (2 pi), B51PhaseSpaceWeight x
// B51IntegralVolume (MFactorized.cc:160-183, 418-450); C: BNPhaseSpaceWeight x
// BNIntegralVolume (MContinuum.cc:619-656); 1 / S, GeV^-2 -> barn and the flux.
GRN_HD double nbody_jacobian(const Consts &K, const NBEvent &e, const NBLegs &g) {
  const double E1 = 0.5 * (g.p1.p + g.p1.m), pz1 = 0.5 * (g.p1.p - g.p1.m);
  const double E2 = 0.5 * (g.p2.p + g.p2.m), pz2 = 0.5 * (g.p2.p - g.p2.m);
  const double J  = 1.0 / fabs(pz1 / E1 - pz2 / E2);
  const double pt1 = sqrt(e.pt1sq), pt2 = sqrt(e.pt2sq);
  return K.w_const * (pt1 / (2.0 * E1)) * (pt2 / (2.0 * E2)) * J * pt1 * pt2 * e.jx;
}

// kt-loop of the N-body amplitude in FP64 (MProcess::S3ScreenedAmp2 with the node tables of
// the 2-body loop).
template <typename T>
__device__ cx<double> nbody_loop(const KArgs &A, const NBEvent &e, const KtNode<T> *skt,
                                 const PhiNode<T> *sphi) {
  const bool cls_c = A.P.phase_space == GRN_PS_CONTINUUM;
  double ar = 0.0, ai = 0.0;
  for (int j = 0; j < A.n_kt_nodes; ++j) {
    const KtNode<T> nj = skt[j];
    double ir = 0.0, ii = 0.0;
    for (int i = 0; i < A.n_phi_nodes; ++i) {
      const PhiNode<T> ni = sphi[i];
      const double     kx = double(nj.kt) * double(ni.c), ky = double(nj.kt) * double(ni.s);
      const double     q1x = e.p1x - kx, q1y = e.p1y - ky, q2x = e.p2x + kx, q2y = e.p2y + ky;
      NBLegs           g;
      cx<double>       a;
      if (cls_c) {
        NBEvent el = e;
        if (!nbody_build_C(A.K, el, q1x, q1y, q2x, q2y)) continue;
        if (!nbody_finish(A.P, el)) continue;
        if (!nbody_legs(A.K, el, q1x, q1y, q2x, q2y, g)) continue;
        if (!nbody_amp(A.P, A.K, el, g, a)) continue;
      } else {
        if (!nbody_legs(A.K, e, q1x, q1y, q2x, q2y, g)) continue;
        if (!nbody_amp(A.P, A.K, e, g, a)) continue;
      }
      ir += double(ni.u) * a.re;
      ii += double(ni.u) * a.im;
    }
    ar += double(nj.cre) * ir - double(nj.cim) * ii;
    ai += double(nj.cre) * ii + double(nj.cim) * ir;
  }
  return {A.loop_norm_re * ar - A.loop_norm_im * ai, A.loop_norm_re * ai + A.loop_norm_im * ar};
}

// FP32 kt-loop of the N-body amplitude for one Regge trajectory (alpha(t) = a0 + ap t,
// signature factor eta). In both classes the central particles keep their momenta in the loop
// (factorized: MFactorized::LoopKinematics; continuum: their transverse momenta depend on the
// forward legs only through p1T + p2T, which the loop leaves unchanged), so only the forward
// legs move. With one trajectory each ordering (a b c d) of the ladder is
//   eta^3 e^{-i pi ap (t1 + t_ab + t2) / 2} e^{x_1a + x_abc + x_2d} f_a f_ab f_d
// with real exponents x = alpha(t) (ln s - ln s0) of size ~10: their FP32 rounding alone would
// leave ~1e-6 relative error per propagator. So each exponent is split into its tree-level
// value (FP64 per event; rho = e^{x_term - X} per ordering, X the largest) and an increment
//   x - x0 = ap (t - t0) l0 + alpha(t) ln(s / s0)
// formed from explicit differences of the light-cone components (t - t0, s / s0 - 1 and
// t_ab - t_ab0 never subtract two large numbers), which is small where the loop integrand is
// large; the phases e^{-i pi ap t / 2} likewise as tree-level phase times increment. Form
// factors and vertices run in FP32 on the point's own invariants.
template <typename T>
struct LCT {
  T p, m, x, y;
};
template <typename T>
GRN_HD T lct_dot(const LCT<T> &a, const LCT<T> &b) {
  return T(0.5) * (a.p * b.m + a.m * b.p) - a.x * b.x - a.y * b.y;
}

constexpr int kNbPairs = 6;   // unordered pairs {a < b}: (01) (02) (03) (12) (13) (23)
constexpr int kNbTerms = 24;  // orderings, 4 per pair

struct NBLoopF {
  LCT<float> c[kNb];                // central particles
  float      m2[kNb];
  float      p1x, p1y, p2x, p2y;    // tree-level forward transverse momenta
  float      a1, a2, ia1, ia2, L, invL, invL2, mp2;
  float      x1r, x2r;              // tree level x1 - a1 = c2 r2, x2 - a2 = c1 r1
  float      p1m, p2p, g1m, g2p;    // tree level p1-, p2+, q1-, q2+
  float      t1, t2;                // tree level t1, t2
  float      is1[kNb], is2[kNb];    // 1 / s_1a, 1 / s_2a at tree level
  float      l1[kNb], l2[kNb];      // ln s_1a - ln s0, ln s_2a - ln s0 at tree level
  float      tab[kNbPairs];         // t_ab at tree level
  cx<float>  ph[kNbPairs];          // e^{-i pi ap t_ab / 2} at tree level
  float      ljk[kNb][kNb];         // ln s_jk - ln s0
  float      rho[kNbTerms];         // e^{x_term - X} at tree level
  float      a0, ap;
  // process constants in FP32 (converted once per event, not per point): propagator masses^2,
  // couplings, proton form factor poles, off-shell form factor (form and parameters)
  float      MA, MB, g2, gN2, fc1, fc2;
  int        ffform;
  float      bexp, aore, bore, bpow;
};

// Off-shell meson form factor (meson_ff) from the FP32 copies of its parameters.
GRN_HD float meson_ff_f(const NBLoopF &f, float that, float M2) {
  const float tp = that - M2;
  if (f.ffform == 0) return expf(-f.bexp * fabsf(tp));
  if (f.ffform == 1) return expf(-f.bore * sqrtf(fabsf(tp) + f.aore * f.aore) + f.aore * f.bore);
  return 1.f / (1.f - tp / f.bpow);
}

// The ordering o = 0..3 of pair {a < b}: (i, j, k, l) = (a, b, c0, c1), (a, b, c1, c0),
// (b, a, c0, c1), (b, a, c1, c0) with c0 < c1 the two particles left.
GRN_HD void nb_order(int a, int b, int o, int &i, int &j, int &k, int &l) {
  const int c0 = (a == 0) ? (b == 1 ? 2 : 1) : 0;
  const int c1 = 6 - a - b - c0;
  i = o < 2 ? a : b;
  j = o < 2 ? b : a;
  k = (o & 1) ? c1 : c0;
  l = (o & 1) ? c0 : c1;
}

// Tree-level constants of the FP32 loop (FP64 in, FP32 out); *omega = eta^3 e^X
// e^{-i pi ap (t1 + t2) / 2} at tree level, the factor applied to the loop sum in FP64. The forward legs close with the two-step form of the point.
GRN_HD void make_nbody_loop_f(const grn_process_params &P, const Consts &K, const NBEvent &e,
                              int q, NBLoopF &f, cx<double> &omega) {
  const double a0 = P.regge.a0[q], ap = P.regge.ap[q], l0 = K.lns0;
  const double L = K.L, iL = 1.0 / L, iL2 = iL * iL, mp2 = K.mp2;
  const double ia1 = 1.0 / (1.0 - e.a1), ia2 = 1.0 / (1.0 - e.a2);
  const double mT1sq = mp2 + e.pt1sq, mT2sq = mp2 + e.pt2sq;
  const double c1 = mT1sq * iL2, c2 = mT2sq * iL2;
  const double r1 = 1.0 / (1.0 - (e.a1 + c2 * ia2)), r2 = 1.0 / (1.0 - (e.a2 + c1 * ia1));
  const double x1r = c2 * r2, x2r = c1 * r1, x1 = e.a1 + x1r, x2 = e.a2 + x2r;
  const LC4 p1{(1.0 - x1) * L, mT1sq * r1 * iL, e.p1x, e.p1y};
  const LC4 p2{mT2sq * r2 * iL, (1.0 - x2) * L, e.p2x, e.p2y};
  const LC4 g1{x1 * L, -(e.pt1sq + x1 * mp2) * r1 * iL, -e.p1x, -e.p1y};
  const LC4 g2{-(e.pt2sq + x2 * mp2) * r2 * iL, x2 * L, -e.p2x, -e.p2y};
  const double t1 = -(e.pt1sq + x1 * x1 * mp2) * r1, t2 = -(e.pt2sq + x2 * x2 * mp2) * r2;
  double x1a[kNb], x2a[kNb], d1[kNb], ljk[kNb][kNb], tab[kNbPairs], xt[kNbTerms];
  for (int a = 0; a < kNb; ++a) {
    f.c[a]  = {float(e.c[a].p), float(e.c[a].m), float(e.c[a].x), float(e.c[a].y)};
    f.m2[a] = float(e.m2[a]);
    const double s1 = mp2 + e.m2[a] + 2.0 * lc_dot(p1, e.c[a]);
    const double s2 = mp2 + e.m2[a] + 2.0 * lc_dot(p2, e.c[a]);
    f.is1[a] = float(1.0 / s1);
    f.is2[a] = float(1.0 / s2);
    const double l1 = log(s1) - l0, l2 = log(s2) - l0;
    f.l1[a] = float(l1);
    f.l2[a] = float(l2);
    x1a[a]  = (a0 + ap * t1) * l1;
    x2a[a]  = (a0 + ap * t2) * l2;
    d1[a]   = lc_dot(g1, e.c[a]);
    for (int b = 0; b < kNb; ++b) {
      ljk[a][b]   = b == a ? 0.0 : log(e.sbc[a][b]) - l0;
      f.ljk[a][b] = float(ljk[a][b]);
    }
  }
  double X = -1e300;
  for (int a = 0, p = 0; a < kNb; ++a)
    for (int b = a + 1; b < kNb; ++b, ++p) {
      tab[p]   = t1 + e.sbc[a][b] - 2.0 * (d1[a] + d1[b]);
      f.tab[p] = float(tab[p]);
      double sn, cs;
      sincos_pi(-0.5 * ap * tab[p], sn, cs);
      f.ph[p] = {float(cs), float(sn)};
      for (int o = 0; o < 4; ++o) {
        int i, j, k, l;
        nb_order(a, b, o, i, j, k, l);
        xt[4 * p + o] = x1a[i] + (a0 + ap * tab[p]) * ljk[j][k] + x2a[l];
        X = fmax(X, xt[4 * p + o]);
      }
    }
  for (int t = 0; t < kNbTerms; ++t) f.rho[t] = float(exp(xt[t] - X));
  f.p1x = float(e.p1x); f.p1y = float(e.p1y); f.p2x = float(e.p2x); f.p2y = float(e.p2y);
  f.a1 = float(e.a1); f.a2 = float(e.a2); f.ia1 = float(ia1); f.ia2 = float(ia2);
  f.L = float(L); f.invL = float(iL); f.invL2 = float(iL2); f.mp2 = float(mp2);
  f.x1r = float(x1r); f.x2r = float(x2r);
  f.p1m = float(p1.m); f.p2p = float(p2.p); f.g1m = float(g1.m); f.g2p = float(g2.p);
  f.t1 = float(t1); f.t2 = float(t2);
  f.a0 = float(a0); f.ap = float(ap);
  f.MA = float(K.m3sq); f.MB = float(K.M2propB); f.g2 = float(K.g2); f.gN2 = float(K.gN2);
  f.fc1 = float(P.soft.fc1); f.fc2 = float(P.soft.fc2);
  f.ffform = P.regge.offshellFF;
  f.bexp = float(P.regge.b_EXP); f.aore = float(P.regge.a_OREAR);
  f.bore = float(P.regge.b_OREAR); f.bpow = float(P.regge.b_POW);
  const cx<double> eta{K.eta0_re[q], K.eta0_im[q]};
  double sn, cs;
  sincos_pi(-0.5 * ap * (t1 + t2), sn, cs);
  omega = cscale(cmul(cmul(cmul(eta, eta), eta), cx<double>{cs, sn}), exp(X));
}

// ME6 / omega at one loop point (forward legs p1T - k, p2T + k) in FP32; false when the
// point is kinematically invalid or an invariant check fails (as nbody_amp). *mag = |vertex|
// sum over pairs of |f_ab| sum of the pair's four (positive) real ladder factors: the scale of
// the point's FP32 error, with the cancellation among the pairs' phases.
GRN_HD bool nbody_point_f(const grn_process_params &P, const Consts &K, const NBLoopF &f,
                          float kx, float ky, cx<float> &A, float &mag) {
  (void)P;
  (void)K;
  const float q1x = f.p1x - kx, q1y = f.p1y - ky, q2x = f.p2x + kx, q2y = f.p2y + ky;
  const float pt1sq = q1x * q1x + q1y * q1y, pt2sq = q2x * q2x + q2y * q2y;
  const float mT1sq = f.mp2 + pt1sq, mT2sq = f.mp2 + pt2sq;
  const float c1 = mT1sq * f.invL2, c2 = mT2sq * f.invL2;
  const float r1 = 1.f / (1.f - (f.a1 + c2 * f.ia2)), r2 = 1.f / (1.f - (f.a2 + c1 * f.ia1));
  const float x1r = c2 * r2, x2r = c1 * r1;
  const float x1 = f.a1 + x1r, x2 = f.a2 + x2r;
  if (!(x1 > 0.f && x2 > 0.f && x1 < 1.f && x2 < 1.f)) return false;
  // t = -(pT^2 + x^2 mp^2) r: its increment from pT'^2 - pT^2 = k^2 -+ 2 pT.k and
  // x - x0 = x1r - x1r0 (r - r0 = r r0 (x - x0)), exact where k -> 0
  const float dx1 = x1r - f.x1r, dx2 = x2r - f.x2r;
  const float k2 = kx * kx + ky * ky;
  const float dpt1 = k2 - 2.f * (f.p1x * kx + f.p1y * ky);
  const float dpt2 = k2 + 2.f * (f.p2x * kx + f.p2y * ky);
  const float dt1 = f.t1 * r1 * dx1 - (dpt1 + dx1 * (2.f * f.a1 + x1r + f.x1r) * f.mp2) * r1;
  const float dt2 = f.t2 * r2 * dx2 - (dpt2 + dx2 * (2.f * f.a2 + x2r + f.x2r) * f.mp2) * r2;
  const float t1 = f.t1 + dt1, t2 = f.t2 + dt2;
  if (t1 > 0.f || t2 > 0.f) return false;
  // increments of p1 = ((1 - x1) L, p1-, q1T), p2, q1 = (x1 L, q1-, -q1T), q2 over the tree
  // level; their transverse parts are -k, +k, +k, -k
  const float dx1L = dx1 * f.L, dx2L = dx2 * f.L;
  const float dp1m = mT1sq * r1 * f.invL - f.p1m, dp2p = mT2sq * r2 * f.invL - f.p2p;
  const float dg1m = -(pt1sq + x1 * f.mp2) * r1 * f.invL - f.g1m;
  const float dg2p = -(pt2sq + x2 * f.mp2) * r2 * f.invL - f.g2p;
  const float g1p = x1 * f.L, g1m = f.g1m + dg1m, g2m = x2 * f.L, g2p = f.g2p + dg2p;
  const float al1 = f.a0 + f.ap * t1, al2 = f.a0 + f.ap * t2;
  const float MA = f.MA, MB = f.MB;
  float e1[kNb], e2[kNb], f1[kNb], f2[kNb], dd1[kNb];
#pragma unroll
  for (int a = 0; a < kNb; ++a) {
    const LCT<float> &c  = f.c[a];
    const float       kc = kx * c.x + ky * c.y;
    // s / s0 - 1 = 2 (dp . c) / s0
    const float y1 = (-dx1L * c.m + dp1m * c.p + 2.f * kc) * f.is1[a];
    const float y2 = (dp2p * c.m - dx2L * c.p - 2.f * kc) * f.is2[a];
    if (!(y1 >= -1.f && y2 >= -1.f)) return false;
    e1[a]  = f.ap * dt1 * f.l1[a] + al1 * log1pf(y1);
    e2[a]  = f.ap * dt2 * f.l2[a] + al2 * log1pf(y2);
    dd1[a] = 0.5f * (dx1L * c.m + dg1m * c.p) - kc;
    const float d1 = 0.5f * (g1p * c.m + g1m * c.p) + q1x * c.x + q1y * c.y;
    const float d2 = 0.5f * (g2p * c.m + g2m * c.p) + q2x * c.x + q2y * c.y;
    const float ta = t1 + f.m2[a] - 2.f * d1, td = t2 + f.m2[a] - 2.f * d2;
    f1[a] = meson_ff_f(f, ta, MA) / (ta - MA);
    f2[a] = meson_ff_f(f, td, MB) / (td - MB);
  }
  cx<float> S{0.f, 0.f};
  float     M = 0.f;
#pragma unroll
  for (int a = 0, p = 0; a < kNb; ++a)
#pragma unroll
    for (int b = a + 1; b < kNb; ++b, ++p) {
      const float dtab = dt1 - 2.f * (dd1[a] + dd1[b]);
      const float tab  = f.tab[p] + dtab;
      const float fab  = meson_ff_f(f, tab, MA) * meson_ff_f(f, tab, MB);
      const float apd  = f.ap * dtab;
      float       Sp   = 0.f;
#pragma unroll
      for (int o = 0; o < 4; ++o) {
        int i, j, k, l;
        nb_order(a, b, o, i, j, k, l);
        Sp += f.rho[4 * p + o] * exp(e1[i] + apd * f.ljk[j][k] + e2[l]) * (f1[i] * f2[l]);
      }
      float sn, cs;
      sincos_pi(-0.5f * apd, sn, cs);
      const cx<float> ph = cmul(f.ph[p], cx<float>{cs, sn});
      S.re += fab * Sp * ph.re;
      S.im += fab * Sp * ph.im;
      M += fabsf(fab * Sp);
    }
  float sn, cs;
  sincos_pi(-0.5f * f.ap * (dt1 + dt2), sn, cs);
  const float vtx = f.gN2 * proton_ff<float>(f.fc1, f.fc2, t1) * proton_ff<float>(f.fc1, f.fc2, t2) *
                    f.g2 * f.g2;
  A   = cscale(cmul(S, cx<float>{cs, sn}), vtx);
  mag = M * fabsf(vtx);
  return true;
}

// FP32 loop integral with compensated sums (one trajectory); *mag: sum_ij |U_i c_j| mag_ij in
// units of the returned amplitude (see loop_integral for the summation part).
static __device__ cx<double> nbody_loop_f(const KArgs &A, const NBEvent &e,
                                          const KtNode<float> *skt, const PhiNode<float> *sphi,
                                          double *mag) {
  const int q = A.K.active[0] ? 0 : (A.K.active[1] ? 1 : 2);
  NBLoopF    f;
  cx<double> omega;
  make_nbody_loop_f(A.P, A.K, e, q, f, omega);
  float ar = 0.f, ai = 0.f, cr = 0.f, ci = 0.f, m = 0.f;
  for (int j = 0; j < A.n_kt_nodes; ++j) {
    const KtNode<float> nj = skt[j];
    float ir = 0.f, ii = 0.f, dr = 0.f, di = 0.f, ab = 0.f;
    for (int i = 0; i < A.n_phi_nodes; ++i) {
      const PhiNode<float> ni = sphi[i];
      cx<float> a;
      float     ma;
      if (!nbody_point_f(A.P, A.K, f, nj.kt * ni.c, nj.kt * ni.s, a, ma)) continue;
      kahan_add(ir, dr, ni.u * a.re);
      kahan_add(ii, di, ni.u * a.im);
      ab += ni.u * ma;
    }
    kahan_add(ar, cr, nj.cre * ir - nj.cim * ii);
    kahan_add(ai, ci, nj.cre * ii + nj.cim * ir);
    m += sqrtf(nj.cre * nj.cre + nj.cim * nj.cim) * ab;
  }
  const double om = sqrt(omega.re * omega.re + omega.im * omega.im);
  *mag = double(m) * om;
  const cx<double> s = cmul(omega, cx<double>{double(ar), double(ai)});
  return {A.loop_norm_re * s.re - A.loop_norm_im * s.im,
          A.loop_norm_re * s.im + A.loop_norm_im * s.re};
}

// Stage A of an N-body point: kinematics, cuts and (unscreened) the weight; true when the
// point needs the kt-loop. Flags as born_stage.
static __device__ __noinline__ bool nbody_born_stage(const KArgs &A, const double *x, double &W,
                                              uint8_t &flags) {
  NBEvent e;
  NBLegs  g;
  bool kin = nbody_kinematics(A.P, A.K, x, e);
  kin = kin && nbody_legs(A.K, e, e.p1x, e.p1y, e.p2x, e.p2y, g);
  cx<double> A0{0.0, 0.0};
  kin = kin && nbody_amp(A.P, A.K, e, g, A0);
  const bool fid  = kin && nbody_fiducial(A.P, e, g);
  const bool veto = !kin || !e.veto;
  flags = (kin ? GRN_FLAG_KINEMATICS_OK : 0) | (fid ? GRN_FLAG_FIDCUTS_OK : 0) |
          (veto ? GRN_FLAG_VETOCUTS_OK : 0) | GRN_FLAG_AMPLITUDE_OK;
  W = 0.0;
  if (!(kin && fid && veto)) return false;
  if (A.P.screening) return true;
  W = nbody_jacobian(A.K, e, g) * (A0.re * A0.re + A0.im * A0.im);
  if (!isfinite(W)) {
    W = 0.0;
    flags &= ~GRN_FLAG_AMPLITUDE_OK;
  }
  return false;
}

// Screened weight of an N-body point that passed stage A: T = double the FP64 loop; T = float
// the FP32 loop for one trajectory (the FP64 loop for several), and with refine non-null
// *refine tells whether its estimated relative error 2 kRefineKappa u |norm| mag / |A0 + A_loop|
// exceeds A.refine_tol (or is not finite): the caller then recomputes the point with T = double.
template <typename T>
__device__ __noinline__ double nbody_screened_weight(const KArgs &A, const double *x,
                                                     uint8_t &flags, const KtNode<T> *skt,
                                                     const PhiNode<T> *sphi,
                                                     bool *refine = nullptr) {
  NBEvent e;
  NBLegs  g;
  cx<double> A0{0.0, 0.0};
  nbody_kinematics(A.P, A.K, x, e);
  nbody_legs(A.K, e, e.p1x, e.p1y, e.p2x, e.p2y, g);
  nbody_amp(A.P, A.K, e, g, A0);
  cx<double> Al;
  bool       fp32 = false;
  if (refine) *refine = false;
  if constexpr (sizeof(T) == sizeof(float)) {
    if (A.K.n_active == 1 && e.n == kNb) {
      fp32        = true;
      double mag  = 0.0;
      Al = nbody_loop_f(A, e, skt, sphi, &mag);
      const double re = A0.re + Al.re, im = A0.im + Al.im;
      if (refine) {
        const double norm =
            sqrt(A.loop_norm_re * A.loop_norm_re + A.loop_norm_im * A.loop_norm_im);
        const double est = 2.0 * kRefineKappa * 0x1p-24 * norm * mag;
        *refine = A.refine_tol > 0.0 && !(est <= A.refine_tol * sqrt(re * re + im * im));
      }
    }
  }
  if (!fp32) Al = nbody_loop<T>(A, e, skt, sphi);
  const double re = A0.re + Al.re, im = A0.im + Al.im;
  double W = nbody_jacobian(A.K, e, g) * (re * re + im * im);
  flags = GRN_FLAG_KINEMATICS_OK | GRN_FLAG_FIDCUTS_OK | GRN_FLAG_VETOCUTS_OK |
          GRN_FLAG_AMPLITUDE_OK;
  if (!isfinite(W)) {
    W = 0.0;
    flags &= ~GRN_FLAG_AMPLITUDE_OK;
  }
  return W;
}

}  // namespace grn
