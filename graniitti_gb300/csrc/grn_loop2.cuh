// grn_loop2.cuh — the FP32 kt-loop of two events per thread on the packed FP32x2
// arithmetic of the sm_100 family (one instruction = two FP32 FMA / MUL / ADD).
//
// The arithmetic is that of loop_point_amp_fast (grn_physics.cuh) with lane x = event A
// and lane y = event B; both events run over the same loop grid, so the loop-node values
// come from shared memory as duplicated pairs {v, v} (one 64-bit load, no broadcast
// instructions). Transcendentals and the division stay per lane (MUFU). Sums are
// Kahan-compensated per lane, as in the scalar loop. This form tests every point for
// kinematic validity; the record-mode kernels run the azimuth-outer loop of grn_loop3.cuh
// and fall back to this one for events outside its validity bound.
#pragma once

#include <cuda_runtime.h>

#include "grn_physics.cuh"

namespace grn {

__device__ __forceinline__ float2 f2s(float a) { return make_float2(a, a); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
// a - b as one packed FMA: b * (-1) + a (exact product, single rounding like a subtraction)
__device__ __forceinline__ float2 sub2(float2 a, float2 b) {
  return __ffma2_rn(b, make_float2(-1.f, -1.f), a);
}

// Per-event fields of two events (the record fields) + per-engine constants as pairs.
struct LoopEvent2 {
#define GRN_F2_FIELD(f) float2 f;
  GRN_LOOP_EVENT_FIELDS(GRN_F2_FIELD)
#undef GRN_F2_FIELD
  float2 invL, invL2, mL, mp2, mM2, ap, mifc1, mifc2, ff_b, ff_a2, ff_ab, mhap;
  int    ffmode;
};

__device__ __forceinline__ void make_loop_event2(const LoopEventF<float> &a,
                                                 const LoopEventF<float> &b, LoopEvent2 &e) {
#define GRN_PAIR(f) e.f = make_float2(a.f, b.f);
  GRN_LOOP_EVENT_FIELDS(GRN_PAIR)
#undef GRN_PAIR
  e.invL   = f2s(a.invL);
  e.invL2  = f2s(a.invL2);
  e.mL     = f2s(-a.L);
  e.mp2    = f2s(a.mp2);
  e.mM2    = f2s(-a.M2);
  e.ap     = f2s(a.ap);
  e.mifc1  = f2s(-a.ifc1);
  e.mifc2  = f2s(-a.ifc2);
  e.ff_b   = f2s(a.ff_b);
  e.ff_a2  = f2s(a.ff_a2);
  e.ff_ab  = f2s(a.ff_ab);
  e.mhap   = f2s(-0.5f * a.ap);
  e.ffmode = a.ffmode;
}

// Two loop points (one per event) at the same loop momentum k = (kx, ky).
// ok: bit 0 = event A's point passed the kinematics, bit 1 = event B's.
__device__ __forceinline__ unsigned loop_point_amp2(const LoopEvent2 &e, float2 kx, float2 ky,
                                                    float2 k2, float2 &Are, float2 &Aim) {
  const float2 one = f2s(1.f), two = f2s(2.f), mtwo = f2s(-2.f), mone = f2s(-1.f);
  const float2 kd1  = fma2(kx, e.p1x, mul2(ky, e.p1y));
  const float2 kd2  = fma2(kx, e.p2x, mul2(ky, e.p2y));
  const float2 dm1  = fma2(mtwo, kd1, k2);
  const float2 dm2  = fma2(two, kd2, k2);
  const float2 dc1  = mul2(dm1, e.invL2), dc2 = mul2(dm2, e.invL2);
  const float2 dx1  = mul2(dc2, e.ia2), dx2 = mul2(dc1, e.ia1);
  const float2 dr1  = mul2(e.q1c, dc2), dr2 = mul2(e.q2c, dc1);
  const float2 r1   = add2(e.r10, dr1), r2 = add2(e.r20, dr2);
  const float2 dp1m = mul2(e.invL, fma2(dm1, r1, mul2(e.mT1s0, dr1)));
  const float2 dp2p = mul2(e.invL, fma2(dm2, r2, mul2(e.mT2s0, dr2)));
  const float2 dp1p = mul2(e.mL, dx1), dp2m = mul2(e.mL, dx2);
  const float2 k3   = fma2(kx, e.p3x, mul2(ky, e.p3y));
  const float2 k4   = fma2(kx, e.p4x, mul2(ky, e.p4y));
  const float2 ds13 = fma2(two, k3, fma2(dp1p, e.p3m, mul2(dp1m, e.p3p)));
  const float2 ds14 = fma2(two, k4, fma2(dp1p, e.p4m, mul2(dp1m, e.p4p)));
  const float2 ds23 = fma2(mtwo, k3, fma2(dp2p, e.p3m, mul2(dp2m, e.p3p)));
  const float2 ds24 = fma2(mtwo, k4, fma2(dp2p, e.p4m, mul2(dp2m, e.p4p)));
  const float2 y13  = fma2(ds13, e.is13, one), y14 = fma2(ds14, e.is14, one);
  const float2 y23  = fma2(ds23, e.is23, one), y24 = fma2(ds24, e.is24, one);
  const float2 d13  = make_float2(fast_log2(y13.x), fast_log2(y13.y));
  const float2 d14  = make_float2(fast_log2(y14.x), fast_log2(y14.y));
  const float2 d23  = make_float2(fast_log2(y23.x), fast_log2(y23.y));
  const float2 d24  = make_float2(fast_log2(y24.x), fast_log2(y24.y));
  // dt = -(dm + dx (2 x0 + dx) mp2) r - Tn0 dr
  const float2 h1  = fma2(mul2(dx1, fma2(two, e.x10, dx1)), e.mp2, dm1);
  const float2 h2  = fma2(mul2(dx2, fma2(two, e.x20, dx2)), e.mp2, dm2);
  const float2 dt1 = mul2(mone, fma2(h1, r1, mul2(e.T1n0, dr1)));
  const float2 dt2 = mul2(mone, fma2(h2, r2, mul2(e.T2n0, dr2)));
  const float2 t1  = add2(e.t10, dt1), t2 = add2(e.t20, dt2);
  const float2 dEt = fma2(e.ap, fma2(dt1, add2(e.L13, d13), mul2(dt2, add2(e.L24, d24))),
                          fma2(e.a10, d13, mul2(e.a20, d24)));
  const float2 dEu = fma2(e.ap, fma2(dt1, add2(e.L14, d14), mul2(dt2, add2(e.L23, d23))),
                          fma2(e.a10, d14, mul2(e.a20, d23)));
  // t_hat - M2 and u_hat - M2
  const float2 cx3 = sub2(e.c3x, kx), cy3 = sub2(e.c3y, ky);
  const float2 cx4 = sub2(e.c4x, kx), cy4 = sub2(e.c4y, ky);
  const float2 ta  = sub2(fma2(add2(e.dpa0, dp2p), sub2(e.dma0, dp1m), e.mM2),
                         fma2(cx3, cx3, mul2(cy3, cy3)));
  const float2 tb  = sub2(fma2(add2(e.dpb0, dp2p), sub2(e.dmb0, dp1m), e.mM2),
                         fma2(cx4, cx4, mul2(cy4, cy4)));
  const float2 Pd  = mul2(mul2(fma2(t1, e.mifc1, one), fma2(t1, e.mifc2, one)),
                         mul2(fma2(t2, e.mifc1, one), fma2(t2, e.mifc2, one)));
  float2 num, den;
  if (e.ffmode == 2) {
    const float2 Da = sub2(e.ff_b, ta), Db = sub2(e.ff_b, tb);
    const float2 Da2 = mul2(Da, Da), Db2 = mul2(Db, Db);
    const float2 Xt  = mul2(e.rho_t, make_float2(fast_exp2(dEt.x), fast_exp2(dEt.y)));
    const float2 Xu  = mul2(e.rho_u, make_float2(fast_exp2(dEu.x), fast_exp2(dEu.y)));
    num = fma2(mul2(Xt, Db2), tb, mul2(mul2(Xu, Da2), ta));
    den = mul2(mul2(Pd, mul2(Da2, Db2)), mul2(ta, tb));
  } else {
    float2 fa, fb;  // 2 log2 of the off-shell form factors
    if (e.ffmode == 0) {
      const float c = float(-2.0 * kLog2e);
      fa = make_float2(c * e.ff_b.x * fabsf(ta.x), c * e.ff_b.y * fabsf(ta.y));
      fb = make_float2(c * e.ff_b.x * fabsf(tb.x), c * e.ff_b.y * fabsf(tb.y));
    } else {
      const float c = float(2.0 * kLog2e);
      fa = make_float2(c * (e.ff_ab.x - e.ff_b.x * sqrtf(fabsf(ta.x) + e.ff_a2.x)),
                       c * (e.ff_ab.y - e.ff_b.y * sqrtf(fabsf(ta.y) + e.ff_a2.y)));
      fb = make_float2(c * (e.ff_ab.x - e.ff_b.x * sqrtf(fabsf(tb.x) + e.ff_a2.x)),
                       c * (e.ff_ab.y - e.ff_b.y * sqrtf(fabsf(tb.y) + e.ff_a2.y)));
    }
    const float2 xt = add2(dEt, sub2(fa, e.fa0)), xu = add2(dEu, sub2(fb, e.fb0));
    const float2 Xt = mul2(e.rho_t, make_float2(fast_exp2(xt.x), fast_exp2(xt.y)));
    const float2 Xu = mul2(e.rho_u, make_float2(fast_exp2(xu.x), fast_exp2(xu.y)));
    num = fma2(Xt, tb, mul2(Xu, ta));
    den = mul2(Pd, mul2(ta, tb));
  }
  const float2 ph = mul2(e.mhap, add2(dt1, dt2));
  float2       sn, cs;
  fast_sincos_pi(ph.x, sn.x, cs.x);
  fast_sincos_pi(ph.y, sn.y, cs.y);
  const float2 m = make_float2(fast_div(num.x, den.x), fast_div(num.y, den.y));
  Are = mul2(sub2(mul2(e.pre_re, cs), mul2(e.pre_im, sn)), m);
  Aim = mul2(fma2(e.pre_re, sn, mul2(e.pre_im, cs)), m);
  const float2 x1 = add2(e.x10, dx1), x2 = add2(e.x20, dx2);
  return ((x1.x < 1.f && x2.x < 1.f) ? 1u : 0u) | ((x1.y < 1.f && x2.y < 1.f) ? 2u : 0u);
}

__device__ __forceinline__ void kahan_add2(float2 &sum, float2 &comp, float2 x) {
  const float2 y = sub2(x, comp);
  const float2 t = add2(sum, y);
  comp           = sub2(sub2(t, sum), y);
  sum            = t;
}

// Loop integrals of both events (relative to their exp(Emax)): lane x event A, y event B.
// Every point is tested for kinematic validity. KN, PN: node types with the fields kt, k2,
// cre, cim and c, s, u.
template <typename KN, typename PN>
__device__ __forceinline__ void loop_integral2(const LoopEvent2 &e, int n_kt, int n_phi,
                                               const KN *skt, const PN *sphi,
                                               float2 &out_re, float2 &out_im,
                                               float2 &out_mag) {
  const float2 zero = f2s(0.f);
  float2 ar = zero, ai = zero, cr = zero, ci = zero, am = zero;
  for (int j = 0; j < n_kt; ++j) {
    const KN nj = skt[j];
    float2 ir = zero, ii = zero, dr = zero, di = zero, im = zero;
    for (int i = 0; i < n_phi; ++i) {
      const PN ni = sphi[i];
      float2 are, aim;
      const unsigned ok = loop_point_amp2(e, mul2(nj.kt, ni.c), mul2(nj.kt, ni.s), nj.k2, are, aim);
      float2 xr = mul2(ni.u, are), xi = mul2(ni.u, aim);
      if (!(ok & 1u)) xr.x = xi.x = 0.f;
      if (!(ok & 2u)) xr.y = xi.y = 0.f;
      kahan_add2(ir, dr, xr);
      kahan_add2(ii, di, xi);
      im = add2(im, add2(make_float2(fabsf(xr.x), fabsf(xr.y)),
                         make_float2(fabsf(xi.x), fabsf(xi.y))));
    }
    kahan_add2(ar, cr, sub2(mul2(nj.cre, ir), mul2(nj.cim, ii)));
    kahan_add2(ai, ci, fma2(nj.cre, ii, mul2(nj.cim, ir)));
    am = fma2(nj.cabs, im, am);
  }
  out_re  = ar;
  out_im  = ai;
  out_mag = am;
}

}  // namespace grn
