// grn_loop3.cuh — the record-mode FP32 kt-loop of two events per thread, azimuth-outer form.
//
// Arithmetic of loop_point_amp_fast (grn_physics.cuh: every loop-point quantity as its tree-
// level value plus an explicit increment in the loop momentum k) rearranged for the loop
// order phi outer, kt inner, on packed FP32x2 pairs (lane x event A, lane y event B):
//  * the projections of the event's transverse vectors on the direction (cos phi, sin phi)
//    are formed once per phi node, so k.p = kt (n.p) costs one product inside the kt loop;
//  * |p1T + p3T - k|^2 = (|c3| - kt)^2 + 4 |c3| kt sin^2((phi - phi_c3) / 2): a sum of non-
//    negative terms (no cancellation where k is close to c3), the sine once per phi node;
//  * the couplings x ReggeEta^2 x tree-level phase (a constant of the event) multiply the
//    loop sum once, after it;
//  * signs folded into constants (no multiplication by -1), the proton form-factor product
//    (1 - t/fc1)(1 - t/fc2) as a quadratic in t;
//  * the kinematic validity test of a point (x1, x2 < 1) replaced by a bound per event: the
//    loop moves x by at most (2 kt_max |pT| + kt_max^2) (1 - a)^-1 / L^2 ~ 1e-7, so an event
//    whose tree-level x plus that bound stays below 1 has no invalid point (events outside
//    the bound run the per-point-tested loop_integral2 of grn_loop2.cuh);
//  * sums compensated per block of 8 kt nodes (plain within a block, Kahan across blocks
//    and across phi rings).
// The core is a template on the pair type V so that the same source is instantiated with a
// counting arithmetic on the host (flopcount.cc): the algorithmic work of the timed kernel is
// counted on the function it runs.
#pragma once

#ifdef __CUDACC__
#include "grn_loop2.cuh"
#define GRN_L3 __device__ __forceinline__
#else
#include "grn_physics.cuh"
#define GRN_L3 inline
#endif

namespace grn {

// A pair with both lanes a (specialised per pair type).
template <typename V>
GRN_L3 V splat(float a);

#ifdef __CUDACC__
template <>
__device__ __forceinline__ float2 splat<float2>(float a) {
  return make_float2(a, a);
}
// Lane-wise operations of the float2 pairs (per lane: the special-function unit, or one FP32
// instruction of the lane).
__device__ __forceinline__ float2 log2_2(float2 a) {
  return make_float2(fast_log2(a.x), fast_log2(a.y));
}
__device__ __forceinline__ float2 exp2_2(float2 a) {
  return make_float2(fast_exp2(a.x), fast_exp2(a.y));
}
// a / b per lane: the SFU's reciprocal of each lane, then one packed multiplication
__device__ __forceinline__ float2 div2(float2 a, float2 b) {
  float rx, ry;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(rx) : "f"(b.x));
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(ry) : "f"(b.y));
  return __fmul2_rn(a, make_float2(rx, ry));
}
__device__ __forceinline__ float2 abs2(float2 a) { return make_float2(fabsf(a.x), fabsf(a.y)); }
__device__ __forceinline__ float2 sqrt2(float2 a) { return make_float2(sqrtf(a.x), sqrtf(a.y)); }
// (sin 2 pi h, cos 2 pi h): h reduced to [-1/2, 1/2] turns, then the hardware sine / cosine
// (absolute error ~5e-7 on |2 pi h| <= pi).
__device__ __forceinline__ void sincos_turns2(float2 h, float2 &s, float2 &c) {
  // the nearest integers to h (|h| < 2^22): h + 1.5 2^23 has no fraction bits left, and
  // subtracting 1.5 2^23 back is exact (packed round-to-nearest additions)
  const float2 big = make_float2(12582912.f, 12582912.f);
  const float2 n   = __fadd2_rn(__fadd2_rn(h, big), make_float2(-12582912.f, -12582912.f));
  const float2 a   = __fmul2_rn(make_float2(float(2.0 * kPi), float(2.0 * kPi)),
                                __ffma2_rn(n, make_float2(-1.f, -1.f), h));
  sfu_sincos(a.x, s.x, c.x);
  sfu_sincos(a.y, s.y, c.y);
}
// sin(pi d) for |d| < 1 (accurate: the once-per-phi-node projections).
__device__ __forceinline__ float2 sinpi_turns2(float2 d) {
  return make_float2(sinpif(d.x), sinpif(d.y));
}

// Loop nodes of the azimuth-outer loop, duplicated pairs: kt nodes (kt, kt^2, c_j, -Im c_j,
// |c_j|), phi nodes (cos, sin, U, phi in turns).
struct KtNode3 {
  float2 kt, k2, cre, cim, ncim, cabs;
};
struct PhiNode3 {
  float2 c, s, u, t;
};
#endif

// Per-pair constants of the azimuth-outer loop (V = float2 on the device).
template <typename V>
struct Loop3 {
  // per event (lanes x, y)
  V p1x, p1y, p2x, p2y, p3x, p3y, p4x, p4y;  // tree-level transverse momenta
  V kx1, kx2, kr1, kr2;                       // dx1 = dm2 kx1, dx2 = dm1 kx2, dr1 = dm2 kr1, ...
  V r10, r20, mT1s0, mT2s0, T1n0, T2n0, t10, t20;
  V p3p, p3m, p4p, p4m, is13, is14, is23, is24;
  V a10, a20, mapL13, mapL14, mapL23, mapL24;
  V dpa0, dma0, dpb0, dmb0;
  V c3m, c4m, phc3, phc4, nM2;                // |c3|, |c4|, their azimuths / (2 pi), -M^2
  V tx10mp2, tx20mp2;                         // 2 x1 mp^2, 2 x2 mp^2 (tree level)
  V fa0, fb0, rho_t, rho_u;
  // per engine (equal lanes)
  V invL, mL, mp2, map, hap, s12, m12, ff_b, ff_a2, ff_ab;
  int ffmode;
};

// Everything of one phi node that does not depend on kt.
template <typename V>
struct Phi3 {
  V m2D1, t2D2, t2D3, m2D3, t2D4, m2D4, W3, W4;
};

// The loop-point amplitude relative to the event's constant prefactor and exp(Emax):
// (cs m, sn m) with m the Regge magnitude and (cs, sn) the Regge phase of the point.
template <typename V>
GRN_L3 void loop_point3(const Loop3<V> &e, const Phi3<V> &f, V kt, V k2, V &zr, V &zi) {
  const V one = splat<V>(1.f), two = splat<V>(2.f);
  const V dm1 = fma2(kt, f.m2D1, k2);  // pT1'^2 - pT1^2 = -2 k.p1 + k^2
  const V dm2 = fma2(kt, f.t2D2, k2);  // pT2'^2 - pT2^2 =  2 k.p2 + k^2
  const V dx1 = mul2(dm2, e.kx1), dx2 = mul2(dm1, e.kx2);
  const V dr1 = mul2(dm2, e.kr1), dr2 = mul2(dm1, e.kr2);
  const V r1 = add2(e.r10, dr1), r2 = add2(e.r20, dr2);
  const V dp1m = mul2(e.invL, fma2(dm1, r1, mul2(e.mT1s0, dr1)));
  const V dp2p = mul2(e.invL, fma2(dm2, r2, mul2(e.mT2s0, dr2)));
  const V dp1p = mul2(e.mL, dx1), dp2m = mul2(e.mL, dx2);
  const V ds13 = fma2(kt, f.t2D3, fma2(dp1p, e.p3m, mul2(dp1m, e.p3p)));
  const V ds14 = fma2(kt, f.t2D4, fma2(dp1p, e.p4m, mul2(dp1m, e.p4p)));
  const V ds23 = fma2(kt, f.m2D3, fma2(dp2p, e.p3m, mul2(dp2m, e.p3p)));
  const V ds24 = fma2(kt, f.m2D4, fma2(dp2p, e.p4m, mul2(dp2m, e.p4p)));
  const V d13 = log2_2(fma2(ds13, e.is13, one)), d14 = log2_2(fma2(ds14, e.is14, one));
  const V d23 = log2_2(fma2(ds23, e.is23, one)), d24 = log2_2(fma2(ds24, e.is24, one));
  // -dt = h r + Tn0 dr with h = dm + mp^2 dx (2 x0 + dx)
  const V h1   = fma2(dx1, fma2(dx1, e.mp2, e.tx10mp2), dm1);
  const V h2   = fma2(dx2, fma2(dx2, e.mp2, e.tx20mp2), dm2);
  const V ndt1 = fma2(h1, r1, mul2(e.T1n0, dr1));
  const V ndt2 = fma2(h2, r2, mul2(e.T2n0, dr2));
  const V t1 = sub2(e.t10, ndt1), t2 = sub2(e.t20, ndt2);
  // Regge exponents (log2 units): alpha(t') ln(s'/s0) - alpha(t) ln(s/s0)
  const V A1  = fma2(ndt1, e.map, e.a10), A2 = fma2(ndt2, e.map, e.a20);
  const V dEt = fma2(d13, A1, fma2(d24, A2, fma2(ndt1, e.mapL13, mul2(ndt2, e.mapL24))));
  const V dEu = fma2(d14, A1, fma2(d23, A2, fma2(ndt1, e.mapL14, mul2(ndt2, e.mapL23))));
  // t_hat - M^2 and u_hat - M^2: light-cone part minus |c - k|^2
  const V d3 = sub2(e.c3m, kt), d4 = sub2(e.c4m, kt);
  const V ta = fma2(add2(e.dpa0, dp2p), sub2(e.dma0, dp1m),
                    sub2(e.nM2, fma2(d3, d3, mul2(kt, f.W3))));
  const V tb = fma2(add2(e.dpb0, dp2p), sub2(e.dmb0, dp1m),
                    sub2(e.nM2, fma2(d4, d4, mul2(kt, f.W4))));
  // proton form factors (1 - t/fc1)(1 - t/fc2) = 1 + t (s12 + t m12)
  const V Pd = mul2(fma2(t1, fma2(t1, e.m12, e.s12), one), fma2(t2, fma2(t2, e.m12, e.s12), one));
  V num, den;
  if (e.ffmode == 2) {
    const V Da = sub2(e.ff_b, ta), Db = sub2(e.ff_b, tb);
    const V Da2 = mul2(Da, Da), Db2 = mul2(Db, Db);
    const V Xt = mul2(e.rho_t, exp2_2(dEt)), Xu = mul2(e.rho_u, exp2_2(dEu));
    num = fma2(mul2(Xt, Db2), tb, mul2(mul2(Xu, Da2), ta));
    den = mul2(mul2(Pd, mul2(Da2, Db2)), mul2(ta, tb));
  } else {
    V fa, fb;  // 2 log2 of the off-shell form factors
    if (e.ffmode == 0) {
      fa = mul2(e.ff_b, abs2(ta));  // ff_b = -2 b log2(e) here
      fb = mul2(e.ff_b, abs2(tb));
    } else {
      fa = fma2(e.ff_b, sqrt2(add2(abs2(ta), e.ff_a2)), e.ff_ab);
      fb = fma2(e.ff_b, sqrt2(add2(abs2(tb), e.ff_a2)), e.ff_ab);
    }
    const V Xt = mul2(e.rho_t, exp2_2(add2(dEt, sub2(fa, e.fa0))));
    const V Xu = mul2(e.rho_u, exp2_2(add2(dEu, sub2(fb, e.fb0))));
    num = fma2(Xt, tb, mul2(Xu, ta));
    den = mul2(Pd, mul2(ta, tb));
  }
  // Regge phase exp(-i pi ap (t'1 + t'2 - t1 - t2) / 2) = exp(i pi hap (ndt1 + ndt2))
  V sn, cs;
  sincos_turns2(mul2(e.hap, add2(ndt1, ndt2)), sn, cs);
  const V m = div2(num, den);
  zr = mul2(cs, m);
  zi = mul2(sn, m);
}

template <typename V>
GRN_L3 void kahan_add3(V &sum, V &comp, V x) {
  const V y = sub2(x, comp);
  const V t = add2(sum, y);
  comp      = sub2(sub2(t, sum), y);
  sum       = t;
}

// Loop integral sum_i U_i sum_j c_j z_ij of both events (relative to their prefactors and
// exp(Emax)); kt nodes (kt, kt^2, Re c, Im c, -Im c, |c|), phi nodes (cos, sin, U, phi / (2 pi)).
// out_mag = sum_i U_i sum_j |c_j| (|Re z_ij| + |Im z_ij|), the scale of its rounding error.
template <typename V, typename KN, typename PN>
GRN_L3 void loop_integral3(const Loop3<V> &e, int n_kt, int n_phi, const KN *skt,
                           const PN *sphi, V &out_re, V &out_im, V &out_mag) {
  const V zero = splat<V>(0.f);
  V ar = zero, ai = zero, cr = zero, ci = zero, am = zero;
  for (int i = 0; i < n_phi; ++i) {
    const PN ni = sphi[i];
    Phi3<V> f;
    {
      const V D1 = fma2(ni.c, e.p1x, mul2(ni.s, e.p1y)), D2 = fma2(ni.c, e.p2x, mul2(ni.s, e.p2y));
      const V D3 = fma2(ni.c, e.p3x, mul2(ni.s, e.p3y)), D4 = fma2(ni.c, e.p4x, mul2(ni.s, e.p4y));
      const V mtwo = splat<V>(-2.f), two = splat<V>(2.f);
      f.m2D1 = mul2(mtwo, D1);
      f.t2D2 = mul2(two, D2);
      f.t2D3 = mul2(two, D3);
      f.m2D3 = mul2(mtwo, D3);
      f.t2D4 = mul2(two, D4);
      f.m2D4 = mul2(mtwo, D4);
      // 4 |c| sin^2((phi - phi_c) / 2): sine of half the angle in turns
      const V s3 = sinpi_turns2(sub2(ni.t, e.phc3)), s4 = sinpi_turns2(sub2(ni.t, e.phc4));
      const V four = splat<V>(4.f);
      f.W3 = mul2(mul2(four, e.c3m), mul2(s3, s3));
      f.W4 = mul2(mul2(four, e.c4m), mul2(s4, s4));
    }
    V rr = zero, ri = zero, qr = zero, qi = zero;  // the ring over kt, compensated per block
    V rm = zero;
    for (int j0 = 0; j0 < n_kt; j0 += 8) {
      V br = zero, bi = zero;
      const int j1 = j0 + 8 < n_kt ? j0 + 8 : n_kt;
#pragma unroll 2
      for (int j = j0; j < j1; ++j) {
        const KN nj = skt[j];
        V zr, zi;
        loop_point3(e, f, nj.kt, nj.k2, zr, zi);
        br = fma2(nj.cre, zr, fma2(nj.ncim, zi, br));
        bi = fma2(nj.cre, zi, fma2(nj.cim, zr, bi));
        rm = fma2(nj.cabs, add2(abs2(zr), abs2(zi)), rm);
      }
      kahan_add3(rr, qr, br);
      kahan_add3(ri, qi, bi);
    }
    kahan_add3(ar, cr, mul2(ni.u, rr));
    kahan_add3(ai, ci, mul2(ni.u, ri));
    am = fma2(ni.u, rm, am);
  }
  out_re  = ar;
  out_im  = ai;
  out_mag = am;
}

// The per-pair constants from two loaded records (scalar LoopEventF of events a and b) and
// the engine constants in a; pair(x, y) builds a V from two lane values.
template <typename V, typename S, typename PAIR>
GRN_L3 void make_loop3(const LoopEventF<S> &a, const LoopEventF<S> &b, PAIR pair, Loop3<V> &e) {
#define GRN_P2(dst, expr_a, expr_b) e.dst = pair(expr_a, expr_b);
  GRN_P2(p1x, a.p1x, b.p1x) GRN_P2(p1y, a.p1y, b.p1y) GRN_P2(p2x, a.p2x, b.p2x)
  GRN_P2(p2y, a.p2y, b.p2y) GRN_P2(p3x, a.p3x, b.p3x) GRN_P2(p3y, a.p3y, b.p3y)
  GRN_P2(p4x, a.p4x, b.p4x) GRN_P2(p4y, a.p4y, b.p4y)
  GRN_P2(kx1, a.invL2 * a.ia2, b.invL2 * b.ia2) GRN_P2(kx2, a.invL2 * a.ia1, b.invL2 * b.ia1)
  GRN_P2(kr1, a.q1c * a.invL2, b.q1c * b.invL2) GRN_P2(kr2, a.q2c * a.invL2, b.q2c * b.invL2)
  GRN_P2(r10, a.r10, b.r10) GRN_P2(r20, a.r20, b.r20) GRN_P2(mT1s0, a.mT1s0, b.mT1s0)
  GRN_P2(mT2s0, a.mT2s0, b.mT2s0) GRN_P2(T1n0, a.T1n0, b.T1n0) GRN_P2(T2n0, a.T2n0, b.T2n0)
  GRN_P2(t10, a.t10, b.t10) GRN_P2(t20, a.t20, b.t20)
  GRN_P2(p3p, a.p3p, b.p3p) GRN_P2(p3m, a.p3m, b.p3m) GRN_P2(p4p, a.p4p, b.p4p)
  GRN_P2(p4m, a.p4m, b.p4m) GRN_P2(is13, a.is13, b.is13) GRN_P2(is14, a.is14, b.is14)
  GRN_P2(is23, a.is23, b.is23) GRN_P2(is24, a.is24, b.is24)
  GRN_P2(a10, a.a10, b.a10) GRN_P2(a20, a.a20, b.a20)
  GRN_P2(mapL13, -a.ap * a.L13, -b.ap * b.L13) GRN_P2(mapL14, -a.ap * a.L14, -b.ap * b.L14)
  GRN_P2(mapL23, -a.ap * a.L23, -b.ap * b.L23) GRN_P2(mapL24, -a.ap * a.L24, -b.ap * b.L24)
  GRN_P2(dpa0, a.dpa0, b.dpa0) GRN_P2(dma0, a.dma0, b.dma0) GRN_P2(dpb0, a.dpb0, b.dpb0)
  GRN_P2(dmb0, a.dmb0, b.dmb0)
  GRN_P2(c3m, sqrt(a.c3x * a.c3x + a.c3y * a.c3y), sqrt(b.c3x * b.c3x + b.c3y * b.c3y))
  GRN_P2(c4m, sqrt(a.c4x * a.c4x + a.c4y * a.c4y), sqrt(b.c4x * b.c4x + b.c4y * b.c4y))
  GRN_P2(phc3, atan2(a.c3y, a.c3x) * S(0.5 / kPi), atan2(b.c3y, b.c3x) * S(0.5 / kPi))
  GRN_P2(phc4, atan2(a.c4y, a.c4x) * S(0.5 / kPi), atan2(b.c4y, b.c4x) * S(0.5 / kPi))
  GRN_P2(nM2, -a.M2, -b.M2)
  GRN_P2(tx10mp2, S(2) * a.x10 * a.mp2, S(2) * b.x10 * b.mp2)
  GRN_P2(tx20mp2, S(2) * a.x20 * a.mp2, S(2) * b.x20 * b.mp2)
  GRN_P2(fa0, a.fa0, b.fa0) GRN_P2(fb0, a.fb0, b.fb0) GRN_P2(rho_t, a.rho_t, b.rho_t)
  GRN_P2(rho_u, a.rho_u, b.rho_u)
  GRN_P2(invL, a.invL, b.invL) GRN_P2(mL, -a.L, -b.L) GRN_P2(mp2, a.mp2, b.mp2)
  GRN_P2(map, -a.ap, -b.ap) GRN_P2(hap, S(0.25) * a.ap, S(0.25) * b.ap)
  GRN_P2(s12, -(a.ifc1 + a.ifc2), -(b.ifc1 + b.ifc2))
  GRN_P2(m12, a.ifc1 * a.ifc2, b.ifc1 * b.ifc2)
  GRN_P2(ff_a2, a.ff_a2, b.ff_a2)
#undef GRN_P2
  e.ffmode = a.ffmode;
  // off-shell form factor constants: power law b; exponential -2 b log2(e) (times |t|);
  // Orear 2 log2(e) (a b - b sqrt(|t| + a^2)) = ff_b sqrt(...) + ff_ab
  const S c = S(2.0 * kLog2e);
  if (a.ffmode == 2) {
    e.ff_b  = pair(a.ff_b, b.ff_b);
    e.ff_ab = pair(a.ff_ab, b.ff_ab);
  } else if (a.ffmode == 0) {
    e.ff_b  = pair(-c * a.ff_b, -c * b.ff_b);
    e.ff_ab = pair(S(0), S(0));
  } else {
    e.ff_b  = pair(-c * a.ff_b, -c * b.ff_b);
    e.ff_ab = pair(c * a.ff_ab, c * b.ff_ab);
  }
}

// The loop leaves x1, x2 below 1 at every point of an event when its tree-level x plus the
// largest increment, (2 kt_max |pT| + kt_max^2) / ((1 - a) L^2), stays below 1.
template <typename S>
GRN_L3 bool loop3_safe(const LoopEventF<S> &a, S kt_max) {
  const S p1 = sqrt(a.p1x * a.p1x + a.p1y * a.p1y), p2 = sqrt(a.p2x * a.p2x + a.p2y * a.p2y);
  const S d1 = (S(2) * kt_max * p2 + kt_max * kt_max) * a.invL2 * a.ia2;
  const S d2 = (S(2) * kt_max * p1 + kt_max * kt_max) * a.invL2 * a.ia1;
  return a.x10 + S(2) * d1 < S(1) && a.x20 + S(2) * d2 < S(1);
}

}  // namespace grn
