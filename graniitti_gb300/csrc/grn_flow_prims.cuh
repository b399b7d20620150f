// grn_flow_prims.cuh — device primitives shared by the flow kernels (grn_flow.cu,
// grn_flow_wide.cu): warp-level BF16 mma.sync fragments, the FP32 rational-quadratic
// spline and its gradient, and the tcgen05 / bulk-copy / mbarrier wrappers.
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "grn_flow.cuh"

namespace grn {
namespace flow {

using bf16 = __nv_bfloat16;

constexpr float kMinW = 1e-3f, kMinH = 1e-3f, kMinD = 1e-3f;
constexpr int kRawF = 64;  // TMEM / forward-operand columns per transformed coordinate
constexpr int kSpinLimit = 1 << 22;  // polls of a bounded mbarrier wait

// ---------------------------------------------------------------------------
// Tensor-core primitives (warp-level BF16 m16n8k16, FP32 accumulate).

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void ldsm4(uint32_t (&r)[4], const void *p) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(smem_u32(p)));
}

__device__ __forceinline__ void ldsm4t(uint32_t (&r)[4], const void *p) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(smem_u32(p)));
}

__device__ __forceinline__ void ldsm2t(uint32_t &r0, uint32_t &r1, const void *p) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x2.trans.shared.b16 {%0,%1}, [%2];\n"
               : "=r"(r0), "=r"(r1)
               : "r"(smem_u32(p)));
}

__device__ __forceinline__ void ldsm2(uint32_t &r0, uint32_t &r1, const void *p) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x2.shared.b16 {%0,%1}, [%2];\n"
               : "=r"(r0), "=r"(r1)
               : "r"(smem_u32(p)));
}

__device__ __forceinline__ void mma16816(float (&c)[4], const uint32_t (&a)[4], uint32_t b0,
                                         uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, "
      "{%8,%9}, {%0,%1,%2,%3};\n"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// Fragment addresses for lane l (m16n8k16 operand layouts):
//   A[m][k] row-major (k contiguous):         row m0 + (l & 15), col k0 + (l >> 4) * 8
//   A from S[k][m] (m contiguous), .trans:    row k0 + (l & 7) + (l >> 4) * 8,
//                                             col m0 + ((l >> 3) & 1) * 8
//   B from S[k][n] (n contiguous), .trans:    row k0 + (l & 15), col n0 + (l >> 4) * 8
//                                             (two n-tiles: regs {0,1} tile 0, {2,3} tile 1)
//   B from S[n][k] (k contiguous):            row n0 + (l & 7) + (l >> 4) * 8,
//                                             col k0 + ((l >> 3) & 1) * 8
// Accumulator: c0, c1 at (row g, cols 2t, 2t+1); c2, c3 at (row g + 8, same cols),
// g = l >> 2, t = l & 3.

__device__ __forceinline__ uint32_t pack_bf2(float a, float b) {
  const __nv_bfloat162 v = __floats2bfloat162_rn(a, b);
  return *reinterpret_cast<const uint32_t *>(&v);
}

__device__ __forceinline__ float bfr(float x) { return __bfloat162float(__float2bfloat16_rn(x)); }

// ---------------------------------------------------------------------------
// Spline (FP32). rp points to one thread-owned row of 3K+1 raw outputs.

__device__ __forceinline__ float softplusf(float r) {
  return r > 15.f ? r + log1pf(expf(-r)) : log1pf(expf(r));
}

// In place: rp[0..K) <- bin widths, rp[K..2K) <- bin heights (softmax with floor).
__device__ __forceinline__ void spline_normalize(float *rp) {
  float mw = rp[0], mh = rp[kBins];
#pragma unroll
  for (int k = 1; k < kBins; ++k) {
    mw = fmaxf(mw, rp[k]);
    mh = fmaxf(mh, rp[kBins + k]);
  }
  float sw = 0.f, sh = 0.f;
#pragma unroll
  for (int k = 0; k < kBins; ++k) {
    const float a = __expf(rp[k] - mw), b = __expf(rp[kBins + k] - mh);
    rp[k]         = a;
    rp[kBins + k] = b;
    sw += a;
    sh += b;
  }
  const float cw = (1.f - kBins * kMinW) / sw, ch = (1.f - kBins * kMinH) / sh;
#pragma unroll
  for (int k = 0; k < kBins; ++k) {
    rp[k]         = kMinW + cw * rp[k];
    rp[kBins + k] = kMinH + ch * rp[kBins + k];
  }
}

struct Bin {
  int   k;
  float xk, w, yk, h, d0, d1;
};

// Bin of x on the x knots (by = false) or of y on the y knots (by = true).
__device__ __forceinline__ Bin spline_bin(const float *rp, float v, bool by) {
  Bin   b;
  float xk = 0.f, yk = 0.f;
  int   k  = 0;
  for (; k < kBins - 1; ++k) {
    const float step = by ? rp[kBins + k] : rp[k];
    if (v < (by ? yk : xk) + step) break;
    xk += rp[k];
    yk += rp[kBins + k];
  }
  b.k  = k;
  b.xk = xk;
  b.yk = yk;
  b.w  = (k == kBins - 1) ? 1.f - xk : rp[k];
  b.h  = (k == kBins - 1) ? 1.f - yk : rp[kBins + k];
  b.d0 = kMinD + softplusf(rp[2 * kBins + k]);
  b.d1 = kMinD + softplusf(rp[2 * kBins + k + 1]);
  return b;
}

// Gradient of gy * y + gl * log dy/dx with respect to x (returned) and to the raw
// row (written over rp[0..3K], which on entry holds the normalized widths and
// heights and the raw derivative parameters).
__device__ inline float spline_backward(float *rp, float x, float gy, float gl) {
  const Bin b   = spline_bin(rp, x, false);
  const float w = b.w, h = b.h, d0 = b.d0, d1 = b.d1;
  const float s = h / w;
  float xi      = (x - b.xk) / w;
  xi            = fminf(fmaxf(xi, 0.f), 1.f);
  const float om  = xi * (1.f - xi);
  const float t   = d0 + d1 - 2.f * s;
  const float den = s + t * om;
  const float N1  = s * xi * xi + d0 * om;
  const float Q   = d1 * xi * xi + 2.f * s * om + d0 * (1.f - xi) * (1.f - xi);
  const float iden = 1.f / den, iQ = 1.f / Q;
  const float hd2  = h * iden * iden;
  // partials in (xi, s, d0, d1)
  const float dden_xi = t * (1.f - 2.f * xi), dden_s = 1.f - 2.f * om, dden_d = om;
  const float dN1_xi = 2.f * s * xi + d0 * (1.f - 2.f * xi), dN1_s = xi * xi, dN1_d0 = om;
  const float dQ_xi = 2.f * d1 * xi + 2.f * s * (1.f - 2.f * xi) - 2.f * d0 * (1.f - xi);
  const float dQ_s = 2.f * om, dQ_d0 = (1.f - xi) * (1.f - xi), dQ_d1 = xi * xi;
  const float Gxi = gy * hd2 * (dN1_xi * den - N1 * dden_xi) +
                    gl * (dQ_xi * iQ - 2.f * dden_xi * iden);
  const float Gs = gy * hd2 * (dN1_s * den - N1 * dden_s) +
                   gl * (dQ_s * iQ - 2.f * dden_s * iden + 2.f / s);
  const float Gd0 = gy * hd2 * (dN1_d0 * den - N1 * dden_d) +
                    gl * (dQ_d0 * iQ - 2.f * dden_d * iden);
  const float Gd1 = gy * hd2 * (-N1 * dden_d) + gl * (dQ_d1 * iQ - 2.f * dden_d * iden);
  const float Gh  = gy * N1 * iden + Gs / w;
  const float Gw  = -(Gxi * xi + Gs * s) / w;
  const float Gxk = -Gxi / w;
  const float Gyk = gy;
  const float gx  = Gxi / w;
  // softmax backward of widths and heights: g_raw = c p (G - sum p G)
  const int   k  = b.k;
  const float cw = 1.f - kBins * kMinW, ch = 1.f - kBins * kMinH;
  float sgw = 0.f, sgh = 0.f;
#pragma unroll
  for (int i = 0; i < kBins; ++i) {
    const float pw = (rp[i] - kMinW) / cw, ph = (rp[kBins + i] - kMinH) / ch;
    const float gw = i < k ? Gxk : (i == k ? Gw : 0.f);
    const float gh = i < k ? Gyk : (i == k ? Gh : 0.f);
    sgw += pw * gw;
    sgh += ph * gh;
  }
#pragma unroll
  for (int i = 0; i < kBins; ++i) {
    const float pw = (rp[i] - kMinW) / cw, ph = (rp[kBins + i] - kMinH) / ch;
    const float gw = i < k ? Gxk : (i == k ? Gw : 0.f);
    const float gh = i < k ? Gyk : (i == k ? Gh : 0.f);
    rp[i]         = cw * pw * (gw - sgw);
    rp[kBins + i] = ch * ph * (gh - sgh);
  }
  // derivative parameters: d = minD + softplus(r), dd/dr = sigmoid(r)
#pragma unroll
  for (int i = 0; i <= kBins; ++i) {
    const float r  = rp[2 * kBins + i];
    const float gd = i == k ? Gd0 : (i == k + 1 ? Gd1 : 0.f);
    rp[2 * kBins + i] = gd / (1.f + expf(-r));
  }
  return gx;
}


// ---------------------------------------------------------------------------
// tcgen05 / bulk-copy / mbarrier wrappers and the register-resident spline.

__device__ __forceinline__ uint64_t umma_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= static_cast<uint64_t>((saddr >> 4) & 0x3FFFu);
  d |= static_cast<uint64_t>((lbo >> 4) & 0x3FFFu) << 16;
  d |= static_cast<uint64_t>((sbo >> 4) & 0x3FFFu) << 32;
  d |= static_cast<uint64_t>(1) << 46;  // descriptor version (sm_100 family); no swizzle
  return d;
}

// kind::f16 instruction descriptor: BF16 A and B, FP32 D, both K-major.
__host__ __device__ constexpr uint32_t umma_idesc(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | (static_cast<uint32_t>(N >> 3) << 17) |
         (static_cast<uint32_t>(M >> 4) << 24);
}

__device__ __forceinline__ void umma_bf16(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc,
                                          uint32_t acc) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d_tmem),
      "l"(a), "l"(b), "r"(idesc), "r"(acc));
}

__device__ __forceinline__ void umma_commit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                   bar)
               : "memory");
}

__device__ __forceinline__ void tc_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void fence_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ bool mbar_try(uint32_t bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}\n"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}

// Bounded wait: false after `limit` polls (kSpinLimit by default).
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, int limit = kSpinLimit) {
  for (int i = 0; i < limit; ++i)
    if (mbar_try(bar, parity)) return true;
  return false;
}

__device__ __forceinline__ void bulk_g2s(uint32_t dst, const void *src, uint32_t bytes,
                                         uint32_t bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          dst),
      "l"(src), "r"(bytes), "r"(bar)
      : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes)
               : "memory");
}

// TMEM loads: 32 lanes x 32-bit, N consecutive columns per thread.
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32]) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,"
      "%14,%15,%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]),
        "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]),
        "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float *v) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,"
      "%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ void tmem_ld8(uint32_t taddr, float *v) {
  uint32_t r[8];
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]),
                 "=r"(r[6]), "=r"(r[7])
               : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 8; ++i) v[i] = __uint_as_float(r[i]);
}

// Spline of one coordinate from its 3K+1 parameters held in registers (static
// indexing only: the bin is selected with predicated moves).
template <bool INV>
__device__ __forceinline__ float spline_reg(const float (&r)[kRawP], float v, float &ld) {
  float mw = r[0], mh = r[kBins];
#pragma unroll
  for (int k = 1; k < kBins; ++k) {
    mw = fmaxf(mw, r[k]);
    mh = fmaxf(mh, r[kBins + k]);
  }
  float ew[kBins], eh[kBins], sw = 0.f, sh = 0.f;
#pragma unroll
  for (int k = 0; k < kBins; ++k) {
    ew[k] = __expf(r[k] - mw);
    eh[k] = __expf(r[kBins + k] - mh);
    sw += ew[k];
    sh += eh[k];
  }
  const float cw = (1.f - kBins * kMinW) / sw, ch = (1.f - kBins * kMinH) / sh;
  float X = 0.f, Y = 0.f;
  float xk = 0.f, yk = 0.f, w = kMinW + cw * ew[0], h = kMinH + ch * eh[0];
  float r0 = r[2 * kBins], r1 = r[2 * kBins + 1];
#pragma unroll
  for (int k = 1; k < kBins; ++k) {
    X += kMinW + cw * ew[k - 1];
    Y += kMinH + ch * eh[k - 1];
    const bool sel = INV ? (v >= Y) : (v >= X);
    if (sel) {
      xk = X;
      yk = Y;
      w  = (k == kBins - 1) ? 1.f - X : kMinW + cw * ew[k];
      h  = (k == kBins - 1) ? 1.f - Y : kMinH + ch * eh[k];
      r0 = r[2 * kBins + k];
      r1 = r[2 * kBins + k + 1];
    }
  }
  const float d0 = kMinD + softplusf(r0), d1 = kMinD + softplusf(r1);
  const float s = h / w;
  float       xi, out;
  if (INV) {
    const float dy = v - yk;
    const float t  = d1 + d0 - 2.f * s;
    const float qa = h * (s - d0) + dy * t;
    const float qb = h * d0 - dy * t;
    const float qc = -s * dy;
    const float dn = -qb - sqrtf(fmaxf(qb * qb - 4.f * qa * qc, 0.f));
    xi             = dn != 0.f ? 2.f * qc / dn : 0.f;
    xi             = fminf(fmaxf(xi, 0.f), 1.f);
    out            = fminf(xk + xi * w, 1.f);
  } else {
    xi = fminf(fmaxf((v - xk) / w, 0.f), 1.f);
  }
  const float om  = xi * (1.f - xi);
  const float den = s + (d0 + d1 - 2.f * s) * om;
  const float q   = d1 * xi * xi + 2.f * s * om + d0 * (1.f - xi) * (1.f - xi);
  ld              = logf(s * s * q / (den * den));
  if (!INV) out = yk + h * (s * xi * xi + d0 * om) / den;
  return out;
}


}  // namespace flow
}  // namespace grn
