// grn_flow.cu — learned importance sampler: a coupling-layer normalizing flow with
// rational-quadratic spline transforms (Durkan, Bekasov, Murray, Papamakarios,
// "Neural Spline Flows", NeurIPS 2019; coupling layers after Dinh, Sohl-Dickstein,
// Bengio 2017) over the unit hypercube of the phase-space map.
//
// It plays the role of the reference's neural-network integrator prototype
// (MGraniitti::SampleNeuro, src/MGraniitti.cc:1527-1620, network in
// include/Graniitti/MNeuroJacobian.h): points u = T^{-1}(z) with z uniform, weight
// W(u) / q(u). Here the flow stands in front of the VEGAS grid map, so the exact
// per-point weight stays f = W(x(u)) * vw(u) / q(u) and the estimator is unbiased.
//
// Layer l (density direction x -> z): x_A passes through; each x_j, j in B_l, goes
// through a monotone spline on [0, 1] with K bins whose widths, heights and knot
// derivatives come from an MLP of x_A:
//     x_A (4) -> 128 -> ReLU -> 128 -> ReLU -> 4 * (3K + 1)
// log q(x) = sum over layers and j of log dRQS/dx.
//
// Kernels
//   k_flow_pack    FP32 master weights -> BF16 operand copies, padded layouts
//   k_flow_fwd     density (x -> z, log q) or sampling (z -> x, log q), 128-point
//                  tiles; the 128x128 and 128x224 products run on the tensor cores
//                  (BF16 operands, FP32 accumulation); splines in FP32
//   k_flow_bwd     loss gradient w.r.t. all parameters, 64-point tiles; recomputes
//                  the activations of each layer from its saved input
//   k_flow_adam    Adam update of the FP32 master weights
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "grn_flow.cuh"
#include "grn_philox.cuh"

namespace grn {
namespace flow {

using bf16 = __nv_bfloat16;

constexpr float kMinW = 1e-3f, kMinH = 1e-3f, kMinD = 1e-3f;

// Parameter offsets inside one layer (weights stored [in][out], row-major).
constexpr int oW1 = 0;
constexpr int ob1 = oW1 + kDA * kHid;
constexpr int oW2 = ob1 + kHid;
constexpr int ob2 = oW2 + kHid * kHid;
constexpr int oW3 = ob2 + kHid;
constexpr int ob3 = oW3 + kHid * kNOut;
static_assert(ob3 + kNOut == kLayerParams, "layer layout");

// Shared-memory row strides (elements). +8 BF16 = +16 bytes: the eight rows read by
// one ldmatrix fall into disjoint bank quads.
constexpr int HS  = kHid + 8;   // 136, hidden tiles and W2
constexpr int W3S = kNOutP + 8;  // 232, W3 and the raw-gradient tile
constexpr int RS  = 57;          // FP32 spline-parameter rows (odd: conflict-free per thread)

// Conditioning / transformed index sets; layer l uses mask l % 6.
__constant__ int8_t cA[6][4] = {{0, 1, 2, 3}, {4, 5, 6, 7}, {0, 2, 4, 6},
                                {1, 3, 5, 7}, {0, 1, 4, 5}, {2, 3, 6, 7}};
__constant__ int8_t cB[6][4] = {{4, 5, 6, 7}, {0, 1, 2, 3}, {1, 3, 5, 7},
                                {0, 2, 4, 6}, {2, 3, 6, 7}, {0, 1, 4, 5}};

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

// log dy/dx at relative position xi of bin b.
__device__ __forceinline__ float spline_logdet(const Bin &b, float xi) {
  const float s   = b.h / b.w;
  const float om  = xi * (1.f - xi);
  const float den = s + (b.d0 + b.d1 - 2.f * s) * om;
  const float q   = b.d1 * xi * xi + 2.f * s * om + b.d0 * (1.f - xi) * (1.f - xi);
  return logf(s * s * q / (den * den));
}

__device__ __forceinline__ float spline_forward(const float *rp, float x, float &ld) {
  const Bin b   = spline_bin(rp, x, false);
  const float s = b.h / b.w;
  float xi      = (x - b.xk) / b.w;
  xi            = fminf(fmaxf(xi, 0.f), 1.f);
  const float om  = xi * (1.f - xi);
  const float den = s + (b.d0 + b.d1 - 2.f * s) * om;
  ld              = spline_logdet(b, xi);
  return b.yk + b.h * (s * xi * xi + b.d0 * om) / den;
}

__device__ __forceinline__ float spline_inverse(const float *rp, float y, float &ld) {
  const Bin   b  = spline_bin(rp, y, true);
  const float s  = b.h / b.w;
  const float dy = y - b.yk;
  const float t  = b.d1 + b.d0 - 2.f * s;
  const float qa = b.h * (s - b.d0) + dy * t;
  const float qb = b.h * b.d0 - dy * t;
  const float qc = -s * dy;
  const float disc = fmaxf(qb * qb - 4.f * qa * qc, 0.f);
  const float dn   = -qb - sqrtf(disc);
  float xi         = dn != 0.f ? 2.f * qc / dn : 0.f;
  xi               = fminf(fmaxf(xi, 0.f), 1.f);
  ld               = spline_logdet(b, xi);
  return fminf(b.xk + xi * b.w, 1.f);
}

// Gradient of gy * y + gl * log dy/dx with respect to x (returned) and to the raw
// row (written over rp[0..3K], which on entry holds the normalized widths and
// heights and the raw derivative parameters).
__device__ float spline_backward(float *rp, float x, float gy, float gl) {
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
// Weight staging and the per-layer products shared by both kernels.

struct SmallW {
  float W1[kDA * kHid];  // bf16-rounded
  float b1[kHid];
  float b2[kHid];
  float b3[kNOutP];  // padded: column j*56 + r
};

__device__ void stage_layer(const float *__restrict__ theta, const bf16 *__restrict__ w2p,
                            const bf16 *__restrict__ w3p, int l, bf16 *sW2, bf16 *sW3,
                            SmallW *sw) {
  const uint4 *g2 = reinterpret_cast<const uint4 *>(w2p + static_cast<size_t>(l) * kHid * HS);
  const uint4 *g3 = reinterpret_cast<const uint4 *>(w3p + static_cast<size_t>(l) * kHid * W3S);
  uint4       *s2 = reinterpret_cast<uint4 *>(sW2);
  uint4       *s3 = reinterpret_cast<uint4 *>(sW3);
  constexpr int n2 = kHid * HS * 2 / 16, n3 = kHid * W3S * 2 / 16;
  for (int i = threadIdx.x; i < n2; i += blockDim.x) s2[i] = g2[i];
  for (int i = threadIdx.x; i < n3; i += blockDim.x) s3[i] = g3[i];
  const float *th = theta + static_cast<size_t>(l) * kLayerParams;
  for (int i = threadIdx.x; i < kDA * kHid; i += blockDim.x) sw->W1[i] = bfr(th[oW1 + i]);
  for (int i = threadIdx.x; i < kHid; i += blockDim.x) {
    sw->b1[i] = th[ob1 + i];
    sw->b2[i] = th[ob2 + i];
  }
  for (int i = threadIdx.x; i < kNOutP; i += blockDim.x) {
    const int j = i / kRawP, r = i % kRawP;
    sw->b3[i]   = r < kRaw ? th[ob3 + j * kRaw + r] : 0.f;
  }
}

// h1 = relu(bf16(x_A) . bf16(W1) + b1) for `tile` points (FP32 CUDA cores; K = 4).
__device__ void layer_h1(const float *sX, int tile, int mask, const SmallW *sw, bf16 *sH) {
  const int c = threadIdx.x % kHid;
  for (int p = threadIdx.x / kHid; p < tile; p += blockDim.x / kHid) {
    float a = sw->b1[c];
#pragma unroll
    for (int i = 0; i < kDA; ++i) a = fmaf(bfr(sX[cA[mask][i] * tile + p]), sw->W1[i * kHid + c], a);
    sH[p * HS + c] = __float2bfloat16_rn(fmaxf(a, 0.f));
  }
}

// Warp product over its 16 rows: acc[16 n-tiles] = sA[m0..m0+16)[0..128) . sW[0..128)[0..128)
// with sW stored [k][n]; then relu(acc + b) -> BF16 into sOut (same rows).
__device__ __forceinline__ void warp_h2(const bf16 *sA, const bf16 *sW, const float *bias,
                                        bf16 *sOut, int m0) {
  const int lane = threadIdx.x & 31;
  float     acc[16][4];
#pragma unroll
  for (int i = 0; i < 16; ++i) acc[i][0] = acc[i][1] = acc[i][2] = acc[i][3] = 0.f;
#pragma unroll
  for (int kk = 0; kk < kHid / 16; ++kk) {
    uint32_t a[4];
    ldsm4(a, sA + (m0 + (lane & 15)) * HS + kk * 16 + (lane >> 4) * 8);
#pragma unroll
    for (int np = 0; np < 8; ++np) {
      uint32_t b[4];
      ldsm4t(b, sW + (kk * 16 + (lane & 15)) * HS + np * 16 + (lane >> 4) * 8);
      mma16816(acc[2 * np], a, b[0], b[1]);
      mma16816(acc[2 * np + 1], a, b[2], b[3]);
    }
  }
  __syncwarp();
  const int g = lane >> 2, t = lane & 3;
#pragma unroll
  for (int nt = 0; nt < 16; ++nt) {
    const int   col = nt * 8 + 2 * t;
    const float b0 = bias[col], b1 = bias[col + 1];
    *reinterpret_cast<uint32_t *>(sOut + (m0 + g) * HS + col) =
        pack_bf2(fmaxf(acc[nt][0] + b0, 0.f), fmaxf(acc[nt][1] + b1, 0.f));
    *reinterpret_cast<uint32_t *>(sOut + (m0 + g + 8) * HS + col) =
        pack_bf2(fmaxf(acc[nt][2] + b0, 0.f), fmaxf(acc[nt][3] + b1, 0.f));
  }
  __syncwarp();
}

// Warp product for one pair of transformed dimensions: raw spline parameters of its
// 16 rows, columns [pr*112, pr*112 + 112) of W3, into sRaw[jj][row][r] (r < 49).
__device__ __forceinline__ void warp_raw(const bf16 *sH2, const bf16 *sW3, const float *b3,
                                         float *sRaw, int tile, int m0, int pr) {
  const int lane = threadIdx.x & 31;
  const int cb   = pr * 2 * kRawP;
  float     acc[14][4];
#pragma unroll
  for (int i = 0; i < 14; ++i) acc[i][0] = acc[i][1] = acc[i][2] = acc[i][3] = 0.f;
#pragma unroll
  for (int kk = 0; kk < kHid / 16; ++kk) {
    uint32_t a[4];
    ldsm4(a, sH2 + (m0 + (lane & 15)) * HS + kk * 16 + (lane >> 4) * 8);
#pragma unroll
    for (int np = 0; np < 7; ++np) {
      uint32_t b[4];
      ldsm4t(b, sW3 + (kk * 16 + (lane & 15)) * W3S + cb + np * 16 + (lane >> 4) * 8);
      mma16816(acc[2 * np], a, b[0], b[1]);
      mma16816(acc[2 * np + 1], a, b[2], b[3]);
    }
  }
  const int g = lane >> 2, t = lane & 3;
#pragma unroll
  for (int nt = 0; nt < 14; ++nt) {
    const int col = nt * 8 + 2 * t;  // within the pair block
    const int jj = col / kRawP, r = col % kRawP;
    if (r < kRaw) {
      float *row0 = sRaw + (jj * tile + m0 + g) * RS;
      float *row1 = sRaw + (jj * tile + m0 + g + 8) * RS;
      row0[r]     = acc[nt][0] + b3[cb + col];
      row1[r]     = acc[nt][2] + b3[cb + col];
      if (r + 1 < kRaw) {
        row0[r + 1] = acc[nt][1] + b3[cb + col + 1];
        row1[r + 1] = acc[nt][3] + b3[cb + col + 1];
      }
    }
  }
}

// ---------------------------------------------------------------------------
// Forward kernel: 128-point tiles, 8 warps (16 rows each), persistent grid.

constexpr int kFwdTile = 128, kFwdThreads = 256;
constexpr size_t kFwdSmem = size_t(kHid) * HS * 2 + size_t(kHid) * W3S * 2 +
                            size_t(kFwdTile) * HS * 2 + size_t(2) * kFwdTile * RS * 4 +
                            size_t(kDim) * kFwdTile * 4 + size_t(kFwdTile) * 4 + sizeof(SmallW);

template <int MODE>
__global__ void __launch_bounds__(kFwdThreads, 1)
    k_flow_fwd(const float *__restrict__ theta, const bf16 *__restrict__ w2p,
               const bf16 *__restrict__ w3p, int layers, const float *__restrict__ xin,
               int64_t ld_in, int64_t n, uint64_t seed, uint32_t stream, int64_t first,
               float *__restrict__ xout, int64_t ld_out, float *__restrict__ lq_out,
               float *__restrict__ xs_store) {
  extern __shared__ __align__(16) unsigned char smem[];
  bf16   *sW2  = reinterpret_cast<bf16 *>(smem);
  bf16   *sW3  = sW2 + kHid * HS;
  bf16   *sH   = sW3 + kHid * W3S;
  float  *sRaw = reinterpret_cast<float *>(sH + kFwdTile * HS);
  float  *sX   = sRaw + 2 * kFwdTile * RS;
  float  *sLq  = sX + kDim * kFwdTile;
  SmallW *sw   = reinterpret_cast<SmallW *>(sLq + kFwdTile);

  const int     warp = threadIdx.x >> 5;
  const int     m0   = warp * 16;
  const int64_t ntiles = (n + kFwdTile - 1) / kFwdTile;
  for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const int64_t base = tile * kFwdTile;
    // load the tile (dimension-major)
    for (int i = threadIdx.x; i < kFwdTile; i += blockDim.x) {
      const int64_t e = base + i;
      if (MODE == 1 && xin == nullptr) {
        double u[kDim];
        if (e < n) philox_point(seed, stream, static_cast<uint64_t>(first + e), kDim, u);
#pragma unroll
        for (int j = 0; j < kDim; ++j) sX[j * kFwdTile + i] = e < n ? __double2float_rd(u[j]) : 0.5f;
      } else {
#pragma unroll
        for (int j = 0; j < kDim; ++j) sX[j * kFwdTile + i] = e < n ? xin[j * ld_in + e] : 0.5f;
      }
    }
    float lq = 0.f;
    for (int s = 0; s < layers; ++s) {
      const int l    = MODE == 0 ? s : layers - 1 - s;
      const int mask = l % 6;
      __syncthreads();  // previous layer done with weights, sX settled
      if (xs_store) {
        for (int i = threadIdx.x; i < kFwdTile * kDim; i += blockDim.x) {
          const int j = i / kFwdTile, p = i % kFwdTile;
          if (base + p < n) xs_store[(static_cast<int64_t>(l) * kDim + j) * n + base + p] = sX[i];
        }
      }
      stage_layer(theta, w2p, w3p, l, sW2, sW3, sw);
      __syncthreads();
      layer_h1(sX, kFwdTile, mask, sw, sH);
      __syncthreads();
      warp_h2(sH, sW2, sw->b2, sH, m0);  // warp-private rows: in place
      for (int pr = 0; pr < 2; ++pr) {
        warp_raw(sH, sW3, sw->b3, sRaw, kFwdTile, m0, pr);
        __syncthreads();
        {
          const int p = threadIdx.x % kFwdTile, jj = threadIdx.x / kFwdTile;
          const int j = cB[mask][2 * pr + jj];
          float    *rp = sRaw + (jj * kFwdTile + p) * RS;
          spline_normalize(rp);
          float ld;
          const float v = sX[j * kFwdTile + p];
          sX[j * kFwdTile + p] = MODE == 0 ? spline_forward(rp, v, ld) : spline_inverse(rp, v, ld);
          lq += ld;
        }
        __syncthreads();
      }
    }
    // combine the two threads of each point
    if (threadIdx.x >= kFwdTile) sLq[threadIdx.x - kFwdTile] = lq;
    __syncthreads();
    if (threadIdx.x < kFwdTile) {
      const int64_t e = base + threadIdx.x;
      if (e < n) lq_out[e] = lq + sLq[threadIdx.x];
    }
    if (xout) {
      for (int i = threadIdx.x; i < kFwdTile * kDim; i += blockDim.x) {
        const int j = i / kFwdTile, p = i % kFwdTile;
        if (base + p < n) xout[static_cast<int64_t>(j) * ld_out + base + p] = sX[i];
      }
    }
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
// Backward kernel: 64-point tiles, 4 warps.

constexpr int kBwdTile = 64, kBwdThreads = 128;
constexpr size_t kBwdSmem = size_t(kHid) * HS * 2 + size_t(kHid) * W3S * 2 +
                            2 * size_t(kBwdTile) * HS * 2 + size_t(kBwdTile) * W3S * 2 +
                            size_t(2) * kBwdTile * RS * 4 + 2 * size_t(kDim) * kBwdTile * 4 +
                            size_t(kBwdTile) * 4 + sizeof(SmallW);

// Column sums over the warp's 16 rows of an accumulator tile, added to g[col].
__device__ __forceinline__ void colsum_atomic(const float (&c)[4], float *g, int col) {
  float v0 = c[0] + c[2], v1 = c[1] + c[3];
#pragma unroll
  for (int o = 4; o < 32; o <<= 1) {
    v0 += __shfl_xor_sync(0xffffffffu, v0, o);
    v1 += __shfl_xor_sync(0xffffffffu, v1, o);
  }
  if ((threadIdx.x & 31) < 4) {
    atomicAdd(g + col, v0);
    atomicAdd(g + col + 1, v1);
  }
}

__global__ void __launch_bounds__(kBwdThreads, 1)
    k_flow_bwd(const float *__restrict__ theta, const bf16 *__restrict__ w2p,
               const bf16 *__restrict__ w3p, int layers, const float *__restrict__ xs,
               const float *__restrict__ lq, const float *__restrict__ coef, int64_t n,
               int kind, float inv_n, float *__restrict__ grad, double *__restrict__ loss) {
  extern __shared__ __align__(16) unsigned char smem[];
  bf16   *sW2   = reinterpret_cast<bf16 *>(smem);
  bf16   *sW3   = sW2 + kHid * HS;
  bf16   *sH1   = sW3 + kHid * W3S;
  bf16   *sH2   = sH1 + kBwdTile * HS;
  bf16   *sDraw = sH2 + kBwdTile * HS;
  float  *sRaw  = reinterpret_cast<float *>(sDraw + kBwdTile * W3S);
  float  *sX    = sRaw + 2 * kBwdTile * RS;
  float  *sG    = sX + kDim * kBwdTile;
  float  *sGld  = sG + kDim * kBwdTile;
  SmallW *sw    = reinterpret_cast<SmallW *>(sGld + kBwdTile);
  __shared__ double sLoss[kBwdThreads / 32];

  const int     lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int     g = lane >> 2, t = lane & 3;
  const int     m0 = warp * 16;
  const int64_t ntiles = (n + kBwdTile - 1) / kBwdTile;
  double        my_loss = 0.0;
  for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const int64_t base = tile * kBwdTile;
    __syncthreads();
    if (threadIdx.x < kBwdTile) {
      const int64_t e = base + threadIdx.x;
      float gl = 0.f;
      if (e < n) {
        const float c = coef[e], v = lq[e];
        if (kind == 1) {
          const float ex = c * expf(fminf(-v, 80.f));
          my_loss += ex;
          gl = -ex * inv_n;
        } else {
          my_loss += -static_cast<double>(c) * v;
          gl = -c * inv_n;
        }
      }
      sGld[threadIdx.x] = gl;
    }
    for (int i = threadIdx.x; i < kDim * kBwdTile; i += blockDim.x) sG[i] = 0.f;
    for (int l = layers - 1; l >= 0; --l) {
      const int mask = l % 6;
      const int64_t lo = static_cast<int64_t>(l) * kLayerParams;
      __syncthreads();
      stage_layer(theta, w2p, w3p, l, sW2, sW3, sw);
      for (int i = threadIdx.x; i < kDim * kBwdTile; i += blockDim.x) {
        const int j = i / kBwdTile, p = i % kBwdTile;
        sX[i] = base + p < n ? xs[(static_cast<int64_t>(l) * kDim + j) * n + base + p] : 0.5f;
      }
      __syncthreads();
      layer_h1(sX, kBwdTile, mask, sw, sH1);
      __syncthreads();
      warp_h2(sH1, sW2, sw->b2, sH2, m0);
      for (int pr = 0; pr < 2; ++pr) {
        warp_raw(sH2, sW3, sw->b3, sRaw, kBwdTile, m0, pr);
        __syncthreads();
        {
          const int p = threadIdx.x % kBwdTile, jj = threadIdx.x / kBwdTile;
          const int jb = 2 * pr + jj, j = cB[mask][jb];
          float    *rp = sRaw + (jj * kBwdTile + p) * RS;
          spline_normalize(rp);
          const float gx = spline_backward(rp, sX[j * kBwdTile + p], sG[j * kBwdTile + p], sGld[p]);
          sG[j * kBwdTile + p] = gx;
          bf16 *dr = sDraw + p * W3S + jb * kRawP;
          for (int r = 0; r < kRaw; ++r) dr[r] = __float2bfloat16_rn(rp[r]);
          for (int r = kRaw; r < kRawP; ++r) dr[r] = __float2bfloat16_rn(0.f);
        }
        __syncthreads();
        // b3 gradient: column sums of the FP32 raw gradients
        if (threadIdx.x < 2 * kRaw) {
          const int jj = threadIdx.x / kRaw, r = threadIdx.x % kRaw;
          float     s  = 0.f;
          for (int p = 0; p < kBwdTile; ++p) s += sRaw[(jj * kBwdTile + p) * RS + r];
          if (s != 0.f) atomicAdd(grad + lo + ob3 + (2 * pr + jj) * kRaw + r, s);
        }
        __syncthreads();
      }
      // dW3 = H2^T . G_raw  (M = 128 hidden: warp rows 32w..32w+32; N = 224 in 4 chunks of 56)
      {
        for (int ch = 0; ch < 4; ++ch) {
          float acc[2][7][4];
#pragma unroll
          for (int a = 0; a < 2; ++a)
#pragma unroll
            for (int i = 0; i < 7; ++i) acc[a][i][0] = acc[a][i][1] = acc[a][i][2] = acc[a][i][3] = 0.f;
#pragma unroll
          for (int kk = 0; kk < kBwdTile / 16; ++kk) {
            uint32_t a0[4], a1[4];
            const int kr = kk * 16 + (lane & 7) + (lane >> 4) * 8;
            const int mc = ((lane >> 3) & 1) * 8;
            ldsm4t(a0, sH2 + kr * HS + warp * 32 + mc);
            ldsm4t(a1, sH2 + kr * HS + warp * 32 + 16 + mc);
#pragma unroll
            for (int np = 0; np < 3; ++np) {
              uint32_t b[4];
              ldsm4t(b, sDraw + (kk * 16 + (lane & 15)) * W3S + ch * kRawP + np * 16 + (lane >> 4) * 8);
              mma16816(acc[0][2 * np], a0, b[0], b[1]);
              mma16816(acc[0][2 * np + 1], a0, b[2], b[3]);
              mma16816(acc[1][2 * np], a1, b[0], b[1]);
              mma16816(acc[1][2 * np + 1], a1, b[2], b[3]);
            }
            uint32_t b0, b1;
            ldsm2t(b0, b1, sDraw + (kk * 16 + (lane & 15)) * W3S + ch * kRawP + 48);
            mma16816(acc[0][6], a0, b0, b1);
            mma16816(acc[1][6], a1, b0, b1);
          }
#pragma unroll
          for (int a = 0; a < 2; ++a)
#pragma unroll
            for (int nt = 0; nt < 7; ++nt) {
              const int r = nt * 8 + 2 * t;
              const int h0 = warp * 32 + a * 16 + g;
              float *gw = grad + lo + oW3 + ch * kRaw;
              if (r < kRaw) {
                atomicAdd(gw + h0 * kNOut + r, acc[a][nt][0]);
                atomicAdd(gw + (h0 + 8) * kNOut + r, acc[a][nt][2]);
              }
              if (r + 1 < kRaw) {
                atomicAdd(gw + h0 * kNOut + r + 1, acc[a][nt][1]);
                atomicAdd(gw + (h0 + 8) * kNOut + r + 1, acc[a][nt][3]);
              }
            }
        }
      }
      __syncthreads();
      // dh2 = (G_raw . W3^T) * [h2 > 0]  (warp rows m0; N = 128; K = 224)
      {
        float acc[16][4];
#pragma unroll
        for (int i = 0; i < 16; ++i) acc[i][0] = acc[i][1] = acc[i][2] = acc[i][3] = 0.f;
#pragma unroll 2
        for (int kk = 0; kk < kNOutP / 16; ++kk) {
          uint32_t a[4];
          ldsm4(a, sDraw + (m0 + (lane & 15)) * W3S + kk * 16 + (lane >> 4) * 8);
#pragma unroll
          for (int np = 0; np < 8; ++np) {
            uint32_t b[4];
            ldsm4(b, sW3 + (np * 16 + (lane & 7) + (lane >> 4) * 8) * W3S + kk * 16 +
                         ((lane >> 3) & 1) * 8);
            mma16816(acc[2 * np], a, b[0], b[1]);
            mma16816(acc[2 * np + 1], a, b[2], b[3]);
          }
        }
#pragma unroll
        for (int nt = 0; nt < 16; ++nt) {
          const int col = nt * 8 + 2 * t;
          const bf16 *h0 = sH2 + (m0 + g) * HS + col, *h1 = sH2 + (m0 + g + 8) * HS + col;
          if (!(__bfloat162float(h0[0]) > 0.f)) acc[nt][0] = 0.f;
          if (!(__bfloat162float(h0[1]) > 0.f)) acc[nt][1] = 0.f;
          if (!(__bfloat162float(h1[0]) > 0.f)) acc[nt][2] = 0.f;
          if (!(__bfloat162float(h1[1]) > 0.f)) acc[nt][3] = 0.f;
          colsum_atomic(acc[nt], grad + lo + ob2, col);
        }
        __syncwarp();
#pragma unroll
        for (int nt = 0; nt < 16; ++nt) {
          const int col = nt * 8 + 2 * t;
          *reinterpret_cast<uint32_t *>(sH2 + (m0 + g) * HS + col) = pack_bf2(acc[nt][0], acc[nt][1]);
          *reinterpret_cast<uint32_t *>(sH2 + (m0 + g + 8) * HS + col) = pack_bf2(acc[nt][2], acc[nt][3]);
        }
      }
      __syncthreads();
      // dW2 = H1^T . dH2  (M = 128 in: warp rows 32w..; N = 128 out in 2 chunks of 64)
      for (int ch = 0; ch < 2; ++ch) {
        float acc[2][8][4];
#pragma unroll
        for (int a = 0; a < 2; ++a)
#pragma unroll
          for (int i = 0; i < 8; ++i) acc[a][i][0] = acc[a][i][1] = acc[a][i][2] = acc[a][i][3] = 0.f;
#pragma unroll
        for (int kk = 0; kk < kBwdTile / 16; ++kk) {
          uint32_t a0[4], a1[4];
          const int kr = kk * 16 + (lane & 7) + (lane >> 4) * 8;
          const int mc = ((lane >> 3) & 1) * 8;
          ldsm4t(a0, sH1 + kr * HS + warp * 32 + mc);
          ldsm4t(a1, sH1 + kr * HS + warp * 32 + 16 + mc);
#pragma unroll
          for (int np = 0; np < 4; ++np) {
            uint32_t b[4];
            ldsm4t(b, sH2 + (kk * 16 + (lane & 15)) * HS + ch * 64 + np * 16 + (lane >> 4) * 8);
            mma16816(acc[0][2 * np], a0, b[0], b[1]);
            mma16816(acc[0][2 * np + 1], a0, b[2], b[3]);
            mma16816(acc[1][2 * np], a1, b[0], b[1]);
            mma16816(acc[1][2 * np + 1], a1, b[2], b[3]);
          }
        }
#pragma unroll
        for (int a = 0; a < 2; ++a)
#pragma unroll
          for (int nt = 0; nt < 8; ++nt) {
            const int col = ch * 64 + nt * 8 + 2 * t;
            const int h0  = warp * 32 + a * 16 + g;
            float *gw = grad + lo + oW2;
            atomicAdd(gw + h0 * kHid + col, acc[a][nt][0]);
            atomicAdd(gw + h0 * kHid + col + 1, acc[a][nt][1]);
            atomicAdd(gw + (h0 + 8) * kHid + col, acc[a][nt][2]);
            atomicAdd(gw + (h0 + 8) * kHid + col + 1, acc[a][nt][3]);
          }
      }
      // dh1 = (dH2 . W2^T) * [h1 > 0]  (warp rows m0; N = 128 in; K = 128 out)
      {
        float acc[16][4];
#pragma unroll
        for (int i = 0; i < 16; ++i) acc[i][0] = acc[i][1] = acc[i][2] = acc[i][3] = 0.f;
#pragma unroll
        for (int kk = 0; kk < kHid / 16; ++kk) {
          uint32_t a[4];
          ldsm4(a, sH2 + (m0 + (lane & 15)) * HS + kk * 16 + (lane >> 4) * 8);
#pragma unroll
          for (int np = 0; np < 8; ++np) {
            uint32_t b[4];
            ldsm4(b, sW2 + (np * 16 + (lane & 7) + (lane >> 4) * 8) * HS + kk * 16 +
                         ((lane >> 3) & 1) * 8);
            mma16816(acc[2 * np], a, b[0], b[1]);
            mma16816(acc[2 * np + 1], a, b[2], b[3]);
          }
        }
#pragma unroll
        for (int nt = 0; nt < 16; ++nt) {
          const int col = nt * 8 + 2 * t;
          const bf16 *h0 = sH1 + (m0 + g) * HS + col, *h1 = sH1 + (m0 + g + 8) * HS + col;
          if (!(__bfloat162float(h0[0]) > 0.f)) acc[nt][0] = 0.f;
          if (!(__bfloat162float(h0[1]) > 0.f)) acc[nt][1] = 0.f;
          if (!(__bfloat162float(h1[0]) > 0.f)) acc[nt][2] = 0.f;
          if (!(__bfloat162float(h1[1]) > 0.f)) acc[nt][3] = 0.f;
          colsum_atomic(acc[nt], grad + lo + ob1, col);
        }
        __syncthreads();  // every warp is done reading H1 (dW2) before it is replaced
#pragma unroll
        for (int nt = 0; nt < 16; ++nt) {
          const int col = nt * 8 + 2 * t;
          *reinterpret_cast<uint32_t *>(sH1 + (m0 + g) * HS + col) = pack_bf2(acc[nt][0], acc[nt][1]);
          *reinterpret_cast<uint32_t *>(sH1 + (m0 + g + 8) * HS + col) = pack_bf2(acc[nt][2], acc[nt][3]);
        }
      }
      __syncthreads();
      // dW1[a][c] = sum_p bf16(x_A[a][p]) dH1[p][c]; dx_A[p][a] = sum_c dH1[p][c] bf16(W1[a][c])
      {
        const int c = threadIdx.x;
        float     s[kDA] = {0.f, 0.f, 0.f, 0.f};
        for (int p = 0; p < kBwdTile; ++p) {
          const float d = __bfloat162float(sH1[p * HS + c]);
#pragma unroll
          for (int a = 0; a < kDA; ++a) s[a] = fmaf(bfr(sX[cA[mask][a] * kBwdTile + p]), d, s[a]);
        }
#pragma unroll
        for (int a = 0; a < kDA; ++a)
          if (s[a] != 0.f) atomicAdd(grad + lo + oW1 + a * kHid + c, s[a]);
      }
      {
        const int p = threadIdx.x % kBwdTile, ap = threadIdx.x / kBwdTile;
        float     s0 = 0.f, s1 = 0.f;
        for (int c = 0; c < kHid; ++c) {
          const float d = __bfloat162float(sH1[p * HS + c]);
          s0 = fmaf(d, sw->W1[(2 * ap) * kHid + c], s0);
          s1 = fmaf(d, sw->W1[(2 * ap + 1) * kHid + c], s1);
        }
        sG[cA[mask][2 * ap] * kBwdTile + p] += s0;
        sG[cA[mask][2 * ap + 1] * kBwdTile + p] += s1;
      }
    }
  }
  // loss: warp sums, then one atomic per block
  for (int o = 16; o > 0; o >>= 1) my_loss += __shfl_down_sync(0xffffffffu, my_loss, o);
  if (lane == 0) sLoss[warp] = my_loss;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int w = 0; w < kBwdThreads / 32; ++w) s += sLoss[w];
    atomicAdd(loss, s);
  }
}

// ---------------------------------------------------------------------------
// Packing and Adam.

__global__ void k_flow_pack(const float *__restrict__ theta, int layers, bf16 *__restrict__ w2p,
                            bf16 *__restrict__ w3p) {
  const int64_t n2 = static_cast<int64_t>(layers) * kHid * HS;
  const int64_t n3 = static_cast<int64_t>(layers) * kHid * W3S;
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n2 + n3;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    if (i < n2) {
      const int64_t l = i / (kHid * HS);
      const int     r = static_cast<int>(i % (kHid * HS));
      const int     k = r / HS, c = r % HS;
      w2p[i] = __float2bfloat16_rn(c < kHid ? theta[l * kLayerParams + oW2 + k * kHid + c] : 0.f);
    } else {
      const int64_t i3 = i - n2;
      const int64_t l  = i3 / (kHid * W3S);
      const int     r  = static_cast<int>(i3 % (kHid * W3S));
      const int     k = r / W3S, c = r % W3S;
      const int     j = c / kRawP, q = c % kRawP;
      const bool    real = c < kNOutP && q < kRaw;
      w3p[i3] = __float2bfloat16_rn(real ? theta[l * kLayerParams + oW3 + k * kNOut + j * kRaw + q]
                                         : 0.f);
    }
  }
}

__global__ void k_flow_adam(float *__restrict__ theta, float *__restrict__ m,
                            float *__restrict__ v, const float *__restrict__ grad, int64_t n,
                            float lr_t, float b1, float b2, float eps_t) {
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const float gr = grad[i];
    const float mi = b1 * m[i] + (1.f - b1) * gr;
    const float vi = b2 * v[i] + (1.f - b2) * gr * gr;
    m[i]           = mi;
    v[i]           = vi;
    theta[i] -= lr_t * mi / (sqrtf(vi) + eps_t);
  }
}

__global__ void k_flow_coef(const double *__restrict__ f, const float *__restrict__ lq0,
                            int64_t n, int kind, double inv_norm, float *__restrict__ coef) {
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const double fi = f[i];
    double       c;
    if (kind == 1)
      c = fi * fi * (lq0 ? exp(static_cast<double>(lq0[i])) : 1.0) * inv_norm;
    else
      c = fi * inv_norm;
    coef[i] = static_cast<float>(c);
  }
}

__global__ void k_flow_uniform(uint64_t seed, uint32_t stream, int64_t n, float *__restrict__ u,
                               float *__restrict__ lq) {
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    double v[kDim];
    philox_point(seed, stream, static_cast<uint64_t>(i), kDim, v);
#pragma unroll
    for (int j = 0; j < kDim; ++j) u[j * n + i] = __double2float_rd(v[j]);
    if (lq) lq[i] = 0.f;
  }
}

}  // namespace flow

// ---------------------------------------------------------------------------
// Launchers

using flow::bf16;

size_t flow_w2p_elems(int layers) { return size_t(layers) * flow::kHid * flow::HS; }
size_t flow_w3p_elems(int layers) { return size_t(layers) * flow::kHid * flow::W3S; }

static int sm_count() {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  return sms;
}

cudaError_t launch_flow_pack(const float *theta, int layers, void *w2p, void *w3p,
                             cudaStream_t st) {
  flow::k_flow_pack<<<4 * sm_count(), 256, 0, st>>>(theta, layers, static_cast<bf16 *>(w2p),
                                                    static_cast<bf16 *>(w3p));
  return cudaGetLastError();
}

cudaError_t launch_flow_forward(int mode, const float *theta, const void *w2p, const void *w3p,
                                int layers, const float *xin, int64_t ld_in, int64_t n,
                                uint64_t seed, uint32_t stream, int64_t first, float *xout,
                                int64_t ld_out, float *lq, float *xs_store, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  const int64_t tiles = (n + flow::kFwdTile - 1) / flow::kFwdTile;
  const int     grid  = static_cast<int>(std::min<int64_t>(tiles, sm_count()));
  const size_t  sm    = flow::kFwdSmem;
  if (mode == 0) {
    cudaFuncSetAttribute(flow::k_flow_fwd<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(sm));
    flow::k_flow_fwd<0><<<grid, flow::kFwdThreads, sm, st>>>(
        theta, static_cast<const bf16 *>(w2p), static_cast<const bf16 *>(w3p), layers, xin,
        ld_in, n, seed, stream, first, xout, ld_out, lq, xs_store);
  } else {
    cudaFuncSetAttribute(flow::k_flow_fwd<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(sm));
    flow::k_flow_fwd<1><<<grid, flow::kFwdThreads, sm, st>>>(
        theta, static_cast<const bf16 *>(w2p), static_cast<const bf16 *>(w3p), layers, xin,
        ld_in, n, seed, stream, first, xout, ld_out, lq, xs_store);
  }
  return cudaGetLastError();
}

cudaError_t launch_flow_backward(const float *theta, const void *w2p, const void *w3p, int layers,
                                 const float *xs, const float *lq, const float *coef, int64_t n,
                                 int kind, float *grad, double *loss, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  const int64_t tiles = (n + flow::kBwdTile - 1) / flow::kBwdTile;
  const int     grid  = static_cast<int>(std::min<int64_t>(tiles, sm_count()));
  const size_t  sm    = flow::kBwdSmem;
  cudaFuncSetAttribute(flow::k_flow_bwd, cudaFuncAttributeMaxDynamicSharedMemorySize, int(sm));
  flow::k_flow_bwd<<<grid, flow::kBwdThreads, sm, st>>>(
      theta, static_cast<const bf16 *>(w2p), static_cast<const bf16 *>(w3p), layers, xs, lq,
      coef, n, kind, 1.0f / static_cast<float>(n), grad, loss);
  return cudaGetLastError();
}

cudaError_t launch_flow_adam(float *theta, float *m, float *v, const float *grad, int64_t n,
                             float lr_t, float b1, float b2, float eps_t, cudaStream_t st) {
  flow::k_flow_adam<<<2 * sm_count(), 256, 0, st>>>(theta, m, v, grad, n, lr_t, b1, b2, eps_t);
  return cudaGetLastError();
}

cudaError_t launch_flow_coef(const double *f, const float *lq0, int64_t n, int kind, double norm,
                             float *coef, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  flow::k_flow_coef<<<4 * sm_count(), 256, 0, st>>>(f, lq0, n, kind, 1.0 / norm, coef);
  return cudaGetLastError();
}

cudaError_t launch_flow_uniform(uint64_t seed, uint32_t stream, int64_t n, float *u, float *lq,
                                cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  flow::k_flow_uniform<<<4 * sm_count(), 256, 0, st>>>(seed, stream, n, u, lq);
  return cudaGetLastError();
}

}  // namespace grn
