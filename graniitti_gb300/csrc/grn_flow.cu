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
//   k_flow_fwd     density (x -> z, log q) or sampling (z -> x, log q): tcgen05
//                  products (BF16 operands, FP32 accumulators in TMEM), weights
//                  staged by bulk copies, FP32 splines from the thread's TMEM row
//   (backward)     warp-level BF16 mma.sync products from ldmatrix fragments
//   k_flow_bwd     loss gradient w.r.t. all parameters, 64-point tiles; recomputes
//                  the activations of each layer from its saved input
//   k_flow_adam    Adam update of the FP32 master weights
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "grn_flow.cuh"
#include "grn_flow_prims.cuh"
#include "grn_philox.cuh"

namespace grn {
namespace flow {


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
// Forward kernel on the 5th-generation tensor cores.
//
// One CTA = 256 threads = two warpgroups; thread t owns point t of a 256-point
// subtile (warpgroup g = t / 128 owns rows 0..127 of its own M = 128 products).
// Per layer the CTA stages W2 and W3 once with two bulk copies (TMA engine,
// completion on an mbarrier) and runs four subtiles (a 1024-point supertile)
// through it:
//   h1 = relu(x_A W1 + b1)            CUDA cores, BF16 into the A tile (canonical layout)
//   D2 = h1 . W2                      tcgen05.mma, M=128 N=128 K=128, FP32 in TMEM
//   h2 = relu(D2 + b2)                tcgen05.ld -> BF16 into the A tile
//   D3 = h2 . W3                      tcgen05.mma, M=128 N=256 K=128, FP32 in TMEM
//   splines                           tcgen05.ld of the thread's own row: 4 x 49 values
// Operand layout in shared memory (no swizzle, K-major): element (r, k) of an
// R-row tile at byte (k / 8) * 16R + r * 16 + (k % 8) * 2, i.e. 8x16-byte core
// matrices with leading-byte offset 16R (next 8 columns of k) and stride-byte
// offset 128 (next 8 rows). TMEM: D2 of warpgroup g in columns [128g, 128g+128),
// D3 in [256g, 256g+256) with coordinate jb in columns [64jb, 64jb+49) of it (every
// TMEM load starts on a multiple of its width); 512 columns, one CTA per SM.

constexpr int kFwdThreads = 256, kSub = 256, kSubs = 4, kSuper = kSub * kSubs;
constexpr int kTmemCols = 512;
constexpr int kNOutF = kDA * kRawF;   // D3 columns in all (256)
constexpr uint32_t kW2Bytes = kHid * kHid * 2;    // 32768
constexpr uint32_t kW3Bytes = kNOutF * kHid * 2;  // 65536
constexpr uint32_t kABytes  = 128 * kHid * 2;     // 32768 per warpgroup
constexpr uint32_t kOffW2 = 0, kOffW3 = kOffW2 + kW2Bytes, kOffA = kOffW3 + kW3Bytes;
constexpr uint32_t kOffX  = kOffA + 2 * kABytes;
constexpr uint32_t kOffLq = kOffX + kDim * kSuper * 4;
constexpr uint32_t kOffSw = kOffLq + kSuper * 4;
constexpr uint32_t kOffBar = (kOffSw + sizeof(SmallW) + 15) / 16 * 16;
constexpr size_t   kFwdSmem = kOffBar + 32;
static_assert(kW2Bytes % 16 == 0 && kW3Bytes % 16 == 0 && kOffA % 16 == 0 && kOffX % 16 == 0,
              "bulk copies and descriptors need 16-byte alignment");

template <int MODE>
__global__ void __launch_bounds__(kFwdThreads, 1)
    k_flow_fwd(const float *__restrict__ theta, const bf16 *__restrict__ w2c,
               const bf16 *__restrict__ w3c, int layers, const float *__restrict__ xin,
               int64_t ld_in, int64_t n, uint64_t seed, uint32_t stream, int64_t first,
               float *__restrict__ xout, int64_t ld_out, float *__restrict__ lq_out,
               float *__restrict__ xs_store, int *__restrict__ err, int first_wait_polls) {
  extern __shared__ __align__(1024) unsigned char fwd_smem[];
  unsigned char *smem = fwd_smem;
  float    *sX  = reinterpret_cast<float *>(smem + kOffX);
  float    *sLq = reinterpret_cast<float *>(smem + kOffLq);
  SmallW   *sw  = reinterpret_cast<SmallW *>(smem + kOffSw);
  uint64_t *bars = reinterpret_cast<uint64_t *>(smem + kOffBar);
  uint32_t *tslot = reinterpret_cast<uint32_t *>(smem + kOffBar + 16);
  const uint32_t s_base = smem_u32(smem);
  const uint32_t bar_w = smem_u32(&bars[0]), bar_m = smem_u32(&bars[1]);
  const int      t = threadIdx.x, warp = t >> 5, wg = t >> 7, row = t & 127;

  if (t == 0) {
    mbar_init(bar_w, 1);
    mbar_init(bar_m, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(tslot)),
                 "r"(kTmemCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tslot;
  // this thread's TMEM row (lane) and its warpgroup's column bases
  const uint32_t t_lane = static_cast<uint32_t>((warp & 3) * 32) << 16;
  const uint32_t d2_col = 128u * wg, d3_col = 256u * wg;
  uint8_t       *gA = smem + kOffA + wg * kABytes;
  constexpr uint32_t idesc2 = umma_idesc(128, kHid), idesc3 = umma_idesc(128, kNOutF);
  uint32_t n_w = 0, n_m = 0;  // phases issued on the weight / product barriers
  bool     aborted = false;

  const int64_t nsup = (n + kSuper - 1) / kSuper;
  for (int64_t sup = blockIdx.x; sup < nsup && !aborted; sup += gridDim.x) {
    const int64_t base = sup * kSuper;
    for (int i = t; i < kSuper; i += kFwdThreads) {
      const int64_t e = base + i;
      if (MODE == 1 && xin == nullptr) {
        double u[kDim];
        if (e < n) philox_point(seed, stream, static_cast<uint64_t>(first + e), kDim, u);
#pragma unroll
        for (int j = 0; j < kDim; ++j) sX[j * kSuper + i] = e < n ? __double2float_rd(u[j]) : 0.5f;
      } else {
#pragma unroll
        for (int j = 0; j < kDim; ++j) sX[j * kSuper + i] = e < n ? xin[j * ld_in + e] : 0.5f;
      }
      sLq[i] = 0.f;
    }
    for (int s = 0; s < layers && !aborted; ++s) {
      const int l = MODE == 0 ? s : layers - 1 - s;
      const int mask = l % 6;
      __syncthreads();  // previous layer's products are complete; sX settled
      ++n_w;
      if (t == 0) {
        mbar_expect_tx(bar_w, kW2Bytes + kW3Bytes);
        bulk_g2s(s_base + kOffW2, w2c + static_cast<size_t>(l) * (kW2Bytes / 2), kW2Bytes, bar_w);
        bulk_g2s(s_base + kOffW3, w3c + static_cast<size_t>(l) * (kW3Bytes / 2), kW3Bytes, bar_w);
      }
      {
        const float *th = theta + static_cast<size_t>(l) * kLayerParams;
        for (int i = t; i < kDA * kHid; i += kFwdThreads) sw->W1[i] = bfr(th[oW1 + i]);
        for (int i = t; i < kHid; i += kFwdThreads) {
          sw->b1[i] = th[ob1 + i];
          sw->b2[i] = th[ob2 + i];
        }
        for (int i = t; i < kNOutP; i += kFwdThreads) {
          const int j = i / kRawP, r = i % kRawP;
          sw->b3[i] = r < kRaw ? th[ob3 + j * kRaw + r] : 0.f;
        }
      }
      if (xs_store) {
        for (int i = t; i < kSuper * kDim; i += kFwdThreads) {
          const int j = i / kSuper, p = i % kSuper;
          if (base + p < n) xs_store[(static_cast<int64_t>(l) * kDim + j) * n + base + p] = sX[i];
        }
      }
      // the first weight-copy wait of the CTA may take a caller-set poll limit (the test of
      // the timeout path); the drain waits below keep the default limit
      const bool okw = mbar_wait(bar_w, (n_w - 1) & 1u,
                                 n_w == 1 && first_wait_polls >= 0 ? first_wait_polls : kSpinLimit);
      if (__syncthreads_or(!okw)) {
        aborted = true;
        break;
      }
      for (int sub = 0; sub < kSubs; ++sub) {
        const int p = sub * kSub + t;
        // h1 = relu(bf16(x_A) bf16(W1) + b1) -> BF16 A tile, row `row`
        {
          float xa[kDA];
#pragma unroll
          for (int i = 0; i < kDA; ++i) xa[i] = bfr(sX[cA[mask][i] * kSuper + p]);
#pragma unroll 2
          for (int c = 0; c < kHid / 8; ++c) {
            float v[8];
#pragma unroll
            for (int q = 0; q < 8; ++q) {
              const int col = c * 8 + q;
              float     a   = sw->b1[col];
#pragma unroll
              for (int i = 0; i < kDA; ++i) a = fmaf(xa[i], sw->W1[i * kHid + col], a);
              v[q] = fmaxf(a, 0.f);
            }
            uint4 pk;
            pk.x = pack_bf2(v[0], v[1]);
            pk.y = pack_bf2(v[2], v[3]);
            pk.z = pack_bf2(v[4], v[5]);
            pk.w = pack_bf2(v[6], v[7]);
            *reinterpret_cast<uint4 *>(gA + c * (16 * 128) + row * 16) = pk;
          }
        }
        fence_async_smem();
        tc_fence_before();
        __syncthreads();
        if (t == 0) {
          tc_fence_after();
#pragma unroll 1
          for (int g = 0; g < 2; ++g) {
            const uint32_t a0 = s_base + kOffA + g * kABytes;
#pragma unroll
            for (int kk = 0; kk < kHid / 16; ++kk)
              umma_bf16(tmem + 128u * g, umma_desc(a0 + kk * 2 * 2048, 2048, 128),
                        umma_desc(s_base + kOffW2 + kk * 2 * 2048, 2048, 128), idesc2, kk > 0);
          }
          umma_commit(bar_m);
        }
        ++n_m;
        bool ok = mbar_wait(bar_m, (n_m - 1) & 1u);
        if (__syncthreads_or(!ok)) {
          aborted = true;
          break;
        }
        tc_fence_after();
        // h2 = relu(D2 + b2) -> BF16 A tile (the products that read h1 are complete)
#pragma unroll 1
        for (int c = 0; c < kHid / 32; ++c) {
          float v[32];
          tmem_ld32(tmem + t_lane + d2_col + 32u * c, v);
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            uint4       pk;
            const int   col = c * 32 + q * 8;
            const float *b2 = sw->b2 + col;
            pk.x = pack_bf2(fmaxf(v[q * 8 + 0] + b2[0], 0.f), fmaxf(v[q * 8 + 1] + b2[1], 0.f));
            pk.y = pack_bf2(fmaxf(v[q * 8 + 2] + b2[2], 0.f), fmaxf(v[q * 8 + 3] + b2[3], 0.f));
            pk.z = pack_bf2(fmaxf(v[q * 8 + 4] + b2[4], 0.f), fmaxf(v[q * 8 + 5] + b2[5], 0.f));
            pk.w = pack_bf2(fmaxf(v[q * 8 + 6] + b2[6], 0.f), fmaxf(v[q * 8 + 7] + b2[7], 0.f));
            *reinterpret_cast<uint4 *>(gA + (col / 8) * (16 * 128) + row * 16) = pk;
          }
        }
        fence_async_smem();
        tc_fence_before();
        __syncthreads();
        if (t == 0) {
          tc_fence_after();
#pragma unroll 1
          for (int g = 0; g < 2; ++g) {
            const uint32_t a0 = s_base + kOffA + g * kABytes;
#pragma unroll
            for (int kk = 0; kk < kHid / 16; ++kk)
              umma_bf16(tmem + 256u * g, umma_desc(a0 + kk * 2 * 2048, 2048, 128),
                        umma_desc(s_base + kOffW3 + kk * 2 * (16 * kNOutF), 16 * kNOutF, 128),
                        idesc3, kk > 0);
          }
          umma_commit(bar_m);
        }
        ++n_m;
        ok = mbar_wait(bar_m, (n_m - 1) & 1u);
        if (__syncthreads_or(!ok)) {
          aborted = true;
          break;
        }
        tc_fence_after();
        // splines of the four transformed coordinates of this thread's point
        float lq = 0.f;
#pragma unroll 1
        for (int jb = 0; jb < kDA; ++jb) {
          float r[kRawP];
          const uint32_t ta = tmem + t_lane + d3_col + static_cast<uint32_t>(jb * kRawF);
          float v32[32];
          tmem_ld32(ta, v32);
#pragma unroll
          for (int i = 0; i < 32; ++i) r[i] = v32[i];
          tmem_ld16(ta + 32, r + 32);
          tmem_ld8(ta + 48, r + 48);
#pragma unroll
          for (int i = 0; i < kRaw; ++i) r[i] += sw->b3[jb * kRawP + i];
          const int j  = cB[mask][jb];
          float     ld;
          const float vin = sX[j * kSuper + p];
          sX[j * kSuper + p] = spline_reg<MODE == 1>(r, vin, ld);
          lq += ld;
        }
        sLq[p] += lq;
        tc_fence_before();
        __syncthreads();  // D3 read out before the next subtile's D2 overwrites it
      }
    }
    if (aborted) break;
    __syncthreads();
    for (int i = t; i < kSuper; i += kFwdThreads)
      if (base + i < n) lq_out[base + i] = sLq[i];
    if (xout) {
      for (int i = t; i < kSuper * kDim; i += kFwdThreads) {
        const int j = i / kSuper, p = i % kSuper;
        if (base + p < n) xout[static_cast<int64_t>(j) * ld_out + base + p] = sX[i];
      }
    }
  }
  if (aborted) {
    if (t == 0) atomicExch(err, 1);
    // let outstanding copies and products land before the memory is released
    if (n_w) mbar_wait(bar_w, (n_w - 1) & 1u);
    if (n_m) mbar_wait(bar_m, (n_m - 1) & 1u);
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"(kTmemCols)
                 : "memory");
  }
}

// ---------------------------------------------------------------------------
// Backward kernel: 64-point tiles, 4 warps.

constexpr int kBwdTile = 64, kBwdThreads = 128;
constexpr size_t kBwdSmem = size_t(kHid) * HS * 2 + size_t(kHid) * W3S * 2 +
                            2 * size_t(kBwdTile) * HS * 2 + size_t(kBwdTile) * W3S * 2 +
                            size_t(2) * kBwdTile * RS * 4 + 2 * size_t(kDim) * kBwdTile * 4 +
                            size_t(kBwdTile) * 4 + sizeof(SmallW);

// Column sums over the warp's 16 rows of an accumulator tile into this warp's row of the
// staging array (summed over the warps in a fixed order afterwards).
__device__ __forceinline__ void colsum_stage(const float (&c)[4], float *scol, int col) {
  float v0 = c[0] + c[2], v1 = c[1] + c[3];
#pragma unroll
  for (int o = 4; o < 32; o <<= 1) {
    v0 += __shfl_xor_sync(0xffffffffu, v0, o);
    v1 += __shfl_xor_sync(0xffffffffu, v1, o);
  }
  if ((threadIdx.x & 31) < 4) {
    scol[(threadIdx.x >> 5) * kHid + col]     = v0;
    scol[(threadIdx.x >> 5) * kHid + col + 1] = v1;
  }
}

__global__ void __launch_bounds__(kBwdThreads, 1)
    k_flow_bwd(const float *__restrict__ theta, const bf16 *__restrict__ w2p,
               const bf16 *__restrict__ w3p, int layers, const float *__restrict__ xs,
               const float *__restrict__ lq, const float *__restrict__ coef, int64_t n,
               int kind, float inv_n, float *__restrict__ part, double *__restrict__ loss_part) {
  // this block's private slice of the gradient: every element has one writer at a time,
  // so the accumulation order (and the result) is fixed
  float *__restrict__ grad = part + static_cast<int64_t>(blockIdx.x) * layers * kLayerParams;
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
  __shared__ float  sCol2[(kBwdThreads / 32) * kHid], sCol1[(kBwdThreads / 32) * kHid];

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
          grad[lo + ob3 + (2 * pr + jj) * kRaw + r] += s;
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
                gw[h0 * kNOut + r] += acc[a][nt][0];
                gw[(h0 + 8) * kNOut + r] += acc[a][nt][2];
              }
              if (r + 1 < kRaw) {
                gw[h0 * kNOut + r + 1] += acc[a][nt][1];
                gw[(h0 + 8) * kNOut + r + 1] += acc[a][nt][3];
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
          colsum_stage(acc[nt], sCol2, col);
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
      if (threadIdx.x < kHid) {  // b2 gradient: the warps' column sums in a fixed order
        float v = 0.f;
        for (int w = 0; w < kBwdThreads / 32; ++w) v += sCol2[w * kHid + threadIdx.x];
        grad[lo + ob2 + threadIdx.x] += v;
      }
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
            gw[h0 * kHid + col] += acc[a][nt][0];
            gw[h0 * kHid + col + 1] += acc[a][nt][1];
            gw[(h0 + 8) * kHid + col] += acc[a][nt][2];
            gw[(h0 + 8) * kHid + col + 1] += acc[a][nt][3];
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
          colsum_stage(acc[nt], sCol1, col);
        }
        __syncthreads();  // every warp is done reading H1 (dW2) before it is replaced
        if (threadIdx.x < kHid) {  // b1 gradient: the warps' column sums in a fixed order
          float v = 0.f;
          for (int w = 0; w < kBwdThreads / 32; ++w) v += sCol1[w * kHid + threadIdx.x];
          grad[lo + ob1 + threadIdx.x] += v;
        }
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
          grad[lo + oW1 + a * kHid + c] += s[a];
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
    loss_part[blockIdx.x] = s;
  }
}

// grad[i] = sum over the blocks' slices in block order; loss = sum of the block losses.
__global__ void k_flow_grad_reduce(const float *__restrict__ part, int nslices, int64_t np,
                                   float *__restrict__ grad, const double *__restrict__ loss_part,
                                   double *__restrict__ loss) {
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < np;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    float v = 0.f;
    for (int c = 0; c < nslices; ++c) v += part[c * np + i];
    grad[i] = v;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    double v = 0.0;
    for (int c = 0; c < nslices; ++c) v += loss_part[c];
    *loss = v;
  }
}

// ---------------------------------------------------------------------------
// Packing and Adam.

// FP32 master weights -> BF16 operand copies:
//   w2p, w3p  padded row-major [k][n] tiles for the backward kernel (ldmatrix)
//   w2c, w3c  canonical K-major layouts of W2^T and W3^T for the forward kernel
//             (element (n, k) of an N-row operand at (k/8)*8N + n*8 + k%8)
__global__ void k_flow_pack(const float *__restrict__ theta, int layers, bf16 *__restrict__ w2p,
                            bf16 *__restrict__ w3p, bf16 *__restrict__ w2c,
                            bf16 *__restrict__ w3c) {
  const int64_t n2 = static_cast<int64_t>(layers) * kHid * HS;
  const int64_t n3 = static_cast<int64_t>(layers) * kHid * W3S;
  const int64_t c2 = static_cast<int64_t>(layers) * kHid * kHid;
  const int64_t c3 = static_cast<int64_t>(layers) * kNOutF * kHid;
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
       i < n2 + n3 + c2 + c3; i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    if (i < n2) {
      const int64_t l = i / (kHid * HS);
      const int     r = static_cast<int>(i % (kHid * HS));
      const int     k = r / HS, c = r % HS;
      w2p[i] = __float2bfloat16_rn(c < kHid ? theta[l * kLayerParams + oW2 + k * kHid + c] : 0.f);
    } else if (i < n2 + n3) {
      const int64_t i3 = i - n2;
      const int64_t l  = i3 / (kHid * W3S);
      const int     r  = static_cast<int>(i3 % (kHid * W3S));
      const int     k = r / W3S, c = r % W3S;
      const int     j = c / kRawP, q = c % kRawP;
      const bool    real = c < kNOutP && q < kRaw;
      w3p[i3] = __float2bfloat16_rn(real ? theta[l * kLayerParams + oW3 + k * kNOut + j * kRaw + q]
                                         : 0.f);
    } else if (i < n2 + n3 + c2) {
      const int64_t i2 = i - n2 - n3;
      const int64_t l  = i2 / (kHid * kHid);
      const int     r  = static_cast<int>(i2 % (kHid * kHid));
      const int     kc = r / (8 * kHid), nn = (r / 8) % kHid, k = kc * 8 + r % 8;
      w2c[i2] = __float2bfloat16_rn(theta[l * kLayerParams + oW2 + k * kHid + nn]);
    } else {
      const int64_t i3 = i - n2 - n3 - c2;
      const int64_t l  = i3 / (kNOutF * kHid);
      const int     r  = static_cast<int>(i3 % (kNOutF * kHid));
      const int     kc = r / (8 * kNOutF), nn = (r / 8) % kNOutF, k = kc * 8 + r % 8;
      const int     j = nn / kRawF, q = nn % kRawF;
      w3c[i3] = __float2bfloat16_rn(q < kRaw ? theta[l * kLayerParams + oW3 + k * kNOut + j * kRaw + q]
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

__global__ void k_flow_uniform(uint64_t seed, uint32_t stream, int64_t first, int64_t n,
                               int64_t ld, float *__restrict__ u, float *__restrict__ lq) {
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    double v[kDim];
    philox_point(seed, stream, static_cast<uint64_t>(first + i), kDim, v);
#pragma unroll
    for (int j = 0; j < kDim; ++j) u[j * ld + i] = __double2float_rd(v[j]);
    if (lq) lq[i] = 0.f;
  }
}

// Density of the defensive mixture alpha * uniform + (1 - alpha) * flow from the flow's log q.
__global__ void k_flow_mix(float *__restrict__ lq, int64_t n, double alpha) {
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x)
    lq[i] = static_cast<float>(log(alpha + (1.0 - alpha) * exp(static_cast<double>(lq[i]))));
}

}  // namespace flow

// ---------------------------------------------------------------------------
// Launchers

using flow::bf16;

size_t flow_w2p_elems(int layers) { return size_t(layers) * flow::kHid * flow::HS; }
size_t flow_w3p_elems(int layers) { return size_t(layers) * flow::kHid * flow::W3S; }
size_t flow_w2c_elems(int layers) { return size_t(layers) * flow::kHid * flow::kHid; }
size_t flow_w3c_elems(int layers) { return size_t(layers) * flow::kNOutF * flow::kHid; }

static int sm_count() {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  return sms;
}

cudaError_t launch_flow_pack(const float *theta, int layers, void *w2p, void *w3p, void *w2c,
                             void *w3c, cudaStream_t st) {
  flow::k_flow_pack<<<4 * sm_count(), 256, 0, st>>>(
      theta, layers, static_cast<bf16 *>(w2p), static_cast<bf16 *>(w3p), static_cast<bf16 *>(w2c),
      static_cast<bf16 *>(w3c));
  return cudaGetLastError();
}

cudaError_t launch_flow_forward(int mode, const float *theta, const void *w2c, const void *w3c,
                                int layers, const float *xin, int64_t ld_in, int64_t n,
                                uint64_t seed, uint32_t stream, int64_t first, float *xout,
                                int64_t ld_out, float *lq, float *xs_store, int *err,
                                cudaStream_t st, int first_wait_polls) {
  if (n <= 0) return cudaSuccess;
  const int64_t sup  = (n + flow::kSuper - 1) / flow::kSuper;
  const int     grid = static_cast<int>(std::min<int64_t>(sup, sm_count()));
  const int     sm   = static_cast<int>(flow::kFwdSmem);
  const bf16   *a = static_cast<const bf16 *>(w2c), *b = static_cast<const bf16 *>(w3c);
  if (mode == 0) {
    cudaFuncSetAttribute(flow::k_flow_fwd<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm);
    flow::k_flow_fwd<0><<<grid, flow::kFwdThreads, sm, st>>>(
        theta, a, b, layers, xin, ld_in, n, seed, stream, first, xout, ld_out, lq, xs_store, err,
        first_wait_polls);
  } else {
    cudaFuncSetAttribute(flow::k_flow_fwd<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm);
    flow::k_flow_fwd<1><<<grid, flow::kFwdThreads, sm, st>>>(
        theta, a, b, layers, xin, ld_in, n, seed, stream, first, xout, ld_out, lq, xs_store, err,
        first_wait_polls);
  }
  return cudaGetLastError();
}

int flow_backward_slices() { return sm_count(); }

cudaError_t launch_flow_backward(const float *theta, const void *w2p, const void *w3p, int layers,
                                 const float *xs, const float *lq, const float *coef, int64_t n,
                                 int kind, float *part, double *loss_part, float *grad,
                                 double *loss, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  const int64_t tiles  = (n + flow::kBwdTile - 1) / flow::kBwdTile;
  const int     grid   = static_cast<int>(std::min<int64_t>(tiles, sm_count()));
  const size_t  sm     = flow::kBwdSmem;
  const int64_t np     = static_cast<int64_t>(layers) * flow::kLayerParams;
  cudaError_t   e      = cudaMemsetAsync(part, 0, static_cast<size_t>(grid) * np * sizeof(float), st);
  if (e != cudaSuccess) return e;
  cudaFuncSetAttribute(flow::k_flow_bwd, cudaFuncAttributeMaxDynamicSharedMemorySize, int(sm));
  flow::k_flow_bwd<<<grid, flow::kBwdThreads, sm, st>>>(
      theta, static_cast<const bf16 *>(w2p), static_cast<const bf16 *>(w3p), layers, xs, lq,
      coef, n, kind, 1.0f / static_cast<float>(n), part, loss_part);
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  return launch_flow_grad_reduce(part, grid, np, grad, loss_part, loss, st);
}

cudaError_t launch_flow_grad_reduce(const float *part, int nslices, int64_t np, float *grad,
                                    const double *loss_part, double *loss, cudaStream_t st) {
  flow::k_flow_grad_reduce<<<2 * sm_count(), 256, 0, st>>>(part, nslices, np, grad, loss_part,
                                                            loss);
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

cudaError_t launch_flow_uniform(uint64_t seed, uint32_t stream, int64_t first, int64_t n,
                                int64_t ld, float *u, float *lq, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  flow::k_flow_uniform<<<4 * sm_count(), 256, 0, st>>>(seed, stream, first, n, ld, u, lq);
  return cudaGetLastError();
}

cudaError_t launch_flow_mix(float *lq, int64_t n, double alpha, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  flow::k_flow_mix<<<4 * sm_count(), 256, 0, st>>>(lq, n, alpha);
  return cudaGetLastError();
}

}  // namespace grn
