// grn_flow_wide.cu — the coupling-layer spline flow of grn_flow.cu for more dimensions and
// wider conditioners: D = 8 or 14 hypercube dimensions (2-body processes, two-body
// cascades), MLP width H = 128 or 256. Same model and parameter layout as grn_flow.cu
// (x_A (D/2) -> H -> ReLU -> H -> ReLU -> (D/2)(3K+1), rational-quadratic splines with
// K = 16 bins); the (D, H) = (8, 128) network keeps the kernels of grn_flow.cu, whose two
// layers of weights fit in shared memory at once.
//
// Forward (k_wfwd, tcgen05): a layer's weights (H x H and H x (D/2) 64 BF16) exceed shared
// memory for H = 256, so they stream through two 64-column chunk buffers by bulk copies
// (TMA engine, mbarrier completion), double-buffered across the whole run of a CTA: the H/64
// chunks of W2, then one chunk of W3 per transformed coordinate. A CTA is two warpgroups;
// each owns the 128-row A tile (BF16, K-major canonical layout) of its 128 points and an
// H-column TMEM region: D2 = h1 . W2 fills the region chunk by chunk, and once h2 is
// read out the coordinate products D3_j = h2 . W3_j (64 columns each) alternate between the
// region's first two 64-column slots, the spline of coordinate j running while the product
// of j + 1 is in flight.
//
// Backward (k_wbwd, mma.sync m16n8k16): 64-point tiles as in grn_flow.cu, activations and
// gradients in shared memory, the B fragments of the weight products read from row-major
// BF16 copies in global memory (L2-resident: 0.6 MB per layer at H = 256, D = 14).
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "grn_flow.cuh"
#include "grn_flow_prims.cuh"
#include "grn_philox.cuh"

namespace grn {
namespace flow {
namespace wide {

template <int D, int H>
struct Cfg {
  static constexpr int DA    = D / 2;
  static constexpr int NOut  = DA * kRaw;    // raw conditioner outputs
  static constexpr int NOutP = DA * kRawP;   // padded to 56 per coordinate (backward)
  static constexpr int oW1 = 0, ob1 = DA * H, oW2 = ob1 + H, ob2 = oW2 + H * H, oW3 = ob2 + H,
                       ob3 = oW3 + H * NOut;
  static constexpr int LP  = ob3 + NOut;     // parameters per layer
  static constexpr int NC2 = H / 64;         // W2 chunks (64 output columns each)
  static constexpr int NC  = NC2 + DA;       // chunks per layer
  static constexpr uint32_t kChunkBytes = 64u * H * 2u;
  static constexpr uint32_t kABytes     = 128u * H * 2u;  // one warpgroup's A tile
  static constexpr int      kTmemCols   = 2 * H;          // two warpgroup regions
  // shared memory of the forward kernel
  static constexpr uint32_t oA   = 0;
  static constexpr uint32_t oC   = oA + 2 * kABytes;
  static constexpr uint32_t oX   = oC + 2 * kChunkBytes;
  static constexpr uint32_t oW1s = oX + D * 256 * 4;
  static constexpr uint32_t ob1s = oW1s + DA * H * 4;
  static constexpr uint32_t ob2s = ob1s + H * 4;
  static constexpr uint32_t ob3s = ob2s + H * 4;
  static constexpr uint32_t oBar = (ob3s + DA * kRawF * 4 + 15) / 16 * 16;
  static constexpr size_t   kFwdSmem = oBar + 32;
  static_assert(H % 64 == 0 && H <= 256, "width");
  static_assert(kFwdSmem <= 232448, "forward shared memory");
  static_assert(oC % 16 == 0 && oX % 16 == 0 && kChunkBytes % 16 == 0, "bulk-copy alignment");
};

// Conditioning (A) and transformed (B) sets of layer l (mask l % 6): halves, even / odd,
// pairs of neighbours; the second of each pair of masks swaps A and B.
__constant__ int8_t cA8[6][4] = {{0, 1, 2, 3}, {4, 5, 6, 7}, {0, 2, 4, 6},
                                 {1, 3, 5, 7}, {0, 1, 4, 5}, {2, 3, 6, 7}};
__constant__ int8_t cB8[6][4] = {{4, 5, 6, 7}, {0, 1, 2, 3}, {1, 3, 5, 7},
                                 {0, 2, 4, 6}, {2, 3, 6, 7}, {0, 1, 4, 5}};
__constant__ int8_t cA14[6][7] = {{0, 1, 2, 3, 4, 5, 6},     {7, 8, 9, 10, 11, 12, 13},
                                  {0, 2, 4, 6, 8, 10, 12},    {1, 3, 5, 7, 9, 11, 13},
                                  {0, 1, 4, 5, 8, 9, 12},     {2, 3, 6, 7, 10, 11, 13}};
__constant__ int8_t cB14[6][7] = {{7, 8, 9, 10, 11, 12, 13},  {0, 1, 2, 3, 4, 5, 6},
                                  {1, 3, 5, 7, 9, 11, 13},    {0, 2, 4, 6, 8, 10, 12},
                                  {2, 3, 6, 7, 10, 11, 13},   {0, 1, 4, 5, 8, 9, 12}};

__constant__ int8_t cA12[6][6] = {{0, 1, 2, 3, 4, 5},        {6, 7, 8, 9, 10, 11},
                                  {0, 2, 4, 6, 8, 10},       {1, 3, 5, 7, 9, 11},
                                  {0, 1, 4, 5, 8, 9},        {2, 3, 6, 7, 10, 11}};
__constant__ int8_t cB12[6][6] = {{6, 7, 8, 9, 10, 11},      {0, 1, 2, 3, 4, 5},
                                  {1, 3, 5, 7, 9, 11},       {0, 2, 4, 6, 8, 10},
                                  {2, 3, 6, 7, 10, 11},      {0, 1, 4, 5, 8, 9}};

template <int D>
__device__ __forceinline__ int mask_a(int m, int i) {
  if constexpr (D == 8) return cA8[m][i];
  else if constexpr (D == 12) return cA12[m][i];
  else return cA14[m][i];
}
template <int D>
__device__ __forceinline__ int mask_b(int m, int i) {
  if constexpr (D == 8) return cB8[m][i];
  else if constexpr (D == 12) return cB12[m][i];
  else return cB14[m][i];
}

// ---------------------------------------------------------------------------
// Forward kernel.

// Source of chunk kq (CTA-local running index) of a kernel that runs `layers` layers per
// subtile in the direction of MODE.
template <int MODE, int D, int H>
__device__ __forceinline__ const bf16 *chunk_src(const bf16 *w2c, const bf16 *w3c, int layers,
                                                 int64_t kq) {
  using C = Cfg<D, H>;
  const int q = static_cast<int>(kq % (static_cast<int64_t>(layers) * C::NC));
  const int s = q / C::NC, c = q % C::NC;
  const int l = MODE == 0 ? s : layers - 1 - s;
  if (c < C::NC2) return w2c + (static_cast<size_t>(l) * C::NC2 + c) * (64 * H);
  return w3c + (static_cast<size_t>(l) * C::DA + (c - C::NC2)) * (64 * H);
}

template <int MODE, int D, int H>
__global__ void __launch_bounds__(256, 1)
    k_wfwd(const float *__restrict__ theta, const bf16 *__restrict__ w2c,
           const bf16 *__restrict__ w3c, int layers, const float *__restrict__ xin,
           int64_t ld_in, int64_t n, uint64_t seed, uint32_t stream, int64_t first,
           float *__restrict__ xout, int64_t ld_out, float *__restrict__ lq_out,
           float *__restrict__ xs_store, int *__restrict__ err) {
  using C = Cfg<D, H>;
  constexpr int DA = C::DA;
  extern __shared__ __align__(1024) unsigned char wsm[];
  float    *sX   = reinterpret_cast<float *>(wsm + C::oX);
  float    *sW1  = reinterpret_cast<float *>(wsm + C::oW1s);
  float    *sb1  = reinterpret_cast<float *>(wsm + C::ob1s);
  float    *sb2  = reinterpret_cast<float *>(wsm + C::ob2s);
  float    *sb3  = reinterpret_cast<float *>(wsm + C::ob3s);
  uint64_t *bars = reinterpret_cast<uint64_t *>(wsm + C::oBar);
  uint32_t *tslot = reinterpret_cast<uint32_t *>(wsm + C::oBar + 24);
  const uint32_t s_base = smem_u32(wsm);
  const uint32_t bar_w0 = smem_u32(&bars[0]), bar_w1 = smem_u32(&bars[1]);
  const uint32_t bar_m  = smem_u32(&bars[2]);
  const int      t = threadIdx.x, warp = t >> 5, wg = t >> 7, row = t & 127;

  if (t == 0) {
    mbar_init(bar_w0, 1);
    mbar_init(bar_w1, 1);
    mbar_init(bar_m, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(tslot)),
                 "r"(C::kTmemCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem   = *tslot;
  const uint32_t t_lane = static_cast<uint32_t>((warp & 3) * 32) << 16;
  const uint32_t region = static_cast<uint32_t>(H) * wg;  // this warpgroup's TMEM columns
  uint8_t       *gA     = wsm + C::oA + wg * C::kABytes;
  constexpr uint32_t idesc = umma_idesc(128, 64);

  const int64_t nsub  = (n + 255) / 256;
  const int64_t mine  = blockIdx.x < nsub ? (nsub - blockIdx.x + gridDim.x - 1) / gridDim.x : 0;
  const int64_t total = mine * layers * C::NC;  // chunks this CTA consumes
  int64_t  kq = 0;       // next chunk to consume
  uint32_t n_m = 0;      // product-barrier phases waited
  int64_t  issued = 0;   // chunks whose copy has been issued (thread 0)
  bool     aborted = false, fill_fail = false;

  // thread 0: copy chunk `c` into buffer c & 1
  auto fill = [&](int64_t c) {
    const uint32_t b = static_cast<uint32_t>(c & 1);
    const uint32_t bar = b ? bar_w1 : bar_w0;
    mbar_expect_tx(bar, C::kChunkBytes);
    bulk_g2s(s_base + C::oC + b * C::kChunkBytes, chunk_src<MODE, D, H>(w2c, w3c, layers, c),
             C::kChunkBytes, bar);
  };
  // thread 0: wait for chunk kq's copy, then the two warpgroups' products into TMEM
  // column `col` of each region (N = 64, K = H); commit to the product barrier (also when
  // the copy never landed, so that every thread reaches the check below).
  auto issue = [&](int64_t c, uint32_t col) {
    const uint32_t b = static_cast<uint32_t>(c & 1);
    if (!mbar_wait(b ? bar_w1 : bar_w0, static_cast<uint32_t>((c >> 1) & 1))) {
      fill_fail = true;
    } else {
      tc_fence_after();
      const uint32_t bB = s_base + C::oC + b * C::kChunkBytes;
#pragma unroll 1
      for (int g = 0; g < 2; ++g) {
        const uint32_t a0 = s_base + C::oA + g * C::kABytes;
#pragma unroll 4
        for (int kk = 0; kk < H / 16; ++kk)
          umma_bf16(tmem + static_cast<uint32_t>(H) * g + col,
                    umma_desc(a0 + kk * 2 * 2048, 2048, 128),
                    umma_desc(bB + kk * 2 * 1024, 1024, 128), idesc, kk > 0);
      }
    }
    umma_commit(bar_m);
  };
  // all threads: wait for the last committed products; thread 0 then refills the buffer
  // they read with chunk c + 2. False when a wait gave up.
  auto wait_products = [&](int64_t c) -> bool {
    ++n_m;
    const bool ok = mbar_wait(bar_m, (n_m - 1) & 1u);
    if (__syncthreads_or(!ok || fill_fail)) return false;
    tc_fence_after();
    if (t == 0 && c + 2 < total) {
      fill(c + 2);
      issued = c + 3;
    }
    return true;
  };

  if (t == 0 && total > 0) {
    fill(0);
    issued = 1;
    if (total > 1) {
      fill(1);
      issued = 2;
    }
  }

  for (int64_t sub = blockIdx.x; sub < nsub && !aborted; sub += gridDim.x) {
    const int64_t base = sub * 256, e = base + t;
    if (MODE == 1 && xin == nullptr) {
      double u[D];
      if (e < n) philox_point(seed, stream, static_cast<uint64_t>(first + e), D, u);
#pragma unroll
      for (int j = 0; j < D; ++j) sX[j * 256 + t] = e < n ? __double2float_rd(u[j]) : 0.5f;
    } else {
#pragma unroll
      for (int j = 0; j < D; ++j) sX[j * 256 + t] = e < n ? xin[j * ld_in + e] : 0.5f;
    }
    float lq = 0.f;
    for (int s = 0; s < layers && !aborted; ++s) {
      const int l = MODE == 0 ? s : layers - 1 - s;
      const int mask = l % 6;
      __syncthreads();  // the previous layer's readers of the small weights are done
      {
        const float *th = theta + static_cast<size_t>(l) * C::LP;
        for (int i = t; i < DA * H; i += 256) sW1[i] = bfr(th[C::oW1 + i]);
        for (int i = t; i < H; i += 256) {
          sb1[i] = th[C::ob1 + i];
          sb2[i] = th[C::ob2 + i];
        }
        for (int i = t; i < DA * kRawF; i += 256) {
          const int j = i / kRawF, r = i % kRawF;
          sb3[i]      = r < kRaw ? th[C::ob3 + j * kRaw + r] : 0.f;
        }
      }
      if (xs_store && e < n) {
#pragma unroll
        for (int j = 0; j < D; ++j)
          xs_store[(static_cast<int64_t>(l) * D + j) * n + e] = sX[j * 256 + t];
      }
      __syncthreads();
      // h1 = relu(bf16(x_A) bf16(W1) + b1) -> BF16 A tile, row `row` of this warpgroup
      {
        float xa[DA];
#pragma unroll
        for (int i = 0; i < DA; ++i) xa[i] = bfr(sX[mask_a<D>(mask, i) * 256 + t]);
#pragma unroll 1
        for (int c = 0; c < H / 8; ++c) {
          float v[8];
#pragma unroll
          for (int q = 0; q < 8; ++q) {
            const int col = c * 8 + q;
            float     a   = sb1[col];
#pragma unroll
            for (int i = 0; i < DA; ++i) a = fmaf(xa[i], sW1[i * H + col], a);
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
      // D2 = h1 . W2, chunk by chunk into columns [64c, 64c + 64) of each region
      for (int c = 0; c < C::NC2; ++c) {
        if (t == 0) issue(kq, 64u * c);
        if (!wait_products(kq)) {
          aborted = true;
          break;
        }
        ++kq;
      }
      if (aborted) break;
      // h2 = relu(D2 + b2) -> BF16 A tile (every product that read h1 is complete)
#pragma unroll 1
      for (int c = 0; c < H / 32; ++c) {
        float v[32];
        tmem_ld32(tmem + t_lane + region + 32u * c, v);
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          uint4        pk;
          const int    col = c * 32 + q * 8;
          const float *b2  = sb2 + col;
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
      // D3_j = h2 . W3_j into slot j & 1 (columns [64 (j & 1), +64) of each region); the
      // product of j + 1 runs while the splines of coordinate j are evaluated
      if (t == 0) issue(kq, 0u);
      for (int jb = 0; jb < DA; ++jb) {
        if (!wait_products(kq)) {
          aborted = true;
          break;
        }
        ++kq;
        if (t == 0 && jb + 1 < DA) issue(kq, 64u * ((jb + 1) & 1));
        float r[kRawP];
        {
          const uint32_t ta = tmem + t_lane + region + 64u * (jb & 1);
          float          v32[32];
          tmem_ld32(ta, v32);
#pragma unroll
          for (int i = 0; i < 32; ++i) r[i] = v32[i];
          tmem_ld16(ta + 32, r + 32);
          tmem_ld8(ta + 48, r + 48);
        }
#pragma unroll
        for (int i = 0; i < kRaw; ++i) r[i] += sb3[jb * kRawF + i];
        const int   j = mask_b<D>(mask, jb);
        float       ld;
        const float vin  = sX[j * 256 + t];
        sX[j * 256 + t] = spline_reg<MODE == 1>(r, vin, ld);
        lq += ld;
        tc_fence_before();
        __syncthreads();  // slot jb & 1 read out before the product of jb + 2 overwrites it
      }
    }
    if (aborted) break;
    if (e < n) {
      lq_out[e] = lq;
      if (xout) {
#pragma unroll
        for (int j = 0; j < D; ++j) xout[static_cast<int64_t>(j) * ld_out + e] = sX[j * 256 + t];
      }
    }
  }
  if (aborted) {
    if (t == 0) {
      atomicExch(err, 1);
      // let the copies in flight land and the products finish before the memory goes
      for (int64_t c = kq; c < issued; ++c)
        mbar_wait((c & 1) ? bar_w1 : bar_w0, static_cast<uint32_t>((c >> 1) & 1));
      umma_commit(bar_m);
      mbar_wait(bar_m, n_m & 1u);
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"(C::kTmemCols)
                 : "memory");
  }
}

// ---------------------------------------------------------------------------
// Backward kernel: 64-point tiles, 4 warps; warp w owns tile rows 16w..16w+16 of the
// row-partitioned products. Weight B fragments come from row-major copies in global memory:
//   w2t [out][in] and w3t [o][h] (o = 56 j + r) for the recomputed forward products,
//   w2r [in][out] and w3r [h][o] (o < NOutB, zero beyond 56 j + 49) for the transposed ones.

template <int D, int H>
struct Bwd {
  using C = Cfg<D, H>;
  static constexpr int DA    = C::DA;
  static constexpr int NOutB = (C::NOutP + 15) / 16 * 16;  // K of G_raw . W3^T
  static constexpr int HS    = H + 8;                      // BF16 row strides (+16 bytes)
  static constexpr int GS    = NOutB + 8;
  static constexpr int RS    = 57;
  static constexpr int T     = 64;
  static constexpr size_t oH1 = 0, oH2 = oH1 + size_t(T) * HS * 2, oD1 = oH2 + size_t(T) * HS * 2,
                          oDr = oD1 + size_t(T) * HS * 2, oRaw = oDr + size_t(T) * GS * 2,
                          oX = oRaw + size_t(2) * T * RS * 4, oG = oX + size_t(D) * T * 4,
                          oGl = oG + size_t(D) * T * 4, oW1 = oGl + size_t(T) * 4,
                          ob1 = oW1 + size_t(DA) * H * 4, ob2 = ob1 + size_t(H) * 4,
                          ob3 = ob2 + size_t(H) * 4, oC1 = ob3 + size_t(C::NOutP) * 4,
                          oC2 = oC1 + size_t(4) * H * 4, kSmem = oC2 + size_t(4) * H * 4;
  static_assert(kSmem <= 232448, "backward shared memory");
};

// B fragment (m16n8k16, .col) of B[k][n] held as M[n][k] (k contiguous, leading dimension ldm).
__device__ __forceinline__ void ldg_b(uint32_t &b0, uint32_t &b1, const bf16 *__restrict__ M,
                                      int ldm, int n0, int k0) {
  const int   lane = threadIdx.x & 31;
  const bf16 *p    = M + static_cast<size_t>(n0 + (lane >> 2)) * ldm + k0 + 2 * (lane & 3);
  b0 = __ldg(reinterpret_cast<const unsigned int *>(p));
  b1 = __ldg(reinterpret_cast<const unsigned int *>(p + 8));
}

// Column sums over the warp's 16 rows of an accumulator tile into row `warp` of scol.
template <int H>
__device__ __forceinline__ void colsum_w(const float (&c)[4], float *scol, int col) {
  float v0 = c[0] + c[2], v1 = c[1] + c[3];
#pragma unroll
  for (int o = 4; o < 32; o <<= 1) {
    v0 += __shfl_xor_sync(0xffffffffu, v0, o);
    v1 += __shfl_xor_sync(0xffffffffu, v1, o);
  }
  if ((threadIdx.x & 31) < 4) {
    scol[(threadIdx.x >> 5) * H + col]     = v0;
    scol[(threadIdx.x >> 5) * H + col + 1] = v1;
  }
}

template <int D, int H>
__global__ void __launch_bounds__(128, 1)
    k_wbwd(const float *__restrict__ theta, const bf16 *__restrict__ w2t,
           const bf16 *__restrict__ w2r, const bf16 *__restrict__ w3t,
           const bf16 *__restrict__ w3r, int layers, const float *__restrict__ xs,
           const float *__restrict__ lq, const float *__restrict__ coef, int64_t n, int kind,
           float inv_n, float *__restrict__ part, double *__restrict__ loss_part) {
  using C = Cfg<D, H>;
  using B = Bwd<D, H>;
  constexpr int DA = C::DA, HS = B::HS, GS = B::GS, RS = B::RS, T = B::T;
  float *__restrict__ grad = part + static_cast<int64_t>(blockIdx.x) * layers * C::LP;
  extern __shared__ __align__(16) unsigned char bsm[];
  bf16  *sH1 = reinterpret_cast<bf16 *>(bsm + B::oH1);
  bf16  *sH2 = reinterpret_cast<bf16 *>(bsm + B::oH2);
  bf16  *sD1 = reinterpret_cast<bf16 *>(bsm + B::oD1);
  bf16  *sDr = reinterpret_cast<bf16 *>(bsm + B::oDr);
  float *sRaw = reinterpret_cast<float *>(bsm + B::oRaw);
  float *sX  = reinterpret_cast<float *>(bsm + B::oX);
  float *sG  = reinterpret_cast<float *>(bsm + B::oG);
  float *sGl = reinterpret_cast<float *>(bsm + B::oGl);
  float *sW1 = reinterpret_cast<float *>(bsm + B::oW1);
  float *sb1 = reinterpret_cast<float *>(bsm + B::ob1);
  float *sb2 = reinterpret_cast<float *>(bsm + B::ob2);
  float *sb3 = reinterpret_cast<float *>(bsm + B::ob3);
  float *sC1 = reinterpret_cast<float *>(bsm + B::oC1);
  float *sC2 = reinterpret_cast<float *>(bsm + B::oC2);
  __shared__ double sLoss[4];

  const int     lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int     g = lane >> 2, tq = lane & 3;
  const int     m0 = warp * 16;
  const int64_t ntiles = (n + T - 1) / T;
  double        my_loss = 0.0;
  for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const int64_t base = tile * T;
    __syncthreads();
    if (threadIdx.x < T) {
      const int64_t e  = base + threadIdx.x;
      float         gl = 0.f;
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
      sGl[threadIdx.x] = gl;
    }
    for (int i = threadIdx.x; i < D * T; i += blockDim.x) sG[i] = 0.f;
    for (int l = layers - 1; l >= 0; --l) {
      const int     mask = l % 6;
      const int64_t lo   = static_cast<int64_t>(l) * C::LP;
      const bf16   *W2t = w2t + static_cast<size_t>(l) * H * H;
      const bf16   *W2r = w2r + static_cast<size_t>(l) * H * H;
      const bf16   *W3t = w3t + static_cast<size_t>(l) * C::NOutP * H;
      const bf16   *W3r = w3r + static_cast<size_t>(l) * H * B::NOutB;
      __syncthreads();
      {
        const float *th = theta + lo;
        for (int i = threadIdx.x; i < DA * H; i += blockDim.x) sW1[i] = bfr(th[C::oW1 + i]);
        for (int i = threadIdx.x; i < H; i += blockDim.x) {
          sb1[i] = th[C::ob1 + i];
          sb2[i] = th[C::ob2 + i];
        }
        for (int i = threadIdx.x; i < C::NOutP; i += blockDim.x) {
          const int j = i / kRawP, r = i % kRawP;
          sb3[i]      = r < kRaw ? th[C::ob3 + j * kRaw + r] : 0.f;
        }
        for (int i = threadIdx.x; i < D * T; i += blockDim.x) {
          const int j = i / T, p = i % T;
          sX[i] = base + p < n ? xs[(static_cast<int64_t>(l) * D + j) * n + base + p] : 0.5f;
        }
        // zero the padding columns of the raw-gradient tile once per layer
        for (int i = threadIdx.x; i < T * (GS - C::NOutP); i += blockDim.x) {
          const int p = i / (GS - C::NOutP), c = C::NOutP + i % (GS - C::NOutP);
          sDr[p * GS + c] = __float2bfloat16_rn(0.f);
        }
      }
      __syncthreads();
      // h1 = relu(bf16(x_A) bf16(W1) + b1)  (CUDA cores)
      for (int i = threadIdx.x; i < T * H; i += blockDim.x) {
        const int p = i / H, c = i % H;
        float     a = sb1[c];
#pragma unroll
        for (int k = 0; k < DA; ++k) a = fmaf(bfr(sX[mask_a<D>(mask, k) * T + p]), sW1[k * H + c], a);
        sH1[p * HS + c] = __float2bfloat16_rn(fmaxf(a, 0.f));
      }
      __syncthreads();
      // h2 = relu(h1 . W2 + b2): warp rows m0, 64-column chunks, B from w2t
      for (int ch = 0; ch < H / 64; ++ch) {
        float acc[8][4];
#pragma unroll
        for (int i = 0; i < 8; ++i) acc[i][0] = acc[i][1] = acc[i][2] = acc[i][3] = 0.f;
#pragma unroll 2
        for (int kk = 0; kk < H / 16; ++kk) {
          uint32_t a[4];
          ldsm4(a, sH1 + (m0 + (lane & 15)) * HS + kk * 16 + (lane >> 4) * 8);
#pragma unroll
          for (int nt = 0; nt < 8; ++nt) {
            uint32_t b0, b1;
            ldg_b(b0, b1, W2t, H, ch * 64 + nt * 8, kk * 16);
            mma16816(acc[nt], a, b0, b1);
          }
        }
#pragma unroll
        for (int nt = 0; nt < 8; ++nt) {
          const int   col = ch * 64 + nt * 8 + 2 * tq;
          const float c0 = sb2[col], c1 = sb2[col + 1];
          *reinterpret_cast<uint32_t *>(sH2 + (m0 + g) * HS + col) =
              pack_bf2(fmaxf(acc[nt][0] + c0, 0.f), fmaxf(acc[nt][1] + c1, 0.f));
          *reinterpret_cast<uint32_t *>(sH2 + (m0 + g + 8) * HS + col) =
              pack_bf2(fmaxf(acc[nt][2] + c0, 0.f), fmaxf(acc[nt][3] + c1, 0.f));
        }
      }
      __syncwarp();
      // raw spline parameters two coordinates at a time, then the spline gradients
      for (int pr = 0; pr < (DA + 1) / 2; ++pr) {
        const int ncols = (2 * pr + 1 < DA) ? 2 * kRawP : kRawP;  // 112 or 56
        {
          float acc[14][4];
#pragma unroll
          for (int i = 0; i < 14; ++i) acc[i][0] = acc[i][1] = acc[i][2] = acc[i][3] = 0.f;
#pragma unroll 2
          for (int kk = 0; kk < H / 16; ++kk) {
            uint32_t a[4];
            ldsm4(a, sH2 + (m0 + (lane & 15)) * HS + kk * 16 + (lane >> 4) * 8);
#pragma unroll
            for (int nt = 0; nt < 14; ++nt) {
              if (nt * 8 < ncols) {
                uint32_t b0, b1;
                ldg_b(b0, b1, W3t, H, pr * 2 * kRawP + nt * 8, kk * 16);
                mma16816(acc[nt], a, b0, b1);
              }
            }
          }
#pragma unroll
          for (int nt = 0; nt < 14; ++nt) {
            const int col = nt * 8 + 2 * tq;  // within the pair block
            const int jj = col / kRawP, r = col % kRawP;
            if (col < ncols && r < kRaw) {
              const float *b3 = sb3 + pr * 2 * kRawP + col;
              float *row0 = sRaw + (jj * T + m0 + g) * RS;
              float *row1 = sRaw + (jj * T + m0 + g + 8) * RS;
              row0[r]     = acc[nt][0] + b3[0];
              row1[r]     = acc[nt][2] + b3[0];
              if (r + 1 < kRaw) {
                row0[r + 1] = acc[nt][1] + b3[1];
                row1[r + 1] = acc[nt][3] + b3[1];
              }
            }
          }
        }
        __syncthreads();
        {
          const int p = threadIdx.x % T, jj = threadIdx.x / T;
          const int jb = 2 * pr + jj;
          if (jb < DA) {
            const int j  = mask_b<D>(mask, jb);
            float    *rp = sRaw + (jj * T + p) * RS;
            spline_normalize(rp);
            const float gx = spline_backward(rp, sX[j * T + p], sG[j * T + p], sGl[p]);
            sG[j * T + p]  = gx;
            bf16 *dr = sDr + p * GS + jb * kRawP;
            for (int r = 0; r < kRaw; ++r) dr[r] = __float2bfloat16_rn(rp[r]);
            for (int r = kRaw; r < kRawP; ++r) dr[r] = __float2bfloat16_rn(0.f);
          }
        }
        __syncthreads();
        // b3 gradient: column sums of the FP32 raw gradients
        for (int i = threadIdx.x; i < 2 * kRaw; i += blockDim.x) {
          const int jj = i / kRaw, r = i % kRaw, jb = 2 * pr + jj;
          if (jb < DA) {
            float s = 0.f;
            for (int p = 0; p < T; ++p) s += sRaw[(jj * T + p) * RS + r];
            grad[lo + C::ob3 + jb * kRaw + r] += s;
          }
        }
        __syncthreads();
      }
      // dW3 = H2^T . G_raw: rows (hidden units) in 32-row blocks, warp w takes blocks
      // w, w + 4, ...; columns one coordinate (56) at a time
      for (int rb = warp; rb < H / 32; rb += 4) {
        for (int ch = 0; ch < DA; ++ch) {
          float acc[2][7][4];
#pragma unroll
          for (int a = 0; a < 2; ++a)
#pragma unroll
            for (int i = 0; i < 7; ++i) acc[a][i][0] = acc[a][i][1] = acc[a][i][2] = acc[a][i][3] = 0.f;
#pragma unroll
          for (int kk = 0; kk < T / 16; ++kk) {
            uint32_t  a0[4], a1[4];
            const int kr = kk * 16 + (lane & 7) + (lane >> 4) * 8;
            const int mc = ((lane >> 3) & 1) * 8;
            ldsm4t(a0, sH2 + kr * HS + rb * 32 + mc);
            ldsm4t(a1, sH2 + kr * HS + rb * 32 + 16 + mc);
#pragma unroll
            for (int np = 0; np < 3; ++np) {
              uint32_t b[4];
              ldsm4t(b, sDr + (kk * 16 + (lane & 15)) * GS + ch * kRawP + np * 16 + (lane >> 4) * 8);
              mma16816(acc[0][2 * np], a0, b[0], b[1]);
              mma16816(acc[0][2 * np + 1], a0, b[2], b[3]);
              mma16816(acc[1][2 * np], a1, b[0], b[1]);
              mma16816(acc[1][2 * np + 1], a1, b[2], b[3]);
            }
            uint32_t b0, b1;
            ldsm2t(b0, b1, sDr + (kk * 16 + (lane & 15)) * GS + ch * kRawP + 48);
            mma16816(acc[0][6], a0, b0, b1);
            mma16816(acc[1][6], a1, b0, b1);
          }
#pragma unroll
          for (int a = 0; a < 2; ++a)
#pragma unroll
            for (int nt = 0; nt < 7; ++nt) {
              const int r  = nt * 8 + 2 * tq;
              const int h0 = rb * 32 + a * 16 + g;
              float    *gw = grad + lo + C::oW3 + ch * kRaw;
              if (r < kRaw) {
                gw[h0 * C::NOut + r] += acc[a][nt][0];
                gw[(h0 + 8) * C::NOut + r] += acc[a][nt][2];
              }
              if (r + 1 < kRaw) {
                gw[h0 * C::NOut + r + 1] += acc[a][nt][1];
                gw[(h0 + 8) * C::NOut + r + 1] += acc[a][nt][3];
              }
            }
        }
      }
      __syncthreads();
      // dh2 = (G_raw . W3^T) * [h2 > 0], written over h2 (warp rows m0; 64-column chunks)
      for (int ch = 0; ch < H / 64; ++ch) {
        float acc[8][4];
#pragma unroll
        for (int i = 0; i < 8; ++i) acc[i][0] = acc[i][1] = acc[i][2] = acc[i][3] = 0.f;
#pragma unroll 2
        for (int kk = 0; kk < B::NOutB / 16; ++kk) {
          uint32_t a[4];
          ldsm4(a, sDr + (m0 + (lane & 15)) * GS + kk * 16 + (lane >> 4) * 8);
#pragma unroll
          for (int nt = 0; nt < 8; ++nt) {
            uint32_t b0, b1;
            ldg_b(b0, b1, W3r, B::NOutB, ch * 64 + nt * 8, kk * 16);
            mma16816(acc[nt], a, b0, b1);
          }
        }
#pragma unroll
        for (int nt = 0; nt < 8; ++nt) {
          const int   col = ch * 64 + nt * 8 + 2 * tq;
          const bf16 *h0 = sH2 + (m0 + g) * HS + col, *h1 = sH2 + (m0 + g + 8) * HS + col;
          if (!(__bfloat162float(h0[0]) > 0.f)) acc[nt][0] = 0.f;
          if (!(__bfloat162float(h0[1]) > 0.f)) acc[nt][1] = 0.f;
          if (!(__bfloat162float(h1[0]) > 0.f)) acc[nt][2] = 0.f;
          if (!(__bfloat162float(h1[1]) > 0.f)) acc[nt][3] = 0.f;
          colsum_w<H>(acc[nt], sC2, col);
        }
        __syncwarp();
#pragma unroll
        for (int nt = 0; nt < 8; ++nt) {
          const int col = ch * 64 + nt * 8 + 2 * tq;
          *reinterpret_cast<uint32_t *>(sH2 + (m0 + g) * HS + col) = pack_bf2(acc[nt][0], acc[nt][1]);
          *reinterpret_cast<uint32_t *>(sH2 + (m0 + g + 8) * HS + col) =
              pack_bf2(acc[nt][2], acc[nt][3]);
        }
        __syncwarp();
      }
      __syncthreads();
      for (int c = threadIdx.x; c < H; c += blockDim.x) {  // b2 gradient, warps in order
        float v = 0.f;
        for (int w = 0; w < 4; ++w) v += sC2[w * H + c];
        grad[lo + C::ob2 + c] += v;
      }
      // dW2 = H1^T . dH2: rows (inputs) in 32-row blocks per warp, 64-column chunks
      for (int rb = warp; rb < H / 32; rb += 4) {
        for (int ch = 0; ch < H / 64; ++ch) {
          float acc[2][8][4];
#pragma unroll
          for (int a = 0; a < 2; ++a)
#pragma unroll
            for (int i = 0; i < 8; ++i) acc[a][i][0] = acc[a][i][1] = acc[a][i][2] = acc[a][i][3] = 0.f;
#pragma unroll
          for (int kk = 0; kk < T / 16; ++kk) {
            uint32_t  a0[4], a1[4];
            const int kr = kk * 16 + (lane & 7) + (lane >> 4) * 8;
            const int mc = ((lane >> 3) & 1) * 8;
            ldsm4t(a0, sH1 + kr * HS + rb * 32 + mc);
            ldsm4t(a1, sH1 + kr * HS + rb * 32 + 16 + mc);
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
              const int col = ch * 64 + nt * 8 + 2 * tq;
              const int h0  = rb * 32 + a * 16 + g;
              float    *gw  = grad + lo + C::oW2;
              gw[h0 * H + col] += acc[a][nt][0];
              gw[h0 * H + col + 1] += acc[a][nt][1];
              gw[(h0 + 8) * H + col] += acc[a][nt][2];
              gw[(h0 + 8) * H + col + 1] += acc[a][nt][3];
            }
        }
      }
      // dh1 = (dH2 . W2^T) * [h1 > 0] into sD1 (warp rows m0; 64-column chunks, B from w2r)
      for (int ch = 0; ch < H / 64; ++ch) {
        float acc[8][4];
#pragma unroll
        for (int i = 0; i < 8; ++i) acc[i][0] = acc[i][1] = acc[i][2] = acc[i][3] = 0.f;
#pragma unroll 2
        for (int kk = 0; kk < H / 16; ++kk) {
          uint32_t a[4];
          ldsm4(a, sH2 + (m0 + (lane & 15)) * HS + kk * 16 + (lane >> 4) * 8);
#pragma unroll
          for (int nt = 0; nt < 8; ++nt) {
            uint32_t b0, b1;
            ldg_b(b0, b1, W2r, H, ch * 64 + nt * 8, kk * 16);
            mma16816(acc[nt], a, b0, b1);
          }
        }
#pragma unroll
        for (int nt = 0; nt < 8; ++nt) {
          const int   col = ch * 64 + nt * 8 + 2 * tq;
          const bf16 *h0 = sH1 + (m0 + g) * HS + col, *h1 = sH1 + (m0 + g + 8) * HS + col;
          if (!(__bfloat162float(h0[0]) > 0.f)) acc[nt][0] = 0.f;
          if (!(__bfloat162float(h0[1]) > 0.f)) acc[nt][1] = 0.f;
          if (!(__bfloat162float(h1[0]) > 0.f)) acc[nt][2] = 0.f;
          if (!(__bfloat162float(h1[1]) > 0.f)) acc[nt][3] = 0.f;
          colsum_w<H>(acc[nt], sC1, col);
          *reinterpret_cast<uint32_t *>(sD1 + (m0 + g) * HS + col) = pack_bf2(acc[nt][0], acc[nt][1]);
          *reinterpret_cast<uint32_t *>(sD1 + (m0 + g + 8) * HS + col) =
              pack_bf2(acc[nt][2], acc[nt][3]);
        }
        __syncwarp();
      }
      __syncthreads();
      for (int c = threadIdx.x; c < H; c += blockDim.x) {  // b1 gradient, warps in order
        float v = 0.f;
        for (int w = 0; w < 4; ++w) v += sC1[w * H + c];
        grad[lo + C::ob1 + c] += v;
      }
      // dW1[a][c] = sum_p bf16(x_A[a][p]) dH1[p][c]
      for (int c = threadIdx.x; c < H; c += blockDim.x) {
        float s[DA];
#pragma unroll
        for (int a = 0; a < DA; ++a) s[a] = 0.f;
        for (int p = 0; p < T; ++p) {
          const float d = __bfloat162float(sD1[p * HS + c]);
#pragma unroll
          for (int a = 0; a < DA; ++a) s[a] = fmaf(bfr(sX[mask_a<D>(mask, a) * T + p]), d, s[a]);
        }
#pragma unroll
        for (int a = 0; a < DA; ++a) grad[lo + C::oW1 + a * H + c] += s[a];
      }
      // dx_A[p][a] = sum_c dH1[p][c] bf16(W1[a][c]): point p, coordinates a = ap, ap + 2, ...
      {
        const int p = threadIdx.x % T, ap = threadIdx.x / T;
        for (int a = ap; a < DA; a += 2) {
          float s = 0.f;
          for (int c = 0; c < H; ++c) s = fmaf(__bfloat162float(sD1[p * HS + c]), sW1[a * H + c], s);
          sG[mask_a<D>(mask, a) * T + p] += s;
        }
      }
    }
  }
  for (int o = 16; o > 0; o >>= 1) my_loss += __shfl_down_sync(0xffffffffu, my_loss, o);
  if (lane == 0) sLoss[warp] = my_loss;
  __syncthreads();
  if (threadIdx.x == 0) loss_part[blockIdx.x] = sLoss[0] + sLoss[1] + sLoss[2] + sLoss[3];
}

// ---------------------------------------------------------------------------
// FP32 master weights -> BF16 operand copies of every layer:
//   w2c, w3c  forward chunks: chunk c (64 output columns) in the K-major canonical layout,
//             element (n, k) at (k / 8) 512 + n 8 + k % 8 (W3 chunk j: columns 49 j + r, r < 49)
//   w2t [out][in], w2r [in][out], w3t [56 j + r][h], w3r [h][o < NOutB]
template <int D, int H>
__global__ void k_wpack(const float *__restrict__ theta, int layers, bf16 *__restrict__ w2c,
                        bf16 *__restrict__ w3c, bf16 *__restrict__ w2t, bf16 *__restrict__ w2r,
                        bf16 *__restrict__ w3t, bf16 *__restrict__ w3r) {
  using C = Cfg<D, H>;
  constexpr int NOutB = Bwd<D, H>::NOutB;
  const int64_t n2c = int64_t(layers) * H * H, n3c = int64_t(layers) * C::DA * 64 * H;
  const int64_t n3t = int64_t(layers) * C::NOutP * H, n3r = int64_t(layers) * H * NOutB;
  const int64_t tot = n2c + n3c + 2 * n2c + n3t + n3r;
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < tot;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    int64_t r = i;
    if (r < n2c) {  // w2c
      const int64_t l = r / (H * H);
      const int     q = static_cast<int>(r % (H * H));
      const int     c = q / (64 * H), e = q % (64 * H);
      const int     k = (e / 512) * 8 + e % 8, nn = (e / 8) % 64;
      w2c[r] = __float2bfloat16_rn(theta[l * C::LP + C::oW2 + k * H + c * 64 + nn]);
      continue;
    }
    r -= n2c;
    if (r < n3c) {  // w3c
      const int64_t l = r / (C::DA * 64 * H);
      const int     q = static_cast<int>(r % (C::DA * 64 * H));
      const int     j = q / (64 * H), e = q % (64 * H);
      const int     k = (e / 512) * 8 + e % 8, nn = (e / 8) % 64;
      w3c[r] = __float2bfloat16_rn(nn < kRaw ? theta[l * C::LP + C::oW3 + k * C::NOut + j * kRaw + nn]
                                            : 0.f);
      continue;
    }
    r -= n3c;
    if (r < 2 * n2c) {  // w2t, w2r
      const bool    tr = r < n2c;
      const int64_t q  = tr ? r : r - n2c;
      const int64_t l  = q / (H * H);
      const int     a = static_cast<int>((q % (H * H)) / H), b = static_cast<int>(q % H);
      // w2t[l][a = out][b = in], w2r[l][a = in][b = out]
      const int in = tr ? b : a, out = tr ? a : b;
      (tr ? w2t : w2r)[q] = __float2bfloat16_rn(theta[l * C::LP + C::oW2 + in * H + out]);
      continue;
    }
    r -= 2 * n2c;
    if (r < n3t) {  // w3t[l][o][h]
      const int64_t l = r / (C::NOutP * H);
      const int     q = static_cast<int>(r % (C::NOutP * H));
      const int     o = q / H, h = q % H, j = o / kRawP, rr = o % kRawP;
      w3t[r] = __float2bfloat16_rn(rr < kRaw ? theta[l * C::LP + C::oW3 + h * C::NOut + j * kRaw + rr]
                                            : 0.f);
      continue;
    }
    r -= n3t;
    {  // w3r[l][h][o]
      const int64_t l = r / (H * NOutB);
      const int     q = static_cast<int>(r % (H * NOutB));
      const int     h = q / NOutB, o = q % NOutB, j = o / kRawP, rr = o % kRawP;
      const bool    real = o < C::NOutP && rr < kRaw;
      w3r[r] = __float2bfloat16_rn(real ? theta[l * C::LP + C::oW3 + h * C::NOut + j * kRaw + rr]
                                        : 0.f);
    }
  }
}

template <int D>
__global__ void k_wuniform(uint64_t seed, uint32_t stream, int64_t first, int64_t n, int64_t ld,
                           float *__restrict__ u, float *__restrict__ lq) {
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    double v[D];
    philox_point(seed, stream, static_cast<uint64_t>(first + i), D, v);
#pragma unroll
    for (int j = 0; j < D; ++j) u[j * ld + i] = __double2float_rd(v[j]);
    if (lq) lq[i] = 0.f;
  }
}

}  // namespace wide
}  // namespace flow

// ---------------------------------------------------------------------------
// Launchers of the (D, H) flow kernels.

namespace {

int sm_count_w() {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  return sms;
}

template <int D, int H>
FlowWideSizes sizes_impl(int layers) {
  using C = flow::wide::Cfg<D, H>;
  FlowWideSizes s{};
  s.w2c = size_t(layers) * H * H;
  s.w3c = size_t(layers) * C::DA * 64 * H;
  s.w2t = s.w2r = size_t(layers) * H * H;
  s.w3t = size_t(layers) * C::NOutP * H;
  s.w3r = size_t(layers) * H * flow::wide::Bwd<D, H>::NOutB;
  return s;
}

template <int D, int H>
cudaError_t pack_impl(const float *theta, int layers, const FlowWideBufs &b, cudaStream_t st) {
  flow::wide::k_wpack<D, H><<<4 * sm_count_w(), 256, 0, st>>>(
      theta, layers, static_cast<flow::bf16 *>(b.w2c), static_cast<flow::bf16 *>(b.w3c),
      static_cast<flow::bf16 *>(b.w2t), static_cast<flow::bf16 *>(b.w2r),
      static_cast<flow::bf16 *>(b.w3t), static_cast<flow::bf16 *>(b.w3r));
  return cudaGetLastError();
}

template <int MODE, int D, int H>
cudaError_t forward_impl(const float *theta, const FlowWideBufs &b, int layers, const float *xin,
                         int64_t ld_in, int64_t n, uint64_t seed, uint32_t stream, int64_t first,
                         float *xout, int64_t ld_out, float *lq, float *xs_store, int *err,
                         cudaStream_t st) {
  using C = flow::wide::Cfg<D, H>;
  const int64_t nsub = (n + 255) / 256;
  const int     grid = static_cast<int>(std::min<int64_t>(nsub, sm_count_w()));
  const int     sm   = static_cast<int>(C::kFwdSmem);
  cudaFuncSetAttribute(flow::wide::k_wfwd<MODE, D, H>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       sm);
  flow::wide::k_wfwd<MODE, D, H><<<grid, 256, sm, st>>>(
      theta, static_cast<const flow::bf16 *>(b.w2c), static_cast<const flow::bf16 *>(b.w3c),
      layers, xin, ld_in, n, seed, stream, first, xout, ld_out, lq, xs_store, err);
  return cudaGetLastError();
}

template <int D, int H>
cudaError_t backward_impl(const float *theta, const FlowWideBufs &b, int layers, const float *xs,
                          const float *lq, const float *coef, int64_t n, int kind, float *part,
                          double *loss_part, float *grad, double *loss, cudaStream_t st) {
  using C = flow::wide::Cfg<D, H>;
  using B = flow::wide::Bwd<D, H>;
  const int64_t tiles = (n + B::T - 1) / B::T;
  const int     grid  = static_cast<int>(std::min<int64_t>(tiles, sm_count_w()));
  const int64_t np    = static_cast<int64_t>(layers) * C::LP;
  cudaError_t   e = cudaMemsetAsync(part, 0, static_cast<size_t>(grid) * np * sizeof(float), st);
  if (e != cudaSuccess) return e;
  cudaFuncSetAttribute(flow::wide::k_wbwd<D, H>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       int(B::kSmem));
  flow::wide::k_wbwd<D, H><<<grid, 128, B::kSmem, st>>>(
      theta, static_cast<const flow::bf16 *>(b.w2t), static_cast<const flow::bf16 *>(b.w2r),
      static_cast<const flow::bf16 *>(b.w3t), static_cast<const flow::bf16 *>(b.w3r), layers, xs,
      lq, coef, n, kind, 1.0f / static_cast<float>(n), part, loss_part);
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  return launch_flow_grad_reduce(part, grid, np, grad, loss_part, loss, st);
}

}  // namespace

// The shapes built here: (8, 256), (12, 128), (12, 256), (14, 128), (14, 256).
#define GRN_WIDE_SHAPES(X) X(8, 256) X(12, 128) X(12, 256) X(14, 128) X(14, 256)

bool flow_wide_supported(int dim, int hidden) {
#define GRN_X(d, h) if (dim == d && hidden == h) return true;
  GRN_WIDE_SHAPES(GRN_X)
#undef GRN_X
  return false;
}

int64_t flow_layer_params(int dim, int hidden) {
  const int64_t a = dim / 2, o = a * flow::kRaw;
  return a * hidden + hidden + int64_t(hidden) * hidden + hidden + hidden * o + o;
}

FlowWideSizes flow_wide_sizes(int dim, int hidden, int layers) {
#define GRN_X(d, h) if (dim == d && hidden == h) return sizes_impl<d, h>(layers);
  GRN_WIDE_SHAPES(GRN_X)
#undef GRN_X
  return FlowWideSizes{};
}

cudaError_t launch_wflow_pack(int dim, int hidden, const float *theta, int layers,
                              const FlowWideBufs &b, cudaStream_t st) {
#define GRN_X(d, h) if (dim == d && hidden == h) return pack_impl<d, h>(theta, layers, b, st);
  GRN_WIDE_SHAPES(GRN_X)
#undef GRN_X
  return cudaErrorInvalidValue;
}

cudaError_t launch_wflow_forward(int dim, int hidden, int mode, const float *theta,
                                 const FlowWideBufs &b, int layers, const float *xin,
                                 int64_t ld_in, int64_t n, uint64_t seed, uint32_t stream,
                                 int64_t first, float *xout, int64_t ld_out, float *lq,
                                 float *xs_store, int *err, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
#define GRN_X(d, h)                                                                           \
  if (dim == d && hidden == h)                                                                \
    return mode == 0 ? forward_impl<0, d, h>(theta, b, layers, xin, ld_in, n, seed, stream,   \
                                             first, xout, ld_out, lq, xs_store, err, st)      \
                     : forward_impl<1, d, h>(theta, b, layers, xin, ld_in, n, seed, stream,   \
                                             first, xout, ld_out, lq, xs_store, err, st);
  GRN_WIDE_SHAPES(GRN_X)
#undef GRN_X
  return cudaErrorInvalidValue;
}

cudaError_t launch_wflow_backward(int dim, int hidden, const float *theta, const FlowWideBufs &b,
                                  int layers, const float *xs, const float *lq,
                                  const float *coef, int64_t n, int kind, float *part,
                                  double *loss_part, float *grad, double *loss,
                                  cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
#define GRN_X(d, h)                                                                         \
  if (dim == d && hidden == h)                                                              \
    return backward_impl<d, h>(theta, b, layers, xs, lq, coef, n, kind, part, loss_part,   \
                               grad, loss, st);
  GRN_WIDE_SHAPES(GRN_X)
#undef GRN_X
  return cudaErrorInvalidValue;
}

cudaError_t launch_flow_uniform_dim(int dim, uint64_t seed, uint32_t stream, int64_t first,
                                    int64_t n, int64_t ld, float *u, float *lq, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  if (dim == 8) return launch_flow_uniform(seed, stream, first, n, ld, u, lq, st);
  if (dim == 12)
    flow::wide::k_wuniform<12><<<4 * sm_count_w(), 256, 0, st>>>(seed, stream, first, n, ld, u,
                                                                  lq);
  else if (dim == 14)
    flow::wide::k_wuniform<14><<<4 * sm_count_w(), 256, 0, st>>>(seed, stream, first, n, ld, u,
                                                                  lq);
  else
    return cudaErrorInvalidValue;
  return cudaGetLastError();
}

}  // namespace grn
