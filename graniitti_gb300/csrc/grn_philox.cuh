// grn_philox.cuh — counter-based uniforms shared by the physics and flow kernels.
#pragma once

#include <cstdint>

namespace grn {

// Philox4x32-10 (Salmon et al., SC'11). counter = (index lo, index hi, block,
// stream), key = seed. Each block gives two 53-bit doubles in [0, 1).
__device__ __forceinline__ void philox_block(uint64_t seed, uint32_t stream, uint64_t idx,
                                             uint32_t blk, double &r0, double &r1) {
  uint32_t c0 = static_cast<uint32_t>(idx), c1 = static_cast<uint32_t>(idx >> 32), c2 = blk,
           c3 = stream;
  uint32_t k0 = static_cast<uint32_t>(seed), k1 = static_cast<uint32_t>(seed >> 32);
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    const uint32_t hi0 = __umulhi(0xD2511F53u, c0), lo0 = 0xD2511F53u * c0;
    const uint32_t hi1 = __umulhi(0xCD9E8D57u, c2), lo1 = 0xCD9E8D57u * c2;
    const uint32_t n0 = hi1 ^ c1 ^ k0;
    const uint32_t n2 = hi0 ^ c3 ^ k1;
    c0 = n0;
    c1 = lo1;
    c2 = n2;
    c3 = lo0;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  const uint64_t a = (static_cast<uint64_t>(c1) << 32) | c0;
  const uint64_t b = (static_cast<uint64_t>(c3) << 32) | c2;
  r0 = static_cast<double>(a >> 11) * 0x1.0p-53;
  r1 = static_cast<double>(b >> 11) * 0x1.0p-53;
}

__device__ __forceinline__ void philox_point(uint64_t seed, uint32_t stream, uint64_t idx,
                                             int dim, double *u) {
  for (int blk = 0; 2 * blk < dim; ++blk) {
    double r0, r1;
    philox_block(seed, stream, idx, blk, r0, r1);
    u[2 * blk] = r0;
    if (2 * blk + 1 < dim) u[2 * blk + 1] = r1;
  }
}

}  // namespace grn
