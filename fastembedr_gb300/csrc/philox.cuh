// Counter-based random numbers: Philox4x32 with 10 rounds, as published by Salmon, Moraes,
// Dror and Shaw, "Parallel random numbers: as easy as 1, 2, 3" (SC 2011). Each thread owns a
// stream by putting its id in the counter, so draws are reproducible for any launch shape.
#pragma once

#include <cuda_runtime.h>

namespace fe {

__host__ __device__ __forceinline__ unsigned mulhi32(unsigned a, unsigned b) {
#ifdef __CUDA_ARCH__
  return __umulhi(a, b);
#else
  return (unsigned)(((unsigned long long)a * b) >> 32);
#endif
}

__host__ __device__ __forceinline__ uint4 philox4x32_10(uint4 c, uint2 k) {
  const unsigned M0 = 0xD2511F53u, M1 = 0xCD9E8D57u, W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    const unsigned hi0 = mulhi32(M0, c.x), lo0 = M0 * c.x;
    const unsigned hi1 = mulhi32(M1, c.z), lo1 = M1 * c.z;
    c = make_uint4(hi1 ^ c.y ^ k.x, lo1, hi0 ^ c.w ^ k.y, lo0);
    k.x += W0;
    k.y += W1;
  }
  return c;
}

// uniform in (0, 1) from the top 24 bits
__host__ __device__ __forceinline__ float u01(unsigned x) {
  return ((float)(x >> 8) + 0.5f) * (1.0f / 16777216.0f);
}

// uniform integer in [0, n) by multiply-shift
__host__ __device__ __forceinline__ unsigned bounded(unsigned x, unsigned n) {
  return (unsigned)(((unsigned long long)x * n) >> 32);
}

}  // namespace fe
