// Block-level sorting primitive shared by the graph builders (t-SNE P, UMAP fuzzy graph).
#pragma once

#include <cuda_runtime.h>

namespace fe {

// Always-ascending bitonic network over `pw` (power of two) slots; compare(i, j) keeps the
// minimum at i. Slots at or beyond `len` hold +inf (explicitly in shared memory, virtually
// in global memory), which this formulation never moves below a real key.
template <bool kGlobal>
__device__ __forceinline__ void bitonic_sort(unsigned long long* a, int len, int pw) {
  for (int size = 2; size <= pw; size <<= 1) {
    const int half = size >> 1;
    for (int t = threadIdx.x; t < pw / 2; t += blockDim.x) {
      const int blk = t / half, off = t % half;
      const int i = blk * size + off, j = blk * size + size - 1 - off;
      if (!kGlobal || j < len) {
        const unsigned long long x = a[i], y = a[j];
        if (y < x) {
          a[i] = y;
          a[j] = x;
        }
      }
    }
    __syncthreads();
    for (int stride = half >> 1; stride > 0; stride >>= 1) {
      for (int t = threadIdx.x; t < pw / 2; t += blockDim.x) {
        const int blk = t / stride, off = t % stride;
        const int i = blk * 2 * stride + off, j = i + stride;
        if (!kGlobal || j < len) {
          const unsigned long long x = a[i], y = a[j];
          if (y < x) {
            a[i] = y;
            a[j] = x;
          }
        }
      }
      __syncthreads();
    }
  }
}

}  // namespace fe
