// Stable LSD radix sort of (uint32 key, int32 value) pairs, 8 bits per pass.
// Each pass: per-tile digit histograms (digit-major), one device-wide exclusive scan, and a
// stable scatter in which every tile ranks its keys round by round (warp match + per-warp
// digit counts in shared memory). Used to order points spatially on the device.
#include "tsne.cuh"

namespace fe {

constexpr int kRadixThreads = 256;
constexpr int kRadixItems = 16;
constexpr int kRadixTile = kRadixThreads * kRadixItems;
constexpr int kRadixWarps = kRadixThreads / 32;

int radix_sort_blocks(int n) { return std::max(1, ceil_div(n, kRadixTile)); }

__global__ void __launch_bounds__(kRadixThreads)
radix_hist_kernel(const unsigned* __restrict__ keys, int n, int shift, int* __restrict__ hist) {
  __shared__ int cnt[256];
  cnt[threadIdx.x] = 0;
  __syncthreads();
  const int base = blockIdx.x * kRadixTile;
  for (int t = threadIdx.x; t < kRadixTile; t += kRadixThreads) {
    const int i = base + t;
    if (i < n) atomicAdd(&cnt[(keys[i] >> shift) & 255u], 1);
  }
  __syncthreads();
  hist[threadIdx.x * gridDim.x + blockIdx.x] = cnt[threadIdx.x];
}

__global__ void __launch_bounds__(kRadixThreads)
radix_scatter_kernel(const unsigned* __restrict__ keys, const int* __restrict__ vals, int n, int shift,
                     const long long* __restrict__ offs, unsigned* __restrict__ keys_out, int* __restrict__ vals_out) {
  __shared__ int running[256];
  __shared__ int wcnt[kRadixWarps][256];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  running[threadIdx.x] = 0;
  const int base = blockIdx.x * kRadixTile;
  for (int round = 0; round < kRadixItems; ++round) {
    for (int t = threadIdx.x; t < kRadixWarps * 256; t += kRadixThreads) (&wcnt[0][0])[t] = 0;
    __syncthreads();
    const int i = base + round * kRadixThreads + threadIdx.x;
    const bool valid = i < n;
    const unsigned key = valid ? keys[i] : 0u;
    const int digit = valid ? (int)((key >> shift) & 255u) : 256 + lane;  // invalid lanes never match
    const unsigned peers = __match_any_sync(0xffffffffu, digit);
    const int rank = __popc(peers & ((1u << lane) - 1u));
    if (valid && lane == __ffs(peers) - 1) wcnt[warp][digit] = __popc(peers);
    __syncthreads();
    if (valid) {
      int pre = 0;
      for (int w = 0; w < warp; ++w) pre += wcnt[w][digit];
      const long long dest = offs[(long long)digit * gridDim.x + blockIdx.x] + running[digit] + pre + rank;
      keys_out[dest] = key;
      vals_out[dest] = vals[i];
    }
    __syncthreads();
    int tot = 0;
    for (int w = 0; w < kRadixWarps; ++w) tot += wcnt[w][threadIdx.x];
    running[threadIdx.x] += tot;
    __syncthreads();
  }
}

void radix_sort_pairs(unsigned* keys, int* vals, unsigned* keys_tmp, int* vals_tmp, int n, int bits,
                      const RadixWorkspace& ws, cudaStream_t s) {
  const int nb = radix_sort_blocks(n);
  unsigned *ka = keys, *kb = keys_tmp;
  int *va = vals, *vb = vals_tmp;
  int passes = 0;
  for (int shift = 0; shift < bits; shift += 8, ++passes) {
    radix_hist_kernel<<<nb, kRadixThreads, 0, s>>>(ka, n, shift, ws.hist);
    FE_LAUNCH("radix_hist_kernel");
    exclusive_scan(ws.hist, ws.offs, 256 * nb, ws.scan_tmp, s);
    radix_scatter_kernel<<<nb, kRadixThreads, 0, s>>>(ka, va, n, shift, ws.offs, kb, vb);
    FE_LAUNCH("radix_scatter_kernel");
    std::swap(ka, kb);
    std::swap(va, vb);
  }
  if (passes & 1) {
    FE_CUDA(cudaMemcpyAsync(keys, ka, sizeof(unsigned) * n, cudaMemcpyDeviceToDevice, s));
    FE_CUDA(cudaMemcpyAsync(vals, va, sizeof(int) * n, cudaMemcpyDeviceToDevice, s));
  }
}

}  // namespace fe
