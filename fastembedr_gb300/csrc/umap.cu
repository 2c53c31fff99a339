// UMAP on the GPU: the fuzzy-union graph built from a supplied KNN graph and the SGD epochs.
//
// Reference behaviour followed (fastEmbedR):
//   - smooth_knn_dist, src/fast_knn_umap.cpp:876-1003 (rho = smallest positive distance,
//     sigma bisection to log2(k), best-diff kept, sigma floor 1e-3 * mean distance);
//   - build_graph_csr_native_direct_values, :1562-1780 with compact_directed_rows_inplace
//     (:1284-1365) and attach_csr_epoch_schedule (:1264-1282): directed weights
//     exp(-(d - rho) / sigma), duplicates kept at their maximum, union f + r - f r, entries
//     <= 1e-6 dropped, epochs_per_sample = max_w / max(w, 1e-6);
//   - the COO epoch of fastembedr_cuda_umap_optimize_coo, src/embedding_cuda_kernels.cpp:5483-5608
//     (positive/negative schedules :3044-3084, attractive/repulsive coefficients with the
//     Schraudolph power :364-407, gradient clip 4, linear learning-rate decay, clamp to +-16
//     after each epoch, epoch 0 inactive).
// GB300 layout: the graph is built by the same row-bucket + bitonic sort machinery as the
// t-SNE P; the epoch is one persistent grid-stride kernel over head-sorted COO edges with float2
// vector atomics, negative samples drawn from per-(edge, epoch) Philox4x32-10 streams, and the
// epoch counter lives on the device so a captured CUDA graph of 25 epochs replays unchanged.
#include <algorithm>
#include <cfloat>
#include <climits>
#include <cmath>
#include <future>
#include <map>
#include <memory>
#include <type_traits>
#include <vector>

#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_segmented_radix_sort.cuh>

#include "../../include/fastembedr_cuda.h"
#include "philox.cuh"
#include "sort.cuh"
#include "tsne.cuh"
#include "umap_spectral.cuh"

namespace fe {

// ---------------------------------------------------------------- smooth kNN
__global__ void umap_distance_sum_kernel(const float* __restrict__ dist, long long total, double* __restrict__ acc) {
  double s = 0.0;
  unsigned long long c = 0;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total; t += (long long)gridDim.x * blockDim.x) {
    const float d = dist[t];
    if (isfinite(d) && d >= 0.0f) {
      s += (double)d;
      ++c;
    }
  }
  s = warp_sum(s);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
  if ((threadIdx.x & 31) == 0) {
    atomicAdd(acc, s);
    atomicAdd(reinterpret_cast<unsigned long long*>(acc + 1), c);
  }
}

constexpr int kSmoothRows = 128;

// Membership sum of one row at sigma, in the reference's order and FP64 arithmetic
// (smooth_knn_dist's membership_sum, src/fast_knn_umap.cpp:924-934).
__device__ double smooth_psum_exact(const float* __restrict__ d, int k, double rho, double sigma) {
  const double safe = fmax(sigma, 1.0e-12);
  double psum = 0.0;
  for (int j = 0; j < k; ++j) {
    const float raw = d[j];
    if (!isfinite(raw)) continue;
    const double x = (double)raw - rho;
    psum += x <= 0.0 ? 1.0 : exp(-x / safe);
  }
  return psum;
}

// The reference's sigma search for one row (:961-985) in FP64 throughout.
__device__ double smooth_sigma_exact(const float* __restrict__ d, int k, double rho, double target) {
  double sigma = 1.0, best = 1.0, best_diff = DBL_MAX, lo = 0.0, hi = DBL_MAX;
  for (int it = 0; it < 64; ++it) {
    const double psum = smooth_psum_exact(d, k, rho, sigma);
    const double diff = fabs(psum - target);
    if (diff < best_diff) {
      best_diff = diff;
      best = sigma;
    }
    if (psum > target) {
      hi = sigma;
      sigma = 0.5 * (lo + hi);
    } else {
      lo = sigma;
      sigma = hi == DBL_MAX ? sigma * 2.0 : 0.5 * (lo + hi);
    }
    if (diff < 1.0e-5) break;
  }
  return best;
}

// smooth_knn_dist (:876-996), one thread per row; distances column-major n x k, staged through
// shared memory (blockDim.x rows x (k + 1) raw distances, then as many positive offsets d - rho).
// The search runs its membership sums on the FP32 pipe: exp of float offsets times a float
// 1/sigma, Kahan-summed. Each FP32 term is within 2e-7 of the FP64 term and the Kahan sum adds
// at most 1.2e-7 per unit of the total, so |psum32 - psum64| < 4e-7 k. The decisions of the
// search are the sign of psum - target and the stop test |psum - target| < 1e-5; an FP32 sum
// farther than that margin from the stop boundary takes both as FP64 would (a sum inside the
// stop band stops either way), and one inside the margin is re-evaluated in FP64. The FP64
// search keeps the sigma of the smallest |psum - target|, which at a stop is the stopping sigma
// (every earlier difference was >= 1e-5), so the result is the FP64 search's. A row that does not
// stop within 64 steps is searched again in FP64 from the start.
__global__ void __launch_bounds__(kSmoothRows)
umap_smooth_knn_kernel(const float* __restrict__ dist, int n, int k, const double* __restrict__ acc,
                       float* __restrict__ sigmas, float* __restrict__ rhos) {
  extern __shared__ float s_tile[];
  const int rows = blockDim.x, stride = k + 1;
  float* s_off = s_tile + (long long)rows * stride;
  const int r0 = blockIdx.x * rows;
  const int nrows = min(rows, n - r0);
  for (int t = threadIdx.x; t < nrows * k; t += rows) {
    const int j = t / nrows, rr = t - j * nrows;
    s_tile[rr * stride + j] = dist[(long long)j * n + r0 + rr];
  }
  __syncthreads();
  const int rr = threadIdx.x;
  if (rr >= nrows) return;
  const float* d = s_tile + rr * stride;
  float* off = s_off + rr * stride;
  const unsigned long long cnt = reinterpret_cast<const unsigned long long*>(acc)[1];
  const double global_mean = cnt > 0 ? acc[0] / (double)cnt : 1.0;
  const double target = log2((double)k);
  double rho = INFINITY, row_sum = 0.0;
  int row_count = 0;
  for (int j = 0; j < k; ++j) {
    const float v = d[j];
    if (!isfinite(v)) continue;
    if (v >= 0.0f) {
      row_sum += (double)v;
      ++row_count;
    }
    if (v > 0.0f && (double)v < rho) rho = (double)v;
  }
  if (!isfinite(rho)) rho = 0.0;
  // finite entries at or below rho contribute exactly 1; the others their float offset, which
  // is positive (the difference of two distinct floats does not round to zero in FP32)
  int ones = 0, m = 0;
  for (int j = 0; j < k; ++j) {
    const float v = d[j];
    if (!isfinite(v)) continue;
    const double x = (double)v - rho;
    if (x <= 0.0) ++ones;
    else off[m++] = (float)x;
  }
  const double margin = 4.0e-7 * (double)k;
  double sigma = 1.0, best = 1.0, lo = 0.0, hi = DBL_MAX;
  bool stopped = false;
  for (int it = 0; it < 64; ++it) {
    const float inv = (float)(1.0 / fmax(sigma, 1.0e-12));
    float ps = (float)ones, pc = 0.0f;
    for (int j = 0; j < m; ++j) {
      const float y = expf(-off[j] * inv) - pc;
      const float t = ps + y;
      pc = (t - ps) - y;
      ps = t;
    }
    double psum = (double)ps - (double)pc;
    double diff = fabs(psum - target);
    if (fabs(diff - 1.0e-5) < margin) {
      psum = smooth_psum_exact(d, k, rho, sigma);
      diff = fabs(psum - target);
    }
    if (diff < 1.0e-5) {
      best = sigma;
      stopped = true;
      break;
    }
    if (psum > target) {
      hi = sigma;
      sigma = 0.5 * (lo + hi);
    } else {
      lo = sigma;
      sigma = hi == DBL_MAX ? sigma * 2.0 : 0.5 * (lo + hi);
    }
  }
  if (!stopped) best = smooth_sigma_exact(d, k, rho, target);
  const double row_mean = row_count > 0 ? row_sum / (double)row_count : global_mean;
  const double floor_s = 1.0e-3 * (rho > 0.0 ? row_mean : global_mean);
  best = fmax(best, floor_s);
  rhos[r0 + rr] = (float)rho;
  sigmas[r0 + rr] = (float)fmax(best, 1.0e-12);
}

void smooth_knn(const float* d_dist, int n, int k, const double* acc, float* sig, float* rho, cudaStream_t s) {
  int rows = kSmoothRows;
  while (rows > 1 && (std::size_t)rows * (k + 1) * 2 * sizeof(float) > 96 * 1024) rows >>= 1;
  const std::size_t smem = (std::size_t)rows * (k + 1) * 2 * sizeof(float);
  if (smem > 200 * 1024) throw Error("k is too large for the UMAP smooth-kNN search (at most 25,000 neighbours)");
  if (smem > 48 * 1024)
    FE_CUDA(cudaFuncSetAttribute(umap_smooth_knn_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  umap_smooth_knn_kernel<<<ceil_div(n, rows), rows, smem, s>>>(d_dist, n, k, acc, sig, rho);
  FE_LAUNCH("umap_smooth_knn_kernel");
}

// ---------------------------------------------------------------- fuzzy union graph
__device__ __forceinline__ bool directed_weight(const int* __restrict__ idx, const float* __restrict__ dist,
                                                const float* __restrict__ sig, const float* __restrict__ rho,
                                                int n, int offset, long long t, int& i, int& nb, float& w) {
  i = (int)(t % n);
  nb = idx[t] - offset;
  const float d = dist[t];
  if (nb < 0 || nb >= n || nb == i || !isfinite(d)) return false;
  w = d <= rho[i] ? 1.0f : expf(-(d - rho[i]) / sig[i]);
  return isfinite(w) && w > 0.0f;
}

__global__ void umap_count_kernel(const int* __restrict__ idx, const float* __restrict__ dist,
                                  const float* __restrict__ sig, const float* __restrict__ rho, int n, int k, int offset,
                                  int* __restrict__ counts) {
  const long long total = (long long)n * k;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total; t += (long long)gridDim.x * blockDim.x) {
    int i, nb;
    float w;
    if (!directed_weight(idx, dist, sig, rho, n, offset, t, i, nb, w)) continue;
    atomicAdd(counts + i, 1);
    atomicAdd(counts + nb, 1);
  }
}

// bucket key: column (high word), direction bit 31 (0 = i -> col, 1 = col -> i), weight bits
__global__ void umap_fill_kernel(const int* __restrict__ idx, const float* __restrict__ dist,
                                 const float* __restrict__ sig, const float* __restrict__ rho, int n, int k, int offset,
                                 unsigned long long* __restrict__ cursor, unsigned long long* __restrict__ bucket) {
  const long long total = (long long)n * k;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total; t += (long long)gridDim.x * blockDim.x) {
    int i, nb;
    float w;
    if (!directed_weight(idx, dist, sig, rho, n, offset, t, i, nb, w)) continue;
    const unsigned long long wb = (unsigned long long)__float_as_uint(w);
    bucket[atomicAdd(cursor + i, 1ull)] = ((unsigned long long)(unsigned)nb << 32) | wb;
    bucket[atomicAdd(cursor + nb, 1ull)] = ((unsigned long long)(unsigned)i << 32) | 0x80000000ull | wb;
  }
}

// Forward / reverse weights of one column run [t, end): the maximum per direction (duplicates
// of a directed edge keep their maximum), then the fuzzy union.
__device__ __forceinline__ float union_weight(const unsigned long long* a, int t, int len, unsigned col, int* end) {
  float f = 0.0f, r = 0.0f;
  int u = t;
  for (; u < len && (unsigned)(a[u] >> 32) == col; ++u) {
    const unsigned lo = (unsigned)a[u];
    const float w = __uint_as_float(lo & 0x7fffffffu);
    if (lo & 0x80000000u) r = fmaxf(r, w);
    else f = fmaxf(f, w);
  }
  *end = u;
  return f + r - f * r;
}

constexpr int kUmapSortThreads = 256;
constexpr int kUmapSortCap = 4096;

__global__ void __launch_bounds__(kUmapSortThreads)
umap_union_rows_kernel(unsigned long long* __restrict__ bucket, const long long* __restrict__ offs, int n,
                       int* __restrict__ ucount, float* __restrict__ row_max, int* __restrict__ big_rows,
                       int* __restrict__ big_count) {
  extern __shared__ unsigned long long sm[];
  __shared__ int warp_cnt[kUmapSortThreads / 32];
  __shared__ float s_wmax[kUmapSortThreads / 32];
  for (int row = blockIdx.x; row < n; row += gridDim.x) {
    const long long b = offs[row];
    const int len = (int)(offs[row + 1] - b);
    if (len > kUmapSortCap) {
      if (threadIdx.x == 0) big_rows[atomicAdd(big_count, 1)] = row;
      continue;
    }
    int pw = 1;
    while (pw < len) pw <<= 1;
    for (int t = threadIdx.x; t < pw; t += blockDim.x) sm[t] = t < len ? bucket[b + t] : ~0ull;
    __syncthreads();
    if (len > 1) bitonic_sort<false>(sm, len, pw);
    int kept_before = 0;
    float mymax = 0.0f;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int base = 0; base < len; base += blockDim.x) {
      const int t = base + threadIdx.x;
      bool keep = false;
      float w = 0.0f;
      unsigned col = 0u;
      if (t < len && (t == 0 || (sm[t] >> 32) != (sm[t - 1] >> 32))) {
        col = (unsigned)(sm[t] >> 32);
        int end;
        w = union_weight(sm, t, len, col, &end);
        keep = isfinite(w) && w > 1.0e-6f;
      }
      const unsigned ballot = __ballot_sync(0xffffffffu, keep);
      if (lane == 0) warp_cnt[warp] = __popc(ballot);
      __syncthreads();
      int before = 0, total = 0;
      for (int wi = 0; wi < (int)(blockDim.x / 32); ++wi) {
        if (wi < warp) before += warp_cnt[wi];
        total += warp_cnt[wi];
      }
      if (keep) {
        const int pos = kept_before + before + __popc(ballot & ((1u << lane) - 1u));
        bucket[b + pos] = ((unsigned long long)col << 32) | (unsigned long long)__float_as_uint(w);
        mymax = fmaxf(mymax, w);
      }
      kept_before += total;
      __syncthreads();
    }
    const float m = warp_max(mymax);
    if (lane == 0) s_wmax[warp] = m;
    __syncthreads();
    if (threadIdx.x == 0) {
      float mm = 0.0f;
      for (int wi = 0; wi < (int)(blockDim.x / 32); ++wi) mm = fmaxf(mm, s_wmax[wi]);
      row_max[row] = mm;
      ucount[row] = kept_before;
    }
    __syncthreads();
  }
}

__global__ void __launch_bounds__(1024)
umap_union_big_rows_kernel(unsigned long long* __restrict__ bucket, const long long* __restrict__ offs,
                           const int* __restrict__ big_rows, const int* __restrict__ big_count,
                           int* __restrict__ ucount, float* __restrict__ row_max) {
  const int count = *big_count;
  for (int r = blockIdx.x; r < count; r += gridDim.x) {
    const int row = big_rows[r];
    const long long b = offs[row];
    const int len = (int)(offs[row + 1] - b);
    int pw = 1;
    while (pw < len) pw <<= 1;
    bitonic_sort<true>(bucket + b, len, pw);
    if (threadIdx.x == 0) {
      int w_out = 0;
      float mm = 0.0f;
      for (int t = 0; t < len;) {
        const unsigned col = (unsigned)(bucket[b + t] >> 32);
        int end;
        const float w = union_weight(bucket + b, t, len, col, &end);
        t = end;
        if (isfinite(w) && w > 1.0e-6f) {
          bucket[b + w_out++] = ((unsigned long long)col << 32) | (unsigned long long)__float_as_uint(w);
          mm = fmaxf(mm, w);
        }
      }
      ucount[row] = w_out;
      row_max[row] = mm;
    }
    __syncthreads();
  }
}

__global__ void umap_max_kernel(const float* __restrict__ row_max, int n, float* __restrict__ out) {
  __shared__ float part[1024];
  float m = 0.0f;
  for (int i = threadIdx.x; i < n; i += blockDim.x) m = fmaxf(m, row_max[i]);
  part[threadIdx.x] = m;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) part[threadIdx.x] = fmaxf(part[threadIdx.x], part[threadIdx.x + w]);
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = part[0];
}

__global__ void umap_fill_csr_kernel(const unsigned long long* __restrict__ bucket, const long long* __restrict__ offs,
                                     const long long* __restrict__ out64, int n, const float* __restrict__ max_w,
                                     int* __restrict__ offsets, int* __restrict__ heads, int* __restrict__ neighbors,
                                     float* __restrict__ weights, float* __restrict__ eps) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (warp > n) return;
  if (lane == 0) offsets[warp] = (int)out64[warp];
  if (warp == n) return;
  const float mw = *max_w;
  const long long src = offs[warp], dst = out64[warp];
  const int cnt = (int)(out64[warp + 1] - dst);
  for (int t = lane; t < cnt; t += 32) {
    const unsigned long long e = bucket[src + t];
    const float w = __uint_as_float((unsigned)e);
    if (heads) heads[dst + t] = warp;
    neighbors[dst + t] = (int)(e >> 32);
    weights[dst + t] = w;
    eps[dst + t] = mw > 0.0f ? mw / fmaxf(w, 1.0e-6f) : INFINITY;
  }
}

// Device fuzzy graph (CSR, ascending neighbours, plus the COO heads used by the epoch kernel).
struct UmapGraph {
  int n = 0;
  long long nnz = 0;
  float max_weight = 0.0f;
  int* offsets = nullptr;
  int* heads = nullptr;
  int* neighbors = nullptr;
  float* weights = nullptr;
  float* eps = nullptr;
  Arena arena;
};

// Workspace of the fuzzy-graph build for instances of up to cap_n points with k neighbours. A
// batch reuses one workspace for every instance, in stream order.
struct UmapGraphWork {
  int cap_n = 0, k = 0;
  float *sig = nullptr, *rho = nullptr, *row_max = nullptr, *d_max = nullptr;
  double* acc = nullptr;
  int *counts = nullptr, *ucount = nullptr, *big_rows = nullptr, *big_count = nullptr;
  long long *offs = nullptr, *scan_tmp = nullptr, *out64 = nullptr;
  unsigned long long *cursor = nullptr, *bucket = nullptr;
  Arena arena;

  void alloc(int max_n, int kk) {
    cap_n = max_n;
    k = kk;
    const long long directed = (long long)max_n * k;
    arena.reserve(&sig, max_n);
    arena.reserve(&rho, max_n);
    arena.reserve(&row_max, max_n);
    arena.reserve(&d_max, 1);
    arena.reserve(&acc, 2);
    arena.reserve(&counts, max_n);
    arena.reserve(&ucount, max_n);
    arena.reserve(&big_rows, max_n);
    arena.reserve(&big_count, 1);
    arena.reserve(&offs, max_n + 1);
    arena.reserve(&scan_tmp, std::max(1, ceil_div(max_n, 1024)));
    arena.reserve(&out64, max_n + 1);
    arena.reserve(&cursor, max_n);
    arena.reserve(&bucket, 2 * directed);
    arena.commit("UMAP graph workspace");
  }

  // Enqueues the build of one instance (n <= cap_n) up to its union rows: out64 holds the row
  // offsets of the union graph (out64[n] = its entry count), d_max its largest weight, and the
  // rows' entries sit in bucket at offs.
  void enqueue(const int* d_idx, const float* d_dist, int n, int offset, cudaStream_t s) {
    const long long directed = (long long)n * k;
    const int grid = std::max(1, std::min(ceil_div(directed, 256), sm_count() * 16));
    FE_CUDA(cudaMemsetAsync(acc, 0, 2 * sizeof(double), s));
    FE_CUDA(cudaMemsetAsync(counts, 0, sizeof(int) * n, s));
    FE_CUDA(cudaMemsetAsync(big_count, 0, sizeof(int), s));
    umap_distance_sum_kernel<<<grid, 256, 0, s>>>(d_dist, directed, acc);
    FE_LAUNCH("umap_distance_sum_kernel");
    smooth_knn(d_dist, n, k, acc, sig, rho, s);
    umap_count_kernel<<<grid, 256, 0, s>>>(d_idx, d_dist, sig, rho, n, k, offset, counts);
    FE_LAUNCH("umap_count_kernel");
    exclusive_scan(counts, offs, n, scan_tmp, s);
    FE_CUDA(cudaMemcpyAsync(cursor, offs, sizeof(long long) * n, cudaMemcpyDeviceToDevice, s));
    umap_fill_kernel<<<grid, 256, 0, s>>>(d_idx, d_dist, sig, rho, n, k, offset, cursor, bucket);
    FE_LAUNCH("umap_fill_kernel");
    const std::size_t smem = kUmapSortCap * sizeof(unsigned long long);
    FE_CUDA(cudaFuncSetAttribute(umap_union_rows_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    umap_union_rows_kernel<<<std::min(n, sm_count() * 8), kUmapSortThreads, smem, s>>>(bucket, offs, n, ucount,
                                                                                       row_max, big_rows, big_count);
    FE_LAUNCH("umap_union_rows_kernel");
    umap_union_big_rows_kernel<<<sm_count(), 1024, 0, s>>>(bucket, offs, big_rows, big_count, ucount, row_max);
    FE_LAUNCH("umap_union_big_rows_kernel");
    exclusive_scan(ucount, out64, n, scan_tmp, s);
    umap_max_kernel<<<1, 1024, 0, s>>>(row_max, n, d_max);
    FE_LAUNCH("umap_max_kernel");
  }
};

void umap_build_graph(const int* d_idx, const float* d_dist, int n, int k, int offset, UmapGraph& g, cudaStream_t s) {
  UmapGraphWork w;
  w.alloc(n, k);
  w.enqueue(d_idx, d_dist, n, offset, s);
  long long nnz = 0;
  float mw = 0.0f;
  FE_CUDA(cudaMemcpyAsync(&nnz, w.out64 + n, sizeof(long long), cudaMemcpyDeviceToHost, s));
  FE_CUDA(cudaMemcpyAsync(&mw, w.d_max, sizeof(float), cudaMemcpyDeviceToHost, s));
  FE_CUDA(cudaStreamSynchronize(s));
  if (nnz <= 0 || !(mw > 0.0f)) throw Error("The CSR graph has no usable UMAP edges.");
  if (nnz > INT_MAX) throw Error("UMAP graph exceeds 2^31 - 1 entries.");
  g.n = n;
  g.nnz = nnz;
  g.max_weight = mw;
  g.arena.release();
  g.arena.reserve(&g.offsets, n + 1);
  g.arena.reserve(&g.heads, nnz);
  g.arena.reserve(&g.neighbors, nnz);
  g.arena.reserve(&g.weights, nnz);
  g.arena.reserve(&g.eps, nnz);
  g.arena.commit("UMAP graph");
  umap_fill_csr_kernel<<<ceil_div((long long)(n + 1) * 32, 256), 256, 0, s>>>(
      w.bucket, w.offs, w.out64, n, w.d_max, g.offsets, g.heads, g.neighbors, g.weights, g.eps);
  FE_LAUNCH("umap_fill_csr_kernel");
  FE_CUDA(cudaStreamSynchronize(s));
}

// Batch form of the CSR fill. The instance's first edge is computed on the device from the
// previous instance's (edge_begin[b + 1] = edge_begin[b] + entries of b), with its largest
// weight kept for the host's checks, so consecutive instances need no host round trip.
__global__ void umap_batch_edge_begin_kernel(const long long* __restrict__ entries, const float* __restrict__ max_w,
                                             long long* __restrict__ edge_begin, float* __restrict__ inst_max) {
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    edge_begin[1] = edge_begin[0] + *entries;
    *inst_max = *max_w;
  }
}

// One warp per row: the row's union entries written as COO edges shifted by the instance's first
// vertex v0, with their sampling periods (largest weight / weight, as umap_fill_csr_kernel).
__global__ void umap_fill_batch_kernel(const unsigned long long* __restrict__ bucket,
                                       const long long* __restrict__ offs, const long long* __restrict__ out64, int n,
                                       const float* __restrict__ max_w, const long long* __restrict__ edge_begin,
                                       int v0, int* __restrict__ heads, int* __restrict__ tails,
                                       float* __restrict__ period) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (warp >= n) return;
  const float mw = *max_w;
  const long long src = offs[warp], dst = *edge_begin + out64[warp];
  const int cnt = (int)(out64[warp + 1] - out64[warp]);
  for (int t = lane; t < cnt; t += 32) {
    const unsigned long long e = bucket[src + t];
    const float w = __uint_as_float((unsigned)e);
    heads[dst + t] = warp + v0;
    tails[dst + t] = (int)(e >> 32) + v0;
    period[dst + t] = mw > 0.0f ? mw / fmaxf(w, 1.0e-6f) : INFINITY;
  }
}

// ---------------------------------------------------------------- SGD epoch
struct UmapParams {
  int n, n_epochs, negative_sample_rate;
  unsigned seed;
  float learning_rate, a, b, repulsion_strength;
};

// Positive-base power by IEEE-754 exponent interpolation (Schraudolph 1999), the approximation
// the reference uses in its UMAP force terms (src/embedding_cuda_kernels.cpp:364-383).
__device__ __forceinline__ float schraudolph_pow(float x, float b) {
  if (x <= 0.0f) return 0.0f;
  const float bias = 1064866805.0f;
  const int whole = (int)b;
  const float frac = b - (float)whole;
  const float fp = __uint_as_float((unsigned)(frac * ((float)__float_as_uint(x) - bias) + bias));
  float ip = 1.0f, base = x;
  for (int e = whole; e > 0; e >>= 1) {
    if (e & 1) ip *= base;
    base *= base;
  }
  return ip * fp;
}

__device__ __forceinline__ float clip4(float x) { return fminf(4.0f, fmaxf(-4.0f, x)); }

__device__ __forceinline__ int umap_positive_samples(float period, unsigned epoch) {
  if (period <= 0.0f || !isfinite(period) || epoch == 0u) return 0;
  const int s = (int)floorf((float)epoch / period) - (int)floorf((float)(epoch - 1u) / period);
  return s > 0 ? s : 0;
}

__device__ __forceinline__ int umap_negative_samples(float period, int rate, unsigned epoch) {
  if (rate <= 0 || period <= 0.0f || !isfinite(period) || epoch == 0u) return 0;
  const float now = (float)epoch, prev = (float)(epoch - 1u);
  const int cur = (int)floorf(now / period), pre = (int)floorf(prev / period);
  if (cur <= pre) return 0;
  const float np = period / (float)rate;
  if (np <= 0.0f || !isfinite(np)) return 0;
  const int ct = (int)floorf((now - np) / np);
  int pt = 0;
  if (cur > 1) pt = (int)floorf((ceilf((float)(cur - 1) * period) - np) / np);
  const int s = ct - pt;
  return s > 0 ? s : 0;
}

// Grid-stride over COO edges (sorted by head). The epoch number is read from device memory so
// a captured graph of several epochs replays without re-capture.
__global__ void __launch_bounds__(256)
umap_epoch_kernel(float2* __restrict__ y, const int* __restrict__ heads, const int* __restrict__ tails,
                  const float* __restrict__ eps, long long n_edges, UmapParams p, const unsigned* __restrict__ epoch_ptr,
                  const long long* __restrict__ edge_begin, const int* __restrict__ vert_begin, int ninst) {
  // A batch (ninst > 1) lists its instances' edges one after another (edge_begin, ninst + 1
  // entries) with vertices offset by each instance's first vertex (vert_begin); negatives are
  // drawn inside the edge's own instance and keyed by the instance-local edge id, so an
  // instance draws the same negatives alone and in a batch.
  const unsigned epoch = *epoch_ptr;
  const float alpha = p.learning_rate * (1.0f - (float)epoch / fmaxf(1.0f, (float)p.n_epochs));
  const float fe = 1.1920928955078125e-7f;
  int inst = 0;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n_edges; e += (long long)gridDim.x * blockDim.x) {
    const float period = __ldg(eps + e);
    const int ps = umap_positive_samples(period, epoch);
    if (ps <= 0) continue;
    long long e_local = e;
    int v0 = 0, nv = p.n;
    if (ninst > 1) {
      if (e < edge_begin[inst] || e >= edge_begin[inst + 1]) {
        int lo = 0, hi = ninst - 1;
        while (lo < hi) {
          const int mid = (lo + hi + 1) >> 1;
          if (edge_begin[mid] <= e) lo = mid;
          else hi = mid - 1;
        }
        inst = lo;
      }
      e_local = e - edge_begin[inst];
      v0 = vert_begin[inst];
      nv = vert_begin[inst + 1] - v0;
    }
    const int h = __ldg(heads + e), t = __ldg(tails + e);
    if (h < v0 || h >= v0 + nv || t < v0 || t >= v0 + nv || h == t) continue;
    // The head's own moves go to a register copy and reach memory in one atomic at the end of
    // the edge; later samples of the edge see them, as every sample of the serial reference
    // sees the previous ones. Moves of other threads land through their atomics (Hogwild).
    float2 yh = y[h];
    float mx = 0.0f, my = 0.0f;
    for (int s = 0; s < ps; ++s) {
      const float2 yt = y[t];
      const float dx = yh.x - yt.x, dy = yh.y - yt.y;
      const float d2 = fmaxf(fe, dx * dx + dy * dy);
      const float d2b = schraudolph_pow(d2, p.b);
      const float c = -2.0f * p.a * p.b * (d2b / d2) / (p.a * d2b + 1.0f);
      const float gx = clip4(c * dx) * alpha, gy = clip4(c * dy) * alpha;
      yh.x += gx;
      yh.y += gy;
      mx += gx;
      my += gy;
      atomicAdd(y + t, make_float2(-gx, -gy));
    }
    const int ns = umap_negative_samples(period, p.negative_sample_rate, epoch);
    // negatives four at a time (one Philox block): the four positions are loaded together, then
    // the samples are applied in order
    for (int s0 = 0; s0 < ns; s0 += 4) {
      const uint4 r = philox4x32_10(make_uint4((unsigned)e_local, (unsigned)(e_local >> 32), epoch, (unsigned)(s0 >> 2)),
                                    make_uint2(p.seed, 0x5eed0f0cu));
      const unsigned draws[4] = {r.x, r.y, r.z, r.w};
      int neg[4];
      float2 yn[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        neg[q] = v0 + (int)bounded(draws[q], (unsigned)nv);
        yn[q] = s0 + q < ns ? y[neg[q]] : make_float2(0.0f, 0.0f);
      }
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        if (s0 + q >= ns || neg[q] == h || neg[q] == t) continue;
        const float dx = yh.x - yn[q].x, dy = yh.y - yn[q].y;
        const float d2 = fmaxf(fe, dx * dx + dy * dy);
        const float d2b = schraudolph_pow(d2, p.b);
        const float rc = p.repulsion_strength * 2.0f * p.b / ((0.001f + d2) * (p.a * d2b + 1.0f));
        const float gx = clip4(rc * dx) * alpha, gy = clip4(rc * dy) * alpha;
        yh.x += gx;
        yh.y += gy;
        mx += gx;
        my += gy;
      }
    }
    atomicAdd(y + h, make_float2(mx, my));
  }
}

// NaN -> 0 and clamp to +-16 (umap_sanitize_layout_kernel, :3244-3258); thread 0 advances the
// device epoch counter.
__global__ void umap_sanitize_kernel(float2* __restrict__ y, int n, unsigned* __restrict__ epoch_ptr) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    float2 v = y[i];
    if (!isfinite(v.x)) v.x = 0.0f;
    if (!isfinite(v.y)) v.y = 0.0f;
    y[i] = make_float2(fminf(16.0f, fmaxf(-16.0f, v.x)), fminf(16.0f, fmaxf(-16.0f, v.y)));
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) *epoch_ptr += 1u;
}

// find_ab_params CPU policy (src/fast_knn_umap.cpp:437-497): hard-coded values for the package's
// spreads/min_dists, otherwise the grid search + gradient refinement of that function.
void umap_ab_params(double spread, double min_dist, double* a, double* b) {
  if (std::fabs(spread - 1.0) < 1e-12 && std::fabs(min_dist - 0.01) < 1e-12) {
    *a = 1.895605865596314;
    *b = 0.8006377738365004;
    return;
  }
  if (std::fabs(spread - 1.0) < 1e-12 && std::fabs(min_dist - 0.1) < 1e-12) {
    *a = 1.5769434601962196;
    *b = 0.8950608781227859;
    return;
  }
  if (std::fabs(spread - 1.0) < 1e-12 && std::fabs(min_dist - 0.5) < 1e-12) {
    *a = 0.5830300199018228;
    *b = 1.3341669931033755;
    return;
  }
  double xs[300], ys[300];
  for (int i = 0; i < 300; ++i) {
    xs[i] = (spread * 3.0) * (double)i / 299.0;
    ys[i] = xs[i] < min_dist ? 1.0 : std::exp(-(xs[i] - min_dist) / spread);
  }
  double ba = 1.5769434601962196, bb = 0.8950608781227859, best = INFINITY;
  for (double la = -4.0; la <= 4.0001; la += 0.2)
    for (double bv = 0.25; bv <= 2.0001; bv += 0.05) {
      const double av = std::exp(la);
      double loss = 0.0;
      for (int i = 0; i < 300; ++i) {
        const double e = 1.0 / (1.0 + av * std::pow(xs[i], 2.0 * bv)) - ys[i];
        loss += e * e;
      }
      if (loss < best) {
        best = loss;
        ba = av;
        bb = bv;
      }
    }
  for (int it = 0; it < 80; ++it) {
    double ga = 0.0, gb = 0.0;
    for (int i = 0; i < 300; ++i) {
      const double x = std::max(xs[i], 1e-6);
      const double x2b = std::pow(x, 2.0 * bb);
      const double den = 1.0 + ba * x2b;
      const double e = 1.0 / den - ys[i];
      ga += e * (-x2b / (den * den));
      gb += e * (-(ba * x2b * 2.0 * std::log(x)) / (den * den));
    }
    ba = std::max(1e-4, ba - 0.01 * ga);
    bb = std::max(0.1, bb - 0.01 * gb);
  }
  *a = ba;
  *b = bb;
}

// Optimizer state of one UMAP instance.
// Sort keys of the period-ordered edge list: the bits of epochs_per_sample (non-negative floats,
// so their bit patterns order as the values; inf and NaN, never sampled, sort last).
__global__ void umap_period_keys_kernel(const float* __restrict__ eps, int m, unsigned* __restrict__ keys,
                                        int* __restrict__ idx) {
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < m; e += gridDim.x * blockDim.x) {
    const float v = eps[e];
    keys[e] = v > 0.0f || isnan(v) ? __float_as_uint(v) : 0u;
    idx[e] = e;
  }
}

__global__ void umap_gather_edges_kernel(const int* __restrict__ perm, const int* __restrict__ heads,
                                         const int* __restrict__ tails, const float* __restrict__ eps, int m,
                                         int* __restrict__ oh, int* __restrict__ ot, float* __restrict__ oe) {
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < m; e += gridDim.x * blockDim.x) {
    const int q = perm[e];
    oh[e] = heads[q];
    ot[e] = tails[q];
    oe[e] = eps[q];
  }
}

struct UmapJob {
  Stream stream;
  Arena arena;
  float2* y = nullptr;
  unsigned* epoch = nullptr;
  std::map<int, std::pair<cudaGraph_t, cudaGraphExec_t>> graphs;
  ~UmapJob() {
    for (auto& kv : graphs) {
      if (kv.second.second) cudaGraphExecDestroy(kv.second.second);
      if (kv.second.first) cudaGraphDestroy(kv.second.first);
    }
  }
  void alloc(int n) {
    arena.reserve(&y, n);
    arena.reserve(&epoch, 1);
    arena.commit("UMAP layout");
  }
  // batch view (set for batches: ninst > 1)
  const long long* edge_begin = nullptr;
  const int* vert_begin = nullptr;
  int ninst = 1;
  // Edges ordered by sampling period (stable, within each instance of a batch): the edges of a
  // warp then fire in the same epochs and draw similar numbers of negative samples, where the
  // head-ordered list left most lanes of a warp idle in any one epoch. Only the order of the
  // asynchronous (Hogwild) updates changes.
  Arena ordered;
  void order_by_period(const int*& heads, const int*& tails, const float*& eps, long long n_edges) {
    if (n_edges < 2 || n_edges > INT_MAX) return;
    cudaStream_t s = stream.s;
    const int m = (int)n_edges;
    unsigned *keys = nullptr, *keys_out = nullptr;
    int *idx = nullptr, *perm = nullptr, *oh = nullptr, *ot = nullptr;
    float* oe = nullptr;
    std::size_t temp_bytes = 0;
    if (ninst > 1)
      FE_CUDA(cub::DeviceSegmentedRadixSort::SortPairs(nullptr, temp_bytes, keys, keys_out, idx, perm, m, ninst,
                                                       edge_begin, edge_begin + 1, 0, 32, s));
    else
      FE_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, temp_bytes, keys, keys_out, idx, perm, m, 0, 32, s));
    unsigned char* temp = nullptr;
    Arena work;
    work.reserve(&keys, m);
    work.reserve(&keys_out, m);
    work.reserve(&idx, m);
    work.reserve(&perm, m);
    work.reserve(&temp, std::max<std::size_t>(temp_bytes, 16));
    work.commit("UMAP edge order workspace");
    ordered.release();
    ordered.reserve(&oh, m);
    ordered.reserve(&ot, m);
    ordered.reserve(&oe, m);
    ordered.commit("UMAP edges in period order");
    const int blocks = std::max(1, std::min(ceil_div(m, 256), sm_count() * 8));
    umap_period_keys_kernel<<<blocks, 256, 0, s>>>(eps, m, keys, idx);
    FE_LAUNCH("umap_period_keys_kernel");
    if (ninst > 1)
      FE_CUDA(cub::DeviceSegmentedRadixSort::SortPairs(temp, temp_bytes, keys, keys_out, idx, perm, m, ninst,
                                                       edge_begin, edge_begin + 1, 0, 32, s));
    else
      FE_CUDA(cub::DeviceRadixSort::SortPairs(temp, temp_bytes, keys, keys_out, idx, perm, m, 0, 32, s));
    umap_gather_edges_kernel<<<blocks, 256, 0, s>>>(perm, heads, tails, eps, m, oh, ot, oe);
    FE_LAUNCH("umap_gather_edges_kernel");
    FE_CUDA(cudaStreamSynchronize(s));  // the workspace is released on return
    heads = oh;
    tails = ot;
    eps = oe;
  }
  void run(const int* heads, const int* tails, const float* eps, long long n_edges, const UmapParams& p) {
    cudaStream_t s = stream.s;
    order_by_period(heads, tails, eps, n_edges);
    // captured graphs hold the edge arrays of the run that captured them
    for (auto& kv : graphs) {
      if (kv.second.second) cudaGraphExecDestroy(kv.second.second);
      if (kv.second.first) cudaGraphDestroy(kv.second.first);
    }
    graphs.clear();
    FE_CUDA(cudaMemsetAsync(epoch, 0, sizeof(unsigned), s));
    const int eblocks = std::max(1, std::min(ceil_div(n_edges, 256), sm_count() * 8));
    const int pblocks = std::max(1, std::min(ceil_div(p.n, 256), sm_count() * 4));
    auto one_epoch = [&]() {
      umap_epoch_kernel<<<eblocks, 256, 0, s>>>(y, heads, tails, eps, n_edges, p, epoch, edge_begin, vert_begin,
                                                ninst);
      FE_LAUNCH("umap_epoch_kernel");
      umap_sanitize_kernel<<<pblocks, 256, 0, s>>>(y, p.n, epoch);
      FE_LAUNCH("umap_sanitize_kernel");
    };
    constexpr int kChunk = 25;
    int left = p.n_epochs;
    while (left > 0) {
      const int c = std::min(kChunk, left);
      auto it = graphs.find(c);
      if (it == graphs.end()) {
        cudaGraph_t g = nullptr;
        cudaGraphExec_t ge = nullptr;
        FE_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
        try {
          for (int r = 0; r < c; ++r) one_epoch();
        } catch (...) {
          cudaStreamEndCapture(s, &g);
          if (g) cudaGraphDestroy(g);
          throw;
        }
        FE_CUDA(cudaStreamEndCapture(s, &g));
        FE_CUDA(cudaGraphInstantiate(&ge, g, 0));
        it = graphs.emplace(c, std::make_pair(g, ge)).first;
      }
      FE_CUDA(cudaGraphLaunch(it->second.second, s));
      left -= c;
    }
  }
};

// ---------------------------------------------------------------- diffusion start
// The reference's GPU spectral start (fastembedr_cuda_spectral_init_from_knn,
// src/embedding_cuda_kernels.cpp:4801-4960; kernels :1178-1335), stated for the CPU by the
// reference as initialize_layout_csr_cuda_diffusion (src/fast_knn_umap.cpp:2597-2652): a hashed
// start in [-1, 1]^2 (deterministic_unit, :522-530), whitened (normalize_cuda_like_init,
// :2541-2595: centred, x scaled to unit norm, y made orthogonal to x and scaled to unit norm),
// then rounds of weighted neighbour averaging over the fuzzy graph, whitened after each. Each
// row's average is summed in CSR order in float with separately rounded products, as the CPU
// statement does; the whitening moments are FP64 sums of exact products, reduced in a fixed
// block order, and the whitening arithmetic is FP64 without contraction.
constexpr int kInitThreads = 256;
constexpr int kInitMomentBlocks = 1024;

__device__ __forceinline__ unsigned init_hash(unsigned x) {
  x ^= x >> 16;
  x *= 0x7feb352du;
  x ^= x >> 15;
  x *= 0x846ca68bu;
  x ^= x >> 16;
  return x;
}

__device__ __forceinline__ float init_unit(unsigned seed, int row, int col) {
  unsigned x = seed;
  x ^= (unsigned)(row + 1) * 0x9e3779b9u;
  x ^= (unsigned)(col + 1) * 0x85ebca6bu;
  return __fsub_rn(__fdiv_rn((float)(init_hash(x) & 0x00ffffffu), 8388607.5f), 1.0f);
}

__global__ void diffusion_start_kernel(float2* __restrict__ y, int n, unsigned seed) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    y[i] = make_float2(init_unit(seed, i, 0), init_unit(seed, i, 1));
}

__global__ void diffusion_round_kernel(const int* __restrict__ offsets, const int* __restrict__ neighbors,
                                       const float* __restrict__ weights, int n, const float2* __restrict__ cur,
                                       float2* __restrict__ next) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    float sx = 0.0f, sy = 0.0f, sw = 0.0f;
    for (int p = offsets[i]; p < offsets[i + 1]; ++p) {
      const int nb = neighbors[p];
      const float w = weights[p];
      if (nb < 0 || nb >= n || nb == i || !(w > 0.0f) || !isfinite(w)) continue;
      const float2 c = cur[nb];
      sx = __fadd_rn(sx, __fmul_rn(w, c.x));
      sy = __fadd_rn(sy, __fmul_rn(w, c.y));
      sw = __fadd_rn(sw, w);
    }
    next[i] = sw <= 0.0f ? cur[i] : make_float2(__fdiv_rn(sx, sw), __fdiv_rn(sy, sw));
  }
}

// Block partial moments (sum x, sum y, sum x^2, sum xy, sum y^2) of the layout.
__global__ void __launch_bounds__(kInitThreads)
whiten_moments_kernel(const float2* __restrict__ y, int n, double* __restrict__ partial) {
  __shared__ double sm[5][kInitThreads];
  double a[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const double x = y[i].x, v = y[i].y;
    a[0] += x;
    a[1] += v;
    a[2] += x * x;  // products of floats are exact in double
    a[3] += x * v;
    a[4] += v * v;
  }
#pragma unroll
  for (int c = 0; c < 5; ++c) sm[c][threadIdx.x] = a[c];
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w)
#pragma unroll
      for (int c = 0; c < 5; ++c) sm[c][threadIdx.x] += sm[c][threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x < 5) partial[blockIdx.x * 5 + threadIdx.x] = sm[threadIdx.x][0];
}

// stats = (mean_x, mean_y, 1 / |x|, projection of y on x, 1 / |y residual|), one thread.
__global__ void whiten_finish_kernel(const double* __restrict__ partial, int blocks, int n, double* __restrict__ st) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double m[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
  for (int b = 0; b < blocks; ++b)
    for (int c = 0; c < 5; ++c) m[c] += partial[b * 5 + c];
  const double dn = (double)n;
  const double xss = fmax(__dsub_rn(m[2], __ddiv_rn(__dmul_rn(m[0], m[0]), dn)), 1.0e-24);
  const double yss = fmax(__dsub_rn(m[4], __ddiv_rn(__dmul_rn(m[1], m[1]), dn)), 1.0e-24);
  const double xy = __dsub_rn(m[3], __ddiv_rn(__dmul_rn(m[0], m[1]), dn));
  const double nx = __dsqrt_rn(xss);
  const double proj = __ddiv_rn(xy, nx);
  st[0] = __ddiv_rn(m[0], dn);
  st[1] = __ddiv_rn(m[1], dn);
  st[2] = __ddiv_rn(1.0, nx);
  st[3] = proj;
  st[4] = __ddiv_rn(1.0, __dsqrt_rn(fmax(__dsub_rn(yss, __dmul_rn(proj, proj)), 1.0e-24)));
}

__global__ void whiten_apply_kernel(float2* __restrict__ y, int n, const double* __restrict__ st) {
  const double mx = st[0], my = st[1], inx = st[2], proj = st[3], iny = st[4];
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float2 v = y[i];
    const double x = __dmul_rn(__dsub_rn((double)v.x, mx), inx);
    const double r = __dmul_rn(__dsub_rn(__dsub_rn((double)v.y, my), __dmul_rn(proj, x)), iny);
    y[i] = make_float2((float)x, (float)r);
  }
}

__global__ void umap_double_to_float_kernel(const double* __restrict__ in, float* __restrict__ out, long long m) {
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < m; t += (long long)gridDim.x * blockDim.x)
    out[t] = (float)in[t];
}

// Unit weights and sampling periods on the fuzzy graph's structure (the binary graph mode of
// the reference's fused path, binary_graph_weights_kernel, src/embedding_cuda_kernels.cpp:1115).
__global__ void umap_binary_weights_kernel(float* __restrict__ weights, float* __restrict__ eps, long long nnz) {
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < nnz; t += (long long)gridDim.x * blockDim.x) {
    weights[t] = 1.0f;
    eps[t] = 1.0f;
  }
}

void whiten(float2* y, int n, double* partial, double* stats, cudaStream_t s) {
  const int blocks = std::max(1, std::min(ceil_div(n, kInitThreads), kInitMomentBlocks));
  whiten_moments_kernel<<<blocks, kInitThreads, 0, s>>>(y, n, partial);
  FE_LAUNCH("whiten_moments_kernel");
  whiten_finish_kernel<<<1, 32, 0, s>>>(partial, blocks, n, stats);
  FE_LAUNCH("whiten_finish_kernel");
  whiten_apply_kernel<<<std::max(1, std::min(ceil_div(n, kInitThreads), sm_count() * 8)), kInitThreads, 0, s>>>(
      y, n, stats);
  FE_LAUNCH("whiten_apply_kernel");
}

// Diffusion start over g into y (n float2); 4 launches per round.
void umap_diffusion_start(const UmapGraph& g, int n_iter, unsigned seed, float2* y, cudaStream_t s) {
  const int n = g.n;
  float2* tmp = nullptr;
  double* partial = nullptr;
  double* stats = nullptr;
  Arena w;
  w.reserve(&tmp, n);
  w.reserve(&partial, 5 * kInitMomentBlocks);
  w.reserve(&stats, 5);
  w.commit("UMAP diffusion start");
  const int blocks = std::max(1, std::min(ceil_div(n, kInitThreads), sm_count() * 8));
  diffusion_start_kernel<<<blocks, kInitThreads, 0, s>>>(y, n, seed);
  FE_LAUNCH("diffusion_start_kernel");
  whiten(y, n, partial, stats, s);
  float2* cur = y;
  float2* nxt = tmp;
  for (int it = 0; it < n_iter; ++it) {
    diffusion_round_kernel<<<blocks, kInitThreads, 0, s>>>(g.offsets, g.neighbors, g.weights, n, cur, nxt);
    FE_LAUNCH("diffusion_round_kernel");
    whiten(nxt, n, partial, stats, s);
    std::swap(cur, nxt);
  }
  if (cur != y) FE_CUDA(cudaMemcpyAsync(y, cur, sizeof(float2) * n, cudaMemcpyDeviceToDevice, s));
  FE_CUDA(cudaStreamSynchronize(s));
}

// KNN on the device (float distances) -> fuzzy graph (optionally unit-weighted) -> diffusion
// start -> n_epochs of SGD; result row-major n x 2 floats to the host.
void umap_spectral_job(const int* d_idx, const float* d_dist, int n, int k, int n_epochs, int nsr, float lr, float a,
                       float b, float rep, int spectral_n_iter, unsigned seed, int offset, bool binary, float* out) {
  UmapJob job;
  job.alloc(n);
  cudaStream_t s = job.stream.s;
  order_after_legacy_stream(s);  // d_idx / d_dist may be the caller's device buffers
  validate_knn(d_idx, d_dist, n, k, offset, s);
  UmapGraph g;
  umap_build_graph(d_idx, d_dist, n, k, offset, g, s);
  if (binary) {
    umap_binary_weights_kernel<<<std::max(1, std::min(ceil_div(g.nnz, 256), sm_count() * 8)), 256, 0, s>>>(
        g.weights, g.eps, g.nnz);
    FE_LAUNCH("umap_binary_weights_kernel");
  }
  umap_diffusion_start(g, spectral_n_iter, seed, job.y, s);
  const UmapParams p{n, n_epochs, nsr, seed, lr, a, b, rep};
  job.run(g.heads, g.neighbors, g.eps, g.nnz, p);
  FE_CUDA(cudaMemcpyAsync(out, job.y, sizeof(float) * 2 * (std::size_t)n, cudaMemcpyDeviceToHost, s));
  FE_CUDA(cudaStreamSynchronize(s));
}

__global__ void umap_start_to_layout_kernel(const double* __restrict__ emb, int n, float2* __restrict__ y) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    y[i] = make_float2((float)emb[i], (float)emb[(long long)n + i]);
}

// KNN on the device -> fuzzy graph -> the reference CPU spectral start (block subspace
// iteration) -> optionally n_epochs of SGD from it. emb_out (host, column-major n x 2 doubles)
// receives the start, y_out (host, row-major n x 2 floats) the optimised layout; either may be
// null (n_epochs must be 0 when y_out is).
void umap_knn_spectral_job(const int* d_idx, const float* d_dist, int n, int k, int offset, int n_epochs, int nsr,
                           float lr, float min_dist, float rep, int spectral_n_iter, double init_scale,
                           unsigned seed, double* emb_out, float* y_out,
                           std::future<SpectralDraws>* early = nullptr) {
  // the start's host draws (started by the caller before its input copies, or here) run while
  // the GPU validates the KNN and builds the graph
  std::future<SpectralDraws> own;
  if (!early) {
    own = std::async(std::launch::async, spectral_draws, n, (int)seed);
    early = &own;
  }
  UmapJob job;
  job.alloc(n);
  cudaStream_t s = job.stream.s;
  order_after_legacy_stream(s);
  validate_knn(d_idx, d_dist, n, k, offset, s);
  UmapGraph g;
  umap_build_graph(d_idx, d_dist, n, k, offset, g, s);
  SpectralDraws pre = early->get();
  double* emb = nullptr;
  Arena a;
  a.reserve(&emb, 2 * (std::size_t)n);
  a.commit("UMAP spectral start output");
  umap_spectral_start(g.offsets, g.neighbors, g.weights, n, g.nnz, spectral_n_iter, init_scale, (int)seed, emb, s,
                      &pre);
  if (emb_out) FE_CUDA(cudaMemcpyAsync(emb_out, emb, sizeof(double) * 2 * (std::size_t)n, cudaMemcpyDeviceToHost, s));
  if (y_out) {
    umap_start_to_layout_kernel<<<std::max(1, std::min(ceil_div(n, 256), sm_count() * 8)), 256, 0, s>>>(emb, n,
                                                                                                      job.y);
    FE_LAUNCH("umap_start_to_layout_kernel");
    if (n_epochs > 0) {
      double av = 0.0, bv = 0.0;
      umap_ab_params(1.0, min_dist, &av, &bv);
      const UmapParams p{n, n_epochs, nsr, seed, lr, (float)av, (float)bv, rep};
      job.run(g.heads, g.neighbors, g.eps, g.nnz, p);
    }
    FE_CUDA(cudaMemcpyAsync(y_out, job.y, sizeof(float) * 2 * (std::size_t)n, cudaMemcpyDeviceToHost, s));
  }
  FE_CUDA(cudaStreamSynchronize(s));
}

void check_spectral_job(int n, int k, int n_epochs, int nsr, float lr, int spectral_n_iter, int optimizer_mode) {
  if (n < 2 || k < 1 || k > 256 || n_epochs < 1 || nsr < 0 || !(lr > 0.0f) || spectral_n_iter < 1)
    throw Error("invalid fused CUDA UMAP dimensions or parameters");
  if (optimizer_mode != 0)
    throw Error("optimizer_mode 1 (batched delta) is not provided; the package policy uses mode 0");
}

void check_umap_params(int n, long long n_edges, int n_epochs, int nsr, float lr, float rep) {
  if (n < 2 || n_edges < 1 || n_epochs < 1 || nsr < 0 || !(lr > 0.0f) || !(rep > 0.0f))
    throw Error("invalid CUDA COO UMAP optimization parameters");
}

}  // namespace fe

namespace {
template <typename DistT>
int umap_spectral_host(const int* indices, const DistT* distances, int n, int k, int n_epochs, int nsr, float lr,
                       float a, float b, float rep, int spectral_n_iter, unsigned seed, int index_offset,
                       int optimizer_mode, float* out) {
  return fe::guarded([&] {
    if (!indices || !distances || !out) throw fe::Error("null host pointer");
    fe::check_spectral_job(n, k, n_epochs, nsr, lr, spectral_n_iter, optimizer_mode);
    fe::Stream st;
    cudaStream_t s = st.s;
    const std::size_t items = (std::size_t)n * k;
    int* d_idx = nullptr;
    DistT* d_raw = nullptr;
    float* d_dist = nullptr;
    fe::Arena in;
    in.reserve(&d_idx, items);
    if (!std::is_same<DistT, float>::value) in.reserve(&d_raw, items);
    in.reserve(&d_dist, items);
    in.commit("fused CUDA UMAP input");
    fe::upload(d_idx, indices, sizeof(int) * items, s);
    if constexpr (std::is_same<DistT, float>::value) {
      fe::upload(d_dist, distances, sizeof(float) * items, s);
    } else {
      fe::upload(d_raw, distances, sizeof(double) * items, s);
      fe::umap_double_to_float_kernel<<<std::max(1, std::min(fe::ceil_div((long long)items, 256),
                                                              fe::sm_count() * 8)),
                                        256, 0, s>>>(d_raw, d_dist, (long long)items);
      FE_LAUNCH("umap_double_to_float_kernel");
    }
    FE_CUDA(cudaStreamSynchronize(s));
    fe::umap_spectral_job(d_idx, d_dist, n, k, n_epochs, nsr, lr, a, b, rep, spectral_n_iter, seed, index_offset,
                          false, out);
  });
}
}  // namespace

extern "C" {

int fastembedr_cuda_umap_optimize_coo(const int* heads, const int* tails, const float* weights,
                                      const float* epochs_per_sample, const float* init, int n, int n_edges_capacity,
                                      int n_epochs, int negative_sample_rate, float learning_rate, float a, float b,
                                      float repulsion_strength, unsigned int seed, int optimizer_mode, float* out) {
  return fe::guarded([&] {
    if (!heads || !tails || !weights || !epochs_per_sample || !init || !out) throw fe::Error("null host pointer");
    fe::check_umap_params(n, n_edges_capacity, n_epochs, negative_sample_rate, learning_rate, repulsion_strength);
    if (optimizer_mode != 0)
      throw fe::Error("optimizer_mode 1 (batched delta) is not provided; the package policy uses mode 0");
    fe::UmapJob job;
    job.alloc(n);
    cudaStream_t s = job.stream.s;
    int *d_h = nullptr, *d_t = nullptr;
    float* d_e = nullptr;
    fe::Arena in;
    in.reserve(&d_h, n_edges_capacity);
    in.reserve(&d_t, n_edges_capacity);
    in.reserve(&d_e, n_edges_capacity);
    in.commit("CUDA COO UMAP edges");
    fe::upload(d_h, heads, sizeof(int) * n_edges_capacity, s);
    fe::upload(d_t, tails, sizeof(int) * n_edges_capacity, s);
    fe::upload(d_e, epochs_per_sample, sizeof(float) * n_edges_capacity, s);
    FE_CUDA(cudaMemcpyAsync(job.y, init, sizeof(float) * 2 * n, cudaMemcpyHostToDevice, s));
    const fe::UmapParams p{n, n_epochs, negative_sample_rate, seed, learning_rate, a, b, repulsion_strength};
    job.run(d_h, d_t, d_e, n_edges_capacity, p);
    FE_CUDA(cudaMemcpyAsync(out, job.y, sizeof(float) * 2 * n, cudaMemcpyDeviceToHost, s));
    FE_CUDA(cudaStreamSynchronize(s));
  });
}

int fastembedr_cuda_umap_graph_from_knn(const int* indices, const float* distances, int n, int k, int index_offset,
                                        int* offsets, int* neighbors, float* weights, float* epochs_per_sample,
                                        long long capacity, long long* nnz, float* max_weight) {
  return fe::guarded([&] {
    if (!indices || !distances || !offsets || !nnz) throw fe::Error("null UMAP graph pointer");
    if (n < 2 || k < 1) throw fe::Error("invalid UMAP graph dimensions");
    fe::Stream st;
    const std::size_t items = (std::size_t)n * k;
    int* d_idx = nullptr;
    float* d_dist = nullptr;
    fe::Arena a;
    a.reserve(&d_idx, items);
    a.reserve(&d_dist, items);
    a.commit("UMAP graph input");
    fe::upload(d_idx, indices, sizeof(int) * items, st.s);
    fe::upload(d_dist, distances, sizeof(float) * items, st.s);
    fe::validate_knn(d_idx, d_dist, n, k, index_offset, st.s);
    fe::UmapGraph g;
    fe::umap_build_graph(d_idx, d_dist, n, k, index_offset, g, st.s);
    *nnz = g.nnz;
    if (max_weight) *max_weight = g.max_weight;
    FE_CUDA(cudaMemcpyAsync(offsets, g.offsets, sizeof(int) * (n + 1), cudaMemcpyDeviceToHost, st.s));
    if (neighbors && weights && epochs_per_sample && g.nnz <= capacity) {
      FE_CUDA(cudaMemcpyAsync(neighbors, g.neighbors, sizeof(int) * g.nnz, cudaMemcpyDeviceToHost, st.s));
      FE_CUDA(cudaMemcpyAsync(weights, g.weights, sizeof(float) * g.nnz, cudaMemcpyDeviceToHost, st.s));
      FE_CUDA(cudaMemcpyAsync(epochs_per_sample, g.eps, sizeof(float) * g.nnz, cudaMemcpyDeviceToHost, st.s));
    }
    FE_CUDA(cudaStreamSynchronize(st.s));
  });
}

int fastembedr_cuda_umap_from_knn_profile(const int* indices, const float* distances, const float* init, int n,
                                          int k, int index_offset, int n_epochs, int negative_sample_rate,
                                          float learning_rate, float min_dist, float repulsion_strength,
                                          unsigned int seed, float* out, float* graph_ms, float* sgd_ms) {
  return fe::guarded([&] {
    if (!indices || !distances || !init || !out) throw fe::Error("null UMAP input pointer");
    if (n < 2 || k < 1 || n_epochs < 1 || negative_sample_rate < 0 || !(learning_rate > 0.0f) || min_dist < 0.0f ||
        !(repulsion_strength > 0.0f))
      throw fe::Error("invalid CUDA UMAP parameters");
    fe::UmapJob job;
    job.alloc(n);
    cudaStream_t s = job.stream.s;
    const std::size_t items = (std::size_t)n * k;
    int* d_idx = nullptr;
    float* d_dist = nullptr;
    fe::Arena a;
    a.reserve(&d_idx, items);
    a.reserve(&d_dist, items);
    a.commit("UMAP input");
    fe::upload(d_idx, indices, sizeof(int) * items, s);
    fe::upload(d_dist, distances, sizeof(float) * items, s);
    FE_CUDA(cudaMemcpyAsync(job.y, init, sizeof(float) * 2 * n, cudaMemcpyHostToDevice, s));
    cudaEvent_t ev[3] = {nullptr, nullptr, nullptr};
    const bool timed = graph_ms || sgd_ms;
    if (timed)
      for (auto& e : ev) FE_CUDA(cudaEventCreate(&e));
    struct EventGuard {
      cudaEvent_t* e;
      ~EventGuard() {
        for (int i = 0; i < 3; ++i)
          if (e[i]) cudaEventDestroy(e[i]);
      }
    } guard{ev};
    if (timed) FE_CUDA(cudaEventRecord(ev[0], s));
    fe::validate_knn(d_idx, d_dist, n, k, index_offset, s);
    fe::UmapGraph g;
    fe::umap_build_graph(d_idx, d_dist, n, k, index_offset, g, s);
    if (timed) FE_CUDA(cudaEventRecord(ev[1], s));
    double av = 0.0, bv = 0.0;
    fe::umap_ab_params(1.0, min_dist, &av, &bv);
    const fe::UmapParams p{n, n_epochs, negative_sample_rate, seed, learning_rate, (float)av, (float)bv,
                           repulsion_strength};
    job.run(g.heads, g.neighbors, g.eps, g.nnz, p);
    if (timed) FE_CUDA(cudaEventRecord(ev[2], s));
    FE_CUDA(cudaMemcpyAsync(out, job.y, sizeof(float) * 2 * n, cudaMemcpyDeviceToHost, s));
    FE_CUDA(cudaStreamSynchronize(s));
    a.release();
    if (graph_ms) FE_CUDA(cudaEventElapsedTime(graph_ms, ev[0], ev[1]));
    if (sgd_ms) FE_CUDA(cudaEventElapsedTime(sgd_ms, ev[1], ev[2]));
  });
}

}  // extern "C"

namespace fe {

// Row-major nb x k block -> column-major (the layout the graph build reads).
__global__ void umap_rows_to_cols_kernel(const int* __restrict__ idx_rm, const float* __restrict__ dist_rm, int nb,
                                         int k, int* __restrict__ idx_cm, float* __restrict__ dist_cm) {
  const long long total = (long long)nb * k;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
       t += (long long)gridDim.x * blockDim.x) {
    const long long i = t / k, j = t - i * k;
    idx_cm[j * nb + i] = idx_rm[t];
    dist_cm[j * nb + i] = dist_rm[t];
  }
}

// The batched UMAP job: instance b's KNN from idx_u[b] / dist_u[b] (column-major n_b x k, or
// row-major when row_major), its start from init_u[b] (row-major n_b x 2), its layout to
// out_u[b]. One fuzzy graph per instance, appended with vertex offsets, then every epoch one
// launch over all instances' edges.
void umap_batch_job(int n_instances, const int* sizes, const std::vector<const int*>& idx_u,
                    const std::vector<const float*>& dist_u, const std::vector<const float*>& init_u,
                    const std::vector<float*>& out_u, bool row_major, int k, int index_offset, int n_epochs,
                    int negative_sample_rate, float learning_rate, float min_dist, float repulsion_strength,
                    unsigned seed, float* sgd_ms) {
  if (n_instances < 1 || k < 1 || n_epochs < 1 || negative_sample_rate < 0 || !(learning_rate > 0.0f) ||
      min_dist < 0.0f || !(repulsion_strength > 0.0f))
    throw Error("invalid CUDA UMAP batch parameters");
  std::vector<int> vb(n_instances + 1, 0);
  int max_n = 0;
  for (int b = 0; b < n_instances; ++b) {
    if (sizes[b] < 2) throw Error("UMAP batch: every instance needs at least two points");
    if ((long long)vb[b] + sizes[b] > INT_MAX / 2) throw Error("UMAP batch: too many points");
    vb[b + 1] = vb[b] + sizes[b];
    max_n = std::max(max_n, sizes[b]);
  }
  const int n = vb[n_instances];
  UmapJob job;
  job.alloc(n);
  cudaStream_t s = job.stream.s;
  long long n_edges = 0;
  // Every instance's fuzzy graph is built in one reused workspace and written straight into the
  // batch's edge list at a first edge the device computes; the host reads the checks of all
  // instances back once, after the last build. An instance's union graph has at most twice as
  // many entries as it has directed edges.
  const long long cap_edges = std::max(2LL * n * k, 1LL);
  int *heads = nullptr, *tails = nullptr, *d_vb = nullptr;
  float *period = nullptr, *inst_max = nullptr;
  long long* d_eb = nullptr;
  unsigned* flags = nullptr;
  Arena ga;
  ga.reserve(&heads, (std::size_t)cap_edges);
  ga.reserve(&tails, (std::size_t)cap_edges);
  ga.reserve(&period, (std::size_t)cap_edges);
  ga.reserve(&d_eb, n_instances + 1);
  ga.reserve(&d_vb, n_instances + 1);
  ga.reserve(&inst_max, n_instances);
  ga.reserve(&flags, 1);
  ga.commit("UMAP batch graph");
  FE_CUDA(cudaMemsetAsync(d_eb, 0, sizeof(long long), s));
  FE_CUDA(cudaMemsetAsync(flags, 0, sizeof(unsigned), s));
  {
    UmapGraphWork w;
    w.alloc(max_n, k);
    int *d_idx = nullptr, *d_irm = nullptr;
    float *d_dist = nullptr, *d_drm = nullptr;
    Arena in;
    in.reserve(&d_idx, (std::size_t)max_n * k);
    in.reserve(&d_dist, (std::size_t)max_n * k);
    if (row_major) {
      in.reserve(&d_irm, (std::size_t)max_n * k);
      in.reserve(&d_drm, (std::size_t)max_n * k);
    }
    in.commit("UMAP batch input");
    for (int b = 0; b < n_instances; ++b) {
      const int nb = sizes[b];
      const std::size_t items = (std::size_t)nb * k;
      if (row_major) {
        fe::upload(d_irm, idx_u[b], sizeof(int) * items, s);
        fe::upload(d_drm, dist_u[b], sizeof(float) * items, s);
        umap_rows_to_cols_kernel<<<std::max(1, std::min(ceil_div((long long)items, 256), sm_count() * 8)), 256, 0,
                                   s>>>(d_irm, d_drm, nb, k, d_idx, d_dist);
        FE_LAUNCH("umap_rows_to_cols_kernel");
      } else {
        fe::upload(d_idx, idx_u[b], sizeof(int) * items, s);
        fe::upload(d_dist, dist_u[b], sizeof(float) * items, s);
      }
      validate_knn_async(d_idx, d_dist, nb, k, index_offset, flags, s);
      w.enqueue(d_idx, d_dist, nb, index_offset, s);
      umap_batch_edge_begin_kernel<<<1, 32, 0, s>>>(w.out64 + nb, w.d_max, d_eb + b, inst_max + b);
      FE_LAUNCH("umap_batch_edge_begin_kernel");
      umap_fill_batch_kernel<<<ceil_div((long long)nb * 32, 256), 256, 0, s>>>(
          w.bucket, w.offs, w.out64, nb, w.d_max, d_eb + b, vb[b], heads, tails, period);
      FE_LAUNCH("umap_fill_batch_kernel");
    }
    std::vector<long long> eb(n_instances + 1, 0);
    std::vector<float> mx(n_instances, 0.0f);
    unsigned hflags = 0u;
    FE_CUDA(cudaMemcpyAsync(eb.data(), d_eb, sizeof(long long) * eb.size(), cudaMemcpyDeviceToHost, s));
    FE_CUDA(cudaMemcpyAsync(mx.data(), inst_max, sizeof(float) * mx.size(), cudaMemcpyDeviceToHost, s));
    FE_CUDA(cudaMemcpyAsync(&hflags, flags, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
    FE_CUDA(cudaStreamSynchronize(s));
    knn_flags_check(hflags);
    for (int b = 0; b < n_instances; ++b) {
      const long long nnz = eb[b + 1] - eb[b];
      if (nnz <= 0 || !(mx[b] > 0.0f)) throw Error("The CSR graph has no usable UMAP edges.");
      if (nnz > INT_MAX) throw Error("UMAP graph exceeds 2^31 - 1 entries.");
    }
    n_edges = eb[n_instances];
  }
  FE_CUDA(cudaMemcpyAsync(d_vb, vb.data(), sizeof(int) * vb.size(), cudaMemcpyHostToDevice, s));
  for (int b = 0; b < n_instances; ++b)
    FE_CUDA(cudaMemcpyAsync(job.y + vb[b], init_u[b], sizeof(float) * 2 * (std::size_t)sizes[b],
                            cudaMemcpyHostToDevice, s));
  FE_CUDA(cudaStreamSynchronize(s));
  double av = 0.0, bv = 0.0;
  umap_ab_params(1.0, min_dist, &av, &bv);
  const UmapParams p{n, n_epochs, negative_sample_rate, seed, learning_rate, (float)av, (float)bv,
                     repulsion_strength};
  job.edge_begin = d_eb;
  job.vert_begin = d_vb;
  job.ninst = n_instances;
  cudaEvent_t ev[2] = {nullptr, nullptr};
  for (auto& e : ev) FE_CUDA(cudaEventCreate(&e));
  FE_CUDA(cudaEventRecord(ev[0], s));
  job.run(heads, tails, period, n_edges, p);
  FE_CUDA(cudaEventRecord(ev[1], s));
  for (int b = 0; b < n_instances; ++b)
    FE_CUDA(cudaMemcpyAsync(out_u[b], job.y + vb[b], sizeof(float) * 2 * (std::size_t)sizes[b],
                            cudaMemcpyDeviceToHost, s));
  FE_CUDA(cudaStreamSynchronize(s));
  float ms = 0.0f;
  cudaEventElapsedTime(&ms, ev[0], ev[1]);
  for (auto& e : ev) cudaEventDestroy(e);
  if (sgd_ms) *sgd_ms = ms;
}

}  // namespace fe

extern "C" {

int fastembedr_cuda_umap_batch_from_knn(int n_instances, const int* sizes, const int* indices, const float* distances,
                                        const float* init, int k, int index_offset, int n_epochs,
                                        int negative_sample_rate, float learning_rate, float min_dist,
                                        float repulsion_strength, unsigned int seed, float* out, float* sgd_ms) {
  return fe::guarded([&] {
    if (!sizes || !indices || !distances || !init || !out) throw fe::Error("null UMAP batch pointer");
    if (n_instances < 1) throw fe::Error("invalid CUDA UMAP batch parameters");
    std::vector<const int*> iu(n_instances);
    std::vector<const float*> du(n_instances), yu(n_instances);
    std::vector<float*> ou(n_instances);
    std::size_t at = 0;
    for (int b = 0; b < n_instances; ++b) {
      iu[b] = indices + at * k;
      du[b] = distances + at * k;
      yu[b] = init + 2 * at;
      ou[b] = out + 2 * at;
      at += (std::size_t)std::max(sizes[b], 0);
    }
    fe::umap_batch_job(n_instances, sizes, iu, du, yu, ou, false, k, index_offset, n_epochs, negative_sample_rate,
                       learning_rate, min_dist, repulsion_strength, seed, sgd_ms);
  });
}

int fastembedr_cuda_umap_batch_from_knn_rows(int n_instances, const int* sizes, const int* const* indices,
                                             const float* const* distances, const float* const* inits, int k,
                                             int index_offset, int n_epochs, int negative_sample_rate,
                                             float learning_rate, float min_dist, float repulsion_strength,
                                             unsigned int seed, float* const* outs, float* sgd_ms) {
  return fe::guarded([&] {
    if (!sizes || !indices || !distances || !inits || !outs || n_instances < 1)
      throw fe::Error("null UMAP batch pointer");
    std::vector<const int*> iu(indices, indices + n_instances);
    std::vector<const float*> du(distances, distances + n_instances), yu(inits, inits + n_instances);
    std::vector<float*> ou(outs, outs + n_instances);
    for (int b = 0; b < n_instances; ++b)
      if (!iu[b] || !du[b] || !yu[b] || !ou[b]) throw fe::Error("null UMAP batch pointer");
    fe::umap_batch_job(n_instances, sizes, iu, du, yu, ou, true, k, index_offset, n_epochs, negative_sample_rate,
                       learning_rate, min_dist, repulsion_strength, seed, sgd_ms);
  });
}

void fastembedr_umap_find_ab_params(double spread, double min_dist, double* a, double* b) {
  double av = 0.0, bv = 0.0;
  fe::umap_ab_params(spread, min_dist, &av, &bv);
  if (a) *a = av;
  if (b) *b = bv;
}

int fastembedr_cuda_umap_spectral_init_from_knn(const int* indices, const float* distances, int n, int k,
                                                int index_offset, int spectral_n_iter, double init_scale, int seed,
                                                double* out) {
  return fe::guarded([&] {
    if (!indices || !distances || !out) throw fe::Error("null host pointer");
    if (n < 2 || k < 1 || spectral_n_iter < 1) throw fe::Error("invalid spectral initialization parameters");
    auto draws = std::async(std::launch::async, fe::spectral_draws, n, seed);
    fe::Stream st;
    const std::size_t items = (std::size_t)n * k;
    int* d_idx = nullptr;
    float* d_dist = nullptr;
    fe::Arena a;
    a.reserve(&d_idx, items);
    a.reserve(&d_dist, items);
    a.commit("UMAP spectral start input");
    fe::upload(d_idx, indices, sizeof(int) * items, st.s);
    fe::upload(d_dist, distances, sizeof(float) * items, st.s);
    FE_CUDA(cudaStreamSynchronize(st.s));
    fe::umap_knn_spectral_job(d_idx, d_dist, n, k, index_offset, 0, 0, 1.0f, 0.01f, 1.0f, spectral_n_iter,
                              init_scale, (unsigned)seed, out, nullptr, &draws);
  });
}

int fastembedr_cuda_umap_spectral_init_csr(const int* offsets, const int* neighbors, const float* weights, int n,
                                           int spectral_n_iter, double init_scale, int seed, double* out) {
  return fe::guarded([&] {
    if (!offsets || !neighbors || !weights || !out) throw fe::Error("null host pointer");
    if (n < 1 || spectral_n_iter < 1) throw fe::Error("invalid spectral initialization parameters");
    // validate_csr_inputs (src/fast_knn_umap.cpp:747-785), plus the symmetry the GPU start relies on
    if (offsets[0] != 0) throw fe::Error("First CSR offset must be zero");
    for (int i = 1; i <= n; ++i)
      if (offsets[i] < offsets[i - 1]) throw fe::Error("CSR offsets must be non-decreasing");
    const long long nnz = offsets[n];
    int lo = INT_MAX, hi = INT_MIN;
    for (long long p = 0; p < nnz; ++p) {
      lo = std::min(lo, neighbors[p]);
      hi = std::max(hi, neighbors[p]);
    }
    const int off = (nnz > 0 && lo >= 1 && hi <= n) ? 1 : 0;
    std::vector<int> nb0((std::size_t)std::max<long long>(nnz, 1));
    for (int r = 0; r < n; ++r) {
      int last = -1;
      for (int p = offsets[r]; p < offsets[r + 1]; ++p) {
        const int j = neighbors[p] - off;
        if (j < 0 || j >= n) throw fe::Error("CSR neighbor index out of range");
        if (j == r) throw fe::Error("CSR graph must not contain self-neighbors");
        if (j < last) throw fe::Error("CSR neighbors must be sorted within each row");
        last = j;
        if (!std::isfinite(weights[p]) || !(weights[p] > 0.0f)) throw fe::Error("CSR weights must be positive and finite");
        nb0[p] = j;
      }
    }
    for (int r = 0; r < n; ++r)
      for (int p = offsets[r]; p < offsets[r + 1]; ++p) {
        const int j = nb0[p];
        const int* b = nb0.data() + offsets[j];
        const int* e = nb0.data() + offsets[j + 1];
        const int* it = std::lower_bound(b, e, r);
        if (it == e || *it != r || weights[offsets[j] + (it - b)] != weights[p])
          throw fe::Error("the GPU spectral start needs a symmetric CSR graph (w_ij == w_ji)");
      }
    fe::Stream st;
    cudaStream_t s = st.s;
    int *d_off = nullptr, *d_nb = nullptr;
    float* d_w = nullptr;
    double* d_out = nullptr;
    fe::Arena a;
    a.reserve(&d_off, n + 1);
    a.reserve(&d_nb, (std::size_t)std::max<long long>(nnz, 1));
    a.reserve(&d_w, (std::size_t)std::max<long long>(nnz, 1));
    a.reserve(&d_out, 2 * (std::size_t)n);
    a.commit("UMAP spectral start (CSR)");
    FE_CUDA(cudaMemcpyAsync(d_off, offsets, sizeof(int) * (n + 1), cudaMemcpyHostToDevice, s));
    if (nnz > 0) {
      fe::upload(d_nb, nb0.data(), sizeof(int) * nnz, s);
      fe::upload(d_w, weights, sizeof(float) * nnz, s);
    }
    fe::umap_spectral_start(d_off, d_nb, d_w, n, nnz, spectral_n_iter, init_scale, seed, d_out, s);
    FE_CUDA(cudaMemcpyAsync(out, d_out, sizeof(double) * 2 * (std::size_t)n, cudaMemcpyDeviceToHost, s));
    FE_CUDA(cudaStreamSynchronize(s));
  });
}

int fastembedr_cuda_umap_knn_spectral(const int* indices, const float* distances, int n, int k, int index_offset,
                                      int n_epochs, int negative_sample_rate, float learning_rate, float min_dist,
                                      float repulsion_strength, int spectral_n_iter, double init_scale,
                                      unsigned int seed, float* out) {
  return fe::guarded([&] {
    if (!indices || !distances || !out) throw fe::Error("null host pointer");
    if (n < 2 || k < 1 || n_epochs < 1 || negative_sample_rate < 0 || !(learning_rate > 0.0f) || min_dist < 0.0f ||
        !(repulsion_strength > 0.0f) || spectral_n_iter < 1)
      throw fe::Error("invalid CUDA UMAP parameters");
    auto draws = std::async(std::launch::async, fe::spectral_draws, n, (int)seed);
    fe::Stream st;
    const std::size_t items = (std::size_t)n * k;
    int* d_idx = nullptr;
    float* d_dist = nullptr;
    fe::Arena a;
    a.reserve(&d_idx, items);
    a.reserve(&d_dist, items);
    a.commit("UMAP input");
    fe::upload(d_idx, indices, sizeof(int) * items, st.s);
    fe::upload(d_dist, distances, sizeof(float) * items, st.s);
    FE_CUDA(cudaStreamSynchronize(st.s));
    fe::umap_knn_spectral_job(d_idx, d_dist, n, k, index_offset, n_epochs, negative_sample_rate, learning_rate,
                              min_dist, repulsion_strength, spectral_n_iter, init_scale, seed, nullptr, out, &draws);
  });
}

int fastembedr_cuda_spectral_init_from_knn(const int* indices, const double* distances, int n, int k,
                                           int spectral_n_iter, unsigned int seed, int index_offset, float* out) {
  return fe::guarded([&] {
    if (!indices || !distances || !out) throw fe::Error("null host pointer");
    if (n < 2 || k < 1 || k > 256 || spectral_n_iter < 1)
      throw fe::Error("invalid spectral initialization dimensions or parameters");
    fe::Stream st;
    cudaStream_t s = st.s;
    const std::size_t items = (std::size_t)n * k;
    int* d_idx = nullptr;
    double* d_dd = nullptr;
    float* d_dist = nullptr;
    float2* d_y = nullptr;
    fe::Arena a;
    a.reserve(&d_idx, items);
    a.reserve(&d_dd, items);
    a.reserve(&d_dist, items);
    a.reserve(&d_y, n);
    a.commit("CUDA spectral initialization");
    fe::upload(d_idx, indices, sizeof(int) * items, s);
    fe::upload(d_dd, distances, sizeof(double) * items, s);
    fe::umap_double_to_float_kernel<<<std::max(1, std::min(fe::ceil_div((long long)items, 256), fe::sm_count() * 8)),
                                      256, 0, s>>>(d_dd, d_dist, (long long)items);
    FE_LAUNCH("umap_double_to_float_kernel");
    fe::validate_knn(d_idx, d_dist, n, k, index_offset, s);
    fe::UmapGraph g;
    fe::umap_build_graph(d_idx, d_dist, n, k, index_offset, g, s);
    fe::umap_diffusion_start(g, spectral_n_iter, seed, d_y, s);
    FE_CUDA(cudaMemcpyAsync(out, d_y, sizeof(float) * 2 * (std::size_t)n, cudaMemcpyDeviceToHost, s));
    FE_CUDA(cudaStreamSynchronize(s));
  });
}

int fastembedr_cuda_umap_from_knn_spectral(const int* indices, const double* distances, int n, int k, int n_epochs,
                                           int negative_sample_rate, float learning_rate, float a, float b,
                                           float repulsion_strength, int spectral_n_iter, unsigned int seed,
                                           int index_offset, int optimizer_mode, float* out) {
  return umap_spectral_host(indices, distances, n, k, n_epochs, negative_sample_rate, learning_rate, a, b,
                            repulsion_strength, spectral_n_iter, seed, index_offset, optimizer_mode, out);
}

int fastembedr_cuda_umap_from_knn_spectral_float(const int* indices, const float* distances, int n, int k,
                                                 int n_epochs, int negative_sample_rate, float learning_rate, float a,
                                                 float b, float repulsion_strength, int spectral_n_iter,
                                                 unsigned int seed, int index_offset, int optimizer_mode, float* out) {
  return umap_spectral_host(indices, distances, n, k, n_epochs, negative_sample_rate, learning_rate, a, b,
                            repulsion_strength, spectral_n_iter, seed, index_offset, optimizer_mode, out);
}

int fastembedr_cuda_umap_from_device_knn_spectral_float(const int* device_indices, const float* device_distances,
                                                        int n, int k, int n_epochs, int negative_sample_rate,
                                                        float learning_rate, float a, float b,
                                                        float repulsion_strength, int spectral_n_iter,
                                                        unsigned int seed, int index_offset, int optimizer_mode,
                                                        int binary_graph, float* out) {
  return fe::guarded([&] {
    if (!device_indices || !device_distances || !out) throw fe::Error("null device pointer");
    fe::check_spectral_job(n, k, n_epochs, negative_sample_rate, learning_rate, spectral_n_iter, optimizer_mode);
    fe::umap_spectral_job(device_indices, device_distances, n, k, n_epochs, negative_sample_rate, learning_rate, a,
                          b, repulsion_strength, spectral_n_iter, seed, index_offset, binary_graph != 0, out);
  });
}

int fastembedr_cuda_umap_from_knn(const int* indices, const float* distances, const float* init, int n, int k,
                                  int index_offset, int n_epochs, int negative_sample_rate, float learning_rate,
                                  float min_dist, float repulsion_strength, unsigned int seed, float* out) {
  return fastembedr_cuda_umap_from_knn_profile(indices, distances, init, n, k, index_offset, n_epochs,
                                               negative_sample_rate, learning_rate, min_dist, repulsion_strength, seed,
                                               out, nullptr, nullptr);
}

}  // extern "C"
