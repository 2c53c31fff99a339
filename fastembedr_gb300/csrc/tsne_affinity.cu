// t-SNE affinities on the GPU: KNN validation, perplexity bisection and the bit-exact
// symmetrised CSR.
//
// Reference behaviour followed (fastEmbedR):
//   - index/distance validation and messages: src/tsne_neighbors.cpp:630-640
//   - per-row bisection: src/tsne_neighbors.cpp:532-614 (control flow, tolerance 1e-5,
//     200 iterations, uniform fallback) evaluated with FP32 exp and FP64 sums as in the
//     FP64 test oracle tests/testthat/helper-tsne-reference.R:1-54
//   - symmetrisation: src/tsne_neighbors.cpp:616-724 (self edges skipped, duplicate
//     directed edges summed in double, value = float(sum) * float(0.5 / total))
//
// GPU layout: the CPU sorts 64-bit (min, max) pair keys once; here every directed edge is
// emitted into both endpoint rows (bucketed by an atomic counting pass), each row bucket is
// sorted by (column, p bits) with an always-ascending bitonic network, and runs of equal
// columns are reduced. This yields exactly the CPU's CSR structure: the same column set per
// row, ascending, with the same double sums per pair.
#include <cfloat>
#include <climits>
#include <cmath>
#include <cstdlib>
#include <vector>

#include "sort.cuh"
#include "tsne.cuh"

namespace fe {

// ---------------------------------------------------------------- validation
__global__ void validate_knn_kernel(const int* __restrict__ idx, const float* __restrict__ dist,
                                    long long total, int n, int offset, unsigned* flags) {
  unsigned local = 0u;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
       t += (long long)gridDim.x * blockDim.x) {
    const int nb = idx[t] - offset;
    if (nb < 0 || nb >= n) local |= 1u;
    const float d = dist[t];
    if (!isfinite(d) || d < 0.0f) local |= 2u;
  }
  if (local) atomicOr(flags, local);
}

void validate_knn_async(const int* d_idx, const float* d_dist, int n, int k, int offset, unsigned* d_flags,
                        cudaStream_t s) {
  const long long total = (long long)n * k;
  const int blocks = std::max(1, std::min(ceil_div(total, 256), sm_count() * 8));
  validate_knn_kernel<<<blocks, 256, 0, s>>>(d_idx, d_dist, total, n, offset, d_flags);
  FE_LAUNCH("validate_knn_kernel");
}

void knn_flags_check(unsigned flags) {
  if (flags & 1u) throw Error("KNN indices are out of range.");
  if (flags & 2u) throw Error("KNN distances must be finite and non-negative.");
}

void validate_knn(const int* d_idx, const float* d_dist, int n, int k, int offset, cudaStream_t s) {
  unsigned* d_flags = nullptr;
  FE_CUDA(cudaMallocAsync(&d_flags, sizeof(unsigned), s));
  FE_CUDA(cudaMemsetAsync(d_flags, 0, sizeof(unsigned), s));
  validate_knn_async(d_idx, d_dist, n, k, offset, d_flags, s);
  unsigned flags = 0u;
  FE_CUDA(cudaMemcpyAsync(&flags, d_flags, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
  FE_CUDA(cudaStreamSynchronize(s));
  FE_CUDA(cudaFreeAsync(d_flags, s));
  knn_flags_check(flags);
}

// ---------------------------------------------------------------- bisection
// One thread per row. The CTA stages its rows' distances (column-major in global memory, so
// each column read is coalesced) in shared memory with a stride of k + 1 floats (consecutive rows
// on distinct banks), next to each row's shifted squared distances s_j = d_j^2 - min d^2 (FP64,
// rounded to float once). Every thread bisects its own row: per entry FP32 exp of -beta s_j and
// compensated (Kahan) FP32 sums, whose error (~1e-7 relative) stays far inside the 1e-6 band
// around the stop tolerance in which an iteration is re-evaluated from the distances with FP64
// exp and FP64 sums; entropy, the update of beta and the stop test are FP64. The FP64 pipe of
// this part is narrow, so the per-entry work stays on the FP32 pipe. The probabilities overwrite
// the row's distances and the CTA stores them row-major with coalesced writes.
constexpr int kBisectRows = 128;

__global__ void __launch_bounds__(kBisectRows)
row_probabilities_kernel(const float* __restrict__ dist, int n, int k, double log_perplexity,
                         float* __restrict__ p_out, double* __restrict__ entropy_out) {
  extern __shared__ float tile[];  // blockDim.x rows x (k + 1) distances, then as many s_j
  const int rows = blockDim.x, stride = k + 1;
  float* stile = tile + (long long)rows * stride;
  const int r0 = blockIdx.x * rows;
  const int nrows = min(rows, n - r0);
  for (int t = threadIdx.x; t < nrows * k; t += rows) {
    const int j = t / nrows, rr = t - j * nrows;
    tile[rr * stride + j] = dist[(long long)j * n + r0 + rr];
  }
  __syncthreads();
  const int rr = threadIdx.x;
  if (rr < nrows) {
    float* d = tile + rr * stride;
    // zero-spread test in float arithmetic, as compute_row_probabilities_float does it
    float min_f = FLT_MAX, max_f = 0.0f;
    double min_d2 = DBL_MAX;
    for (int j = 0; j < k; ++j) {
      const float df = d[j] * d[j];
      min_f = fminf(min_f, df);
      max_f = fmaxf(max_f, df);
      const double dj = d[j];
      min_d2 = fmin(min_d2, dj * dj);  // exact: a float squared fits in a double
    }
    double entropy_eval;
    if (max_f - min_f <= FLT_EPSILON * fmaxf(1.0f, max_f)) {
      const float u = 1.0f / (float)k;
      for (int j = 0; j < k; ++j) d[j] = u;
      entropy_eval = log((double)k);
    } else {
      float* sf = stile + rr * stride;
      for (int j = 0; j < k; ++j) {
        const double dj = d[j];
        sf[j] = (float)(dj * dj - min_d2);
      }
      double beta = 1.0, beta_min = -DBL_MAX, beta_max = DBL_MAX;
      double beta_eval = beta, sum_eval = 1.0;
      bool exact_eval = false;
      entropy_eval = 0.0;
      for (int it = 0; it < 200; ++it) {
        const float nb = (float)(-beta);
        float ps = 0.0f, pc = 0.0f, ws = 0.0f, wc = 0.0f;
        for (int j = 0; j < k; ++j) {
          const float sj = sf[j];
          const float p = expf(nb * sj);
          const float yp = p - pc;
          const float tp = ps + yp;
          pc = (tp - ps) - yp;
          ps = tp;
          const float yw = sj * p - wc;
          const float tw = ws + yw;
          wc = (tw - ws) - yw;
          ws = tw;
        }
        double sp = (double)ps - (double)pc;
        double sw = (double)ws - (double)wc;
        double entropy = beta * sw / sp + log(sp);
        double diff = entropy - log_perplexity;
        exact_eval = false;
        // The stop test is the only decision FP32 exp can flip: re-evaluate near its boundary
        // with FP64 exp so the bisection follows the FP64 path.
        if (fabs(fabs(diff) - 1e-5) < 1e-6) {
          sp = 0.0;
          sw = 0.0;
          for (int j = 0; j < k; ++j) {
            const double dj = d[j];
            const double s = dj * dj - min_d2;
            const double p = exp(-beta * s);
            sp += p;
            sw += s * p;
          }
          entropy = beta * sw / sp + log(sp);
          diff = entropy - log_perplexity;
          exact_eval = true;
        }
        beta_eval = beta;
        sum_eval = sp;
        entropy_eval = entropy;
        if (fabs(diff) < 1e-5) break;
        if (diff > 0.0) {
          beta_min = beta;
          beta = (beta_max == DBL_MAX) ? beta * 2.0 : 0.5 * (beta + beta_max);
        } else {
          beta_max = beta;
          beta = (beta_min == -DBL_MAX) ? beta * 0.5 : 0.5 * (beta + beta_min);
        }
        if (!isfinite(beta)) break;
      }
      const double inv = 1.0 / sum_eval;
      const float nb = (float)(-beta_eval);
      for (int j = 0; j < k; ++j) {
        const double dj = d[j];
        const double p = exact_eval ? exp(-beta_eval * (dj * dj - min_d2)) : (double)expf(nb * sf[j]);
        d[j] = (float)(p * inv);
      }
    }
    if (entropy_out) entropy_out[r0 + rr] = entropy_eval;
  }
  __syncthreads();
  float* out = p_out + (long long)r0 * k;
  for (int t = threadIdx.x; t < nrows * k; t += rows) {
    const int q = t / k, j = t - q * k;
    out[t] = tile[q * stride + j];
  }
}

void row_probabilities(const int* /*d_idx*/, const float* d_dist, int n, int k, float perplexity,
                       float* d_p, double* d_entropy, cudaStream_t s) {
  int rows = kBisectRows;
  while (rows > 1 && (std::size_t)rows * (k + 1) * 2 * sizeof(float) > 112 * 1024) rows >>= 1;
  const std::size_t smem = (std::size_t)rows * (k + 1) * 2 * sizeof(float);
  if (smem > 48 * 1024)
    FE_CUDA(cudaFuncSetAttribute(row_probabilities_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)smem));
  row_probabilities_kernel<<<ceil_div(n, rows), rows, smem, s>>>(d_dist, n, k, std::log((double)perplexity), d_p,
                                                                 d_entropy);
  FE_LAUNCH("row_probabilities_kernel");
}

// ---------------------------------------------------------------- scan
// Exclusive scan of n int32 counts into n + 1 int64 offsets (three passes).
constexpr int kScanBlock = 1024;

__global__ void scan_blocks_kernel(const int* __restrict__ in, long long* __restrict__ out, int n,
                                   long long* __restrict__ block_sums) {
  __shared__ long long warp_tot[32];
  const int i = blockIdx.x * kScanBlock + threadIdx.x;
  long long v = i < n ? in[i] : 0;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  long long x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const long long y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) warp_tot[warp] = x;
  __syncthreads();
  if (warp == 0) {
    long long w = warp_tot[lane];
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const long long y = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += y;
    }
    warp_tot[lane] = w;
  }
  __syncthreads();
  const long long before = (warp > 0 ? warp_tot[warp - 1] : 0) + x - v;
  if (i < n) out[i] = before;
  if (threadIdx.x == kScanBlock - 1) block_sums[blockIdx.x] = warp_tot[31];
}

__global__ void scan_sums_kernel(long long* sums, int nb, long long* total_out) {
  // single block: sequential carry over chunks of 1024
  __shared__ long long warp_tot[32];
  __shared__ long long carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int base = 0; base < nb; base += kScanBlock) {
    const int i = base + threadIdx.x;
    const long long v = i < nb ? sums[i] : 0;
    long long x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const long long y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) warp_tot[warp] = x;
    __syncthreads();
    if (warp == 0) {
      long long w = warp_tot[lane];
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const long long y = __shfl_up_sync(0xffffffffu, w, o);
        if (lane >= o) w += y;
      }
      warp_tot[lane] = w;
    }
    __syncthreads();
    const long long excl = carry + (warp > 0 ? warp_tot[warp - 1] : 0) + x - v;
    if (i < nb) sums[i] = excl;
    __syncthreads();
    if (threadIdx.x == 0) carry += warp_tot[31];
    __syncthreads();
  }
  if (threadIdx.x == 0) *total_out = carry;
}

__global__ void scan_add_kernel(long long* out, int n, const long long* sums) {
  const int i = blockIdx.x * kScanBlock + threadIdx.x;
  if (i < n) out[i] += sums[blockIdx.x];
}

// out must hold n + 1 values; out[n] = total. tmp must hold ceil(n / 1024) values.
void exclusive_scan(const int* in, long long* out, int n, long long* tmp, cudaStream_t s) {
  const int nb = std::max(1, ceil_div(n, kScanBlock));
  scan_blocks_kernel<<<nb, kScanBlock, 0, s>>>(in, out, n, tmp);
  FE_LAUNCH("scan_blocks_kernel");
  scan_sums_kernel<<<1, kScanBlock, 0, s>>>(tmp, nb, out + n);
  FE_LAUNCH("scan_sums_kernel");
  scan_add_kernel<<<nb, kScanBlock, 0, s>>>(out, n, tmp);
  FE_LAUNCH("scan_add_kernel");
}

// ---------------------------------------------------------------- symmetrisation
__global__ void count_edges_kernel(const int* __restrict__ idx, int n, int k, int offset,
                                   int* __restrict__ counts) {
  const long long total = (long long)n * k;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
       t += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(t % n);
    const int nb = idx[t] - offset;  // column-major: t = j * n + i
    if (nb == i) continue;
    atomicAdd(counts + i, 1);
    atomicAdd(counts + nb, 1);
  }
}

__device__ __forceinline__ unsigned long long edge_key(int col, float p) {
  return ((unsigned long long)(unsigned)col << 32) | (unsigned long long)__float_as_uint(p);
}

__global__ void fill_buckets_kernel(const int* __restrict__ idx, const float* __restrict__ p, int n, int k,
                                    int offset, unsigned long long* __restrict__ cursor,
                                    unsigned long long* __restrict__ bucket) {
  const long long total = (long long)n * k;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
       t += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(t % n);
    const int j = (int)(t / n);
    const int nb = idx[t] - offset;
    if (nb == i) continue;
    const float pv = p[(long long)i * k + j];
    bucket[atomicAdd(cursor + i, 1ull)] = edge_key(nb, pv);
    bucket[atomicAdd(cursor + nb, 1ull)] = edge_key(i, pv);
  }
}

constexpr int kSortThreads = 256;
constexpr int kSortCap = 8192;  // entries of a row sorted in shared memory

// Sort each row bucket by (column, p bits), then collapse runs of equal columns: the compacted
// (column, float(sum)) entries are written back to the start of the bucket, `ucount` gets the
// unique count and `row_mass` the double sum of the row's pair sums. Rows of up to 256 entries
// (nearly all) take one warp each (sort_unique_small_rows_kernel); longer rows are listed for a
// CTA each (this kernel), and rows above kSortCap for the global-memory path.
constexpr int kWarpSortCap = 256;
constexpr int kWarpSortWarps = 8;

// One warp per row of at most kWarpSortCap entries: the same ascending bitonic network in the
// warp's slice of shared memory, then the run sums and the row mass with exactly the arithmetic
// of the CTA path for such a row (thread t of 256 owning position t: each run summed in order by
// its first position, warp sums over positions 32w .. 32w + 31, added for w = 0 .. 7), so the
// result does not depend on which kernel took the row.
__global__ void __launch_bounds__(kWarpSortWarps * 32)
sort_unique_small_rows_kernel(unsigned long long* __restrict__ bucket, const long long* __restrict__ offs, int n,
                              int* __restrict__ ucount, double* __restrict__ row_mass, int* __restrict__ mid_rows,
                              int* __restrict__ mid_count) {
  __shared__ unsigned long long sm[kWarpSortWarps][kWarpSortCap];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  unsigned long long* a = sm[wib];
  const int warps = gridDim.x * kWarpSortWarps;
  for (int row = blockIdx.x * kWarpSortWarps + wib; row < n; row += warps) {
    const long long b = offs[row];
    const int len = (int)(offs[row + 1] - b);
    if (len > kWarpSortCap) {
      if (lane == 0) mid_rows[atomicAdd(mid_count, 1)] = row;
      continue;
    }
    int pw = 1;
    while (pw < len) pw <<= 1;
    for (int t = lane; t < pw; t += 32) a[t] = t < len ? bucket[b + t] : ~0ull;
    __syncwarp();
    for (int size = 2; size <= pw && len > 1; size <<= 1) {
      const int half = size >> 1;
      for (int t = lane; t < pw / 2; t += 32) {
        const int blk = t / half, off = t % half;
        const int i = blk * size + off, j = blk * size + size - 1 - off;
        const unsigned long long x = a[i], y = a[j];
        if (y < x) {
          a[i] = y;
          a[j] = x;
        }
      }
      __syncwarp();
      for (int stride = half >> 1; stride > 0; stride >>= 1) {
        for (int t = lane; t < pw / 2; t += 32) {
          const int blk = t / stride, off = t % stride;
          const int i = blk * 2 * stride + off, j = i + stride;
          const unsigned long long x = a[i], y = a[j];
          if (y < x) {
            a[i] = y;
            a[j] = x;
          }
        }
        __syncwarp();
      }
    }
    int cnt = 0;
    double tot = 0.0;
    for (int w = 0; w < kWarpSortCap / 32; ++w) {
      const int t = w * 32 + lane;
      bool start = false;
      if (t < len) start = (t == 0) || ((a[t] >> 32) != (a[t - 1] >> 32));
      const unsigned ballot = __ballot_sync(0xffffffffu, start);
      double sum = 0.0;
      if (start) {
        const unsigned col = (unsigned)(a[t] >> 32);
        for (int u = t; u < len && (unsigned)(a[u] >> 32) == col; ++u) sum += (double)__uint_as_float((unsigned)a[u]);
        const int pos = cnt + __popc(ballot & ((1u << lane) - 1u));
        bucket[b + pos] = ((unsigned long long)col << 32) | (unsigned long long)__float_as_uint((float)sum);
      }
      cnt += __popc(ballot);
      tot += warp_sum(sum);
    }
    if (lane == 0) {
      row_mass[row] = tot;
      ucount[row] = cnt;
    }
    __syncwarp();
  }
}

__global__ void __launch_bounds__(kSortThreads)
sort_unique_rows_kernel(unsigned long long* __restrict__ bucket, const long long* __restrict__ offs,
                        const int* __restrict__ rows, const int* __restrict__ row_count, int* __restrict__ ucount,
                        double* __restrict__ row_mass, int* __restrict__ big_rows, int* __restrict__ big_count) {
  extern __shared__ unsigned long long sm[];
  __shared__ int warp_cnt[kSortThreads / 32];
  __shared__ double warp_mass[kSortThreads / 32];
  const int count = *row_count;
  for (int q = blockIdx.x; q < count; q += gridDim.x) {
    const int row = rows[q];
    const long long b = offs[row];
    const int len = (int)(offs[row + 1] - b);
    if (len > kSortCap) {
      if (threadIdx.x == 0) big_rows[atomicAdd(big_count, 1)] = row;
      continue;
    }
    int pw = 1;
    while (pw < len) pw <<= 1;
    for (int t = threadIdx.x; t < pw; t += blockDim.x) sm[t] = t < len ? bucket[b + t] : ~0ull;
    __syncthreads();
    if (len > 1) bitonic_sort<false>(sm, len, pw);
    // run starts and sums; each start owns the run that follows it
    int my_cnt = 0;
    double my_mass = 0.0;
    for (int base = 0; base < len; base += blockDim.x) {
      const int t = base + threadIdx.x;
      bool start = false;
      if (t < len) start = (t == 0) || ((sm[t] >> 32) != (sm[t - 1] >> 32));
      const unsigned ballot = __ballot_sync(0xffffffffu, start);
      const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
      if (lane == 0) warp_cnt[warp] = __popc(ballot);
      __syncthreads();
      int before = 0;
      for (int w = 0; w < warp; ++w) before += warp_cnt[w];
      if (start) {
        double sum = 0.0;
        const unsigned col = (unsigned)(sm[t] >> 32);
        for (int u = t; u < len && (unsigned)(sm[u] >> 32) == col; ++u) sum += (double)__uint_as_float((unsigned)sm[u]);
        const int pos = my_cnt + before + __popc(ballot & ((1u << lane) - 1u));
        bucket[b + pos] = ((unsigned long long)col << 32) | (unsigned long long)__float_as_uint((float)sum);
        my_mass += sum;
      }
      int chunk_total = 0;
      for (int w = 0; w < (int)(blockDim.x / 32); ++w) chunk_total += warp_cnt[w];
      my_cnt += chunk_total;  // identical in every thread
      __syncthreads();
    }
    // row mass: block reduction in a fixed order
    double m = warp_sum(my_mass);
    if ((threadIdx.x & 31) == 0) warp_mass[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x == 0) {
      double tot = 0.0;
      for (int w = 0; w < (int)(blockDim.x / 32); ++w) tot += warp_mass[w];
      row_mass[row] = tot;
      ucount[row] = my_cnt;
    }
    __syncthreads();
  }
}

// Rows longer than kSortCap: one CTA sorts the bucket in place in global memory, then a
// single thread collapses the runs (rare, pathological in-degree).
__global__ void __launch_bounds__(1024)
sort_unique_big_rows_kernel(unsigned long long* __restrict__ bucket, const long long* __restrict__ offs,
                            const int* __restrict__ big_rows, const int* __restrict__ big_count,
                            int* __restrict__ ucount, double* __restrict__ row_mass) {
  const int count = *big_count;
  for (int r = blockIdx.x; r < count; r += gridDim.x) {
    const int row = big_rows[r];
    const long long b = offs[row];
    const int len = (int)(offs[row + 1] - b);
    int pw = 1;
    while (pw < len) pw <<= 1;
    bitonic_sort<true>(bucket + b, len, pw);
    if (threadIdx.x == 0) {
      int w = 0;
      double mass = 0.0;
      for (int t = 0; t < len;) {
        const unsigned col = (unsigned)(bucket[b + t] >> 32);
        double sum = 0.0;
        while (t < len && (unsigned)(bucket[b + t] >> 32) == col) {
          sum += (double)__uint_as_float((unsigned)bucket[b + t]);
          ++t;
        }
        bucket[b + w] = ((unsigned long long)col << 32) | (unsigned long long)__float_as_uint((float)sum);
        ++w;
        mass += sum;
      }
      ucount[row] = w;
      row_mass[row] = mass;
    }
    __syncthreads();
  }
}

// Deterministic totals: block b sums the rows [first[b], first[b + 1]) of instance b with a
// fixed assignment and a fixed tree (a single instance is first = {0, n}).
__global__ void total_mass_kernel(const double* __restrict__ row_mass, const int* __restrict__ first,
                                  double* __restrict__ out_total, float* __restrict__ out_norm) {
  __shared__ double part[1024];
  const int r0 = first[blockIdx.x], r1 = first[blockIdx.x + 1];
  double s = 0.0;
  for (int i = r0 + threadIdx.x; i < r1; i += blockDim.x) s += row_mass[i];
  part[threadIdx.x] = s;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) part[threadIdx.x] += part[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    const double total = 0.5 * part[0];  // every pair sum appears in both of its rows
    out_total[blockIdx.x] = total;
    out_norm[blockIdx.x] = (float)(0.5 / total);
  }
}

// Entries of a row past its `real` count are padding (the row itself, value 0): they contribute
// exactly nothing to forces and KL.
__global__ void fill_csr_kernel(const unsigned long long* __restrict__ bucket, const long long* __restrict__ offs,
                                const long long* __restrict__ row_ptr64, const int* __restrict__ real, int n,
                                const int* __restrict__ first, int ninst, const float* __restrict__ norm,
                                int* __restrict__ row_ptr, int* __restrict__ col, float* __restrict__ val) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (warp > n) return;
  if (lane == 0) row_ptr[warp] = (int)row_ptr64[warp];
  if (warp == n) return;
  int lo = 0, hi = ninst - 1;  // the instance holding this row
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (first[mid] <= warp) lo = mid;
    else hi = mid - 1;
  }
  const float nm = norm[lo];
  const long long src = offs[warp];
  const long long dst = row_ptr64[warp];
  const int cnt = (int)(row_ptr64[warp + 1] - dst);
  const int have = real[warp];
  for (int t = lane; t < cnt; t += 32) {
    if (t < have) {
      const unsigned long long e = bucket[src + t];
      col[dst + t] = (int)(e >> 32);
      val[dst + t] = __uint_as_float((unsigned)e) * nm;
    } else {
      col[dst + t] = warp;
      val[dst + t] = 0.0f;
    }
  }
}

__global__ void pad_rows_kernel(int* __restrict__ count, const int2* __restrict__ pads, int m) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < m) count[pads[t].x] += pads[t].y;
}

void symmetrise(const int* d_idx, const float* d_p, int n, int k, int offset, DeviceCsr& out, cudaStream_t s) {
  symmetrise_batch(d_idx, d_p, n, k, offset, std::vector<int>{0, n}, out, nullptr, s);
}

void symmetrise_batch(const int* d_idx, const float* d_p, int n, int k, int offset, const std::vector<int>& first,
                      DeviceCsr& out, std::vector<double>* totals, cudaStream_t s) {
  const int ninst = (int)first.size() - 1;
  if (ninst < 1 || first.front() != 0 || first.back() != n) throw Error("invalid t-SNE instance boundaries");
  const long long directed = (long long)n * k;
  const int nscan = std::max(1, ceil_div(n, kScanBlock));
  int* counts = nullptr;
  long long* offs = nullptr;
  long long* scan_tmp = nullptr;
  unsigned long long* cursor = nullptr;
  unsigned long long* bucket = nullptr;
  int* ucount = nullptr;
  double* row_mass = nullptr;
  int* big_rows = nullptr;
  int* big_count = nullptr;
  int* mid_rows = nullptr;
  int* mid_count = nullptr;
  long long* row_ptr64 = nullptr;
  double* d_total = nullptr;
  float* d_norm = nullptr;
  int* d_first = nullptr;
  int* pcount = nullptr;
  int2* d_pads = nullptr;
  Arena work;
  work.reserve(&counts, n);
  work.reserve(&offs, n + 1);
  work.reserve(&scan_tmp, nscan);
  work.reserve(&cursor, n);
  work.reserve(&bucket, 2 * directed);
  work.reserve(&ucount, n);
  work.reserve(&row_mass, n);
  work.reserve(&big_rows, n);
  work.reserve(&big_count, 1);
  work.reserve(&mid_rows, n);
  work.reserve(&mid_count, 1);
  work.reserve(&row_ptr64, n + 1);
  work.reserve(&d_total, ninst);
  work.reserve(&d_norm, ninst);
  work.reserve(&d_first, ninst + 1);
  if (ninst > 1) {
    work.reserve(&pcount, n);
    work.reserve(&d_pads, ninst);
  }
  work.commit("t-SNE symmetrisation workspace");
  FE_CUDA(cudaMemcpyAsync(d_first, first.data(), sizeof(int) * (ninst + 1), cudaMemcpyHostToDevice, s));

  const int grid = std::max(1, std::min(ceil_div(directed, 256), sm_count() * 16));
  FE_CUDA(cudaMemsetAsync(counts, 0, sizeof(int) * n, s));
  FE_CUDA(cudaMemsetAsync(big_count, 0, sizeof(int), s));
  count_edges_kernel<<<grid, 256, 0, s>>>(d_idx, n, k, offset, counts);
  FE_LAUNCH("count_edges_kernel");
  exclusive_scan(counts, offs, n, scan_tmp, s);
  FE_CUDA(cudaMemcpyAsync(cursor, offs, sizeof(long long) * n, cudaMemcpyDeviceToDevice, s));
  fill_buckets_kernel<<<grid, 256, 0, s>>>(d_idx, d_p, n, k, offset, cursor, bucket);
  FE_LAUNCH("fill_buckets_kernel");

  FE_CUDA(cudaMemsetAsync(mid_count, 0, sizeof(int), s));
  sort_unique_small_rows_kernel<<<std::max(1, std::min(ceil_div(n, kWarpSortWarps), sm_count() * 8)),
                                  kWarpSortWarps * 32, 0, s>>>(bucket, offs, n, ucount, row_mass, mid_rows, mid_count);
  FE_LAUNCH("sort_unique_small_rows_kernel");
  const std::size_t smem = kSortCap * sizeof(unsigned long long);
  FE_CUDA(cudaFuncSetAttribute(sort_unique_rows_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  sort_unique_rows_kernel<<<sm_count() * 3, kSortThreads, smem, s>>>(bucket, offs, mid_rows, mid_count, ucount,
                                                                     row_mass, big_rows, big_count);
  FE_LAUNCH("sort_unique_rows_kernel");
  sort_unique_big_rows_kernel<<<sm_count(), 1024, 0, s>>>(bucket, offs, big_rows, big_count, ucount, row_mass);
  FE_LAUNCH("sort_unique_big_rows_kernel");
  exclusive_scan(ucount, row_ptr64, n, scan_tmp, s);
  total_mass_kernel<<<ninst, 1024, 0, s>>>(row_mass, d_first, d_total, d_norm);
  FE_LAUNCH("total_mass_kernel");

  std::vector<double> tot(ninst);
  std::vector<long long> bounds(ninst + 1);
  for (int b = 0; b <= ninst; ++b)
    FE_CUDA(cudaMemcpyAsync(&bounds[b], row_ptr64 + first[b], sizeof(long long), cudaMemcpyDeviceToHost, s));
  FE_CUDA(cudaMemcpyAsync(tot.data(), d_total, sizeof(double) * ninst, cudaMemcpyDeviceToHost, s));
  FE_CUDA(cudaStreamSynchronize(s));
  long long nnz = bounds[ninst];
  double total = 0.0;
  for (int b = 0; b < ninst; ++b) {
    if (bounds[b + 1] <= bounds[b]) throw Error("KNN graph produced no non-self t-SNE edges.");
    if (!std::isfinite(tot[b]) || tot[b] <= 0.0) throw Error("t-SNE probability normalization failed.");
    total += tot[b];
  }
  const int* real = ucount;
  if (ninst > 1) {
    // every instance's entries start at a multiple of 4 (the attractive pass reads rows with
    // 128-bit loads aligned to the array, so an instance then reads its rows exactly as it does
    // alone): the last row of each instance is padded with zero entries
    std::vector<int2> pads;
    for (int b = 0; b + 1 < ninst; ++b) {
      const long long cnt = bounds[b + 1] - bounds[b];
      const int pad = (int)((4 - cnt % 4) % 4);
      if (pad) pads.push_back(make_int2(first[b + 1] - 1, pad));
    }
    if (!pads.empty()) {
      FE_CUDA(cudaMemcpyAsync(pcount, ucount, sizeof(int) * n, cudaMemcpyDeviceToDevice, s));
      FE_CUDA(cudaMemcpyAsync(d_pads, pads.data(), sizeof(int2) * pads.size(), cudaMemcpyHostToDevice, s));
      pad_rows_kernel<<<ceil_div((long long)pads.size(), 256), 256, 0, s>>>(pcount, d_pads, (int)pads.size());
      FE_LAUNCH("pad_rows_kernel");
      exclusive_scan(pcount, row_ptr64, n, scan_tmp, s);
      for (const int2& p : pads) nnz += p.y;
      FE_CUDA(cudaStreamSynchronize(s));
    }
  }
  if (nnz > INT_MAX) throw Error("symmetrised t-SNE graph exceeds 2^31 - 1 entries.");
  if (totals) *totals = tot;

  out.n = n;
  out.nnz = nnz;
  out.total_mass = total;
  out.arena.release();
  out.arena.reserve(&out.row_ptr, n + 1);
  out.arena.reserve(&out.col, nnz);
  out.arena.reserve(&out.val, nnz);
  out.arena.commit("t-SNE CSR");
  fill_csr_kernel<<<ceil_div((long long)(n + 1) * 32, 256), 256, 0, s>>>(bucket, offs, row_ptr64, real, n, d_first,
                                                                          ninst, d_norm, out.row_ptr, out.col, out.val);
  FE_LAUNCH("fill_csr_kernel");
  FE_CUDA(cudaStreamSynchronize(s));
}

int cuda_fft_grid_size(int n) {
  int g = 512;
  if (n < 20000) g = 256;
  if (n >= 100000) g = 1024;
  const char* env = std::getenv("FASTEMBEDR_TSNE_FFT_GRID");
  if (env && env[0]) {
    const int r = std::atoi(env);
    if (r == 32 || r == 64 || r == 128 || r == 256 || r == 512 || r == 1024) g = r;
  }
  return g;
}

// The reference CPU policy (tsne_fft_grid_size, src/tsne_neighbors.cpp:403-413 without its
// environment override): 128 nodes per side below 50,000 points, 256 from there.
int cpu_fft_grid_size(int n) { return n >= 50000 ? 256 : 128; }

// Default: the reference's bilinear stencil. FASTEMBEDR_TSNE_INTERPOLATION=lagrange selects
// 3-node Lagrange boxes (more accurate forces in L2, but an interpolant that is discontinuous
// at box edges, which measurably degrades the local neighbourhood structure of the result).
int interp_mode_from_env() {
  const char* env = std::getenv("FASTEMBEDR_TSNE_INTERPOLATION");
  if (env && (env[0] == 'l' || env[0] == 'L')) return kInterpLagrange3;
  return kInterpBilinear;
}

}  // namespace fe
