// Exact O(n^2) t-SNE quantities on the GPU: repulsive forces with the all-pairs Z, and the
// KL divergence of evaluate_kl_f (fastEmbedR src/tsne_neighbors.cpp:1034-1059, :1338-1365).
// Pair terms are FP32; each thread accumulates a tile of 1024 partners in FP32 and folds the
// tile into FP64, so the n^2 sums carry FP64 error at N = 1M (5e11 pairs).
#include <algorithm>
#include <cfloat>
#include <cmath>

#include "tsne_exact.cuh"

namespace fe {

constexpr int kPairTile = 1024;

// rep_i = -sum_j q_ij^2 (y_i - y_j) (unnormalised) and zrow_i = sum_{j != i} q_ij.
__global__ void __launch_bounds__(256)
exact_pairs_kernel(const float2* __restrict__ y, int n, double* __restrict__ rep, double* __restrict__ zrow) {
  __shared__ float2 tile[kPairTile];
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const float2 yi = i < n ? y[i] : make_float2(0.0f, 0.0f);
  double gx = 0.0, gy = 0.0, z = 0.0;
  for (int t0 = 0; t0 < n; t0 += kPairTile) {
    const int cnt = min(kPairTile, n - t0);
    __syncthreads();
    for (int t = threadIdx.x; t < cnt; t += blockDim.x) tile[t] = y[t0 + t];
    __syncthreads();
    float fx = 0.0f, fy = 0.0f, fz = 0.0f;
    for (int t = 0; t < cnt; ++t) {
      const float2 yj = tile[t];
      const float dx = yi.x - yj.x, dy = yi.y - yj.y;
      const float q = 1.0f / (1.0f + (dx * dx + dy * dy));
      const float w = (t0 + t == i) ? 0.0f : 1.0f;
      fz += w * q;
      fx += w * q * q * dx;
      fy += w * q * q * dy;
    }
    gx += fx;
    gy += fy;
    z += fz;
  }
  if (i < n) {
    rep[2 * (long long)i] = -gx;
    rep[2 * (long long)i + 1] = -gy;
    zrow[i] = z;
  }
}

// Row sums of q for the KL normaliser only (no force), reused for large n.
__global__ void __launch_bounds__(256)
sum_q_rows_kernel(const float2* __restrict__ y, int n, double* __restrict__ zrow) {
  __shared__ float2 tile[kPairTile];
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const float2 yi = i < n ? y[i] : make_float2(0.0f, 0.0f);
  double z = 0.0;
  for (int t0 = 0; t0 < n; t0 += kPairTile) {
    const int cnt = min(kPairTile, n - t0);
    __syncthreads();
    for (int t = threadIdx.x; t < cnt; t += blockDim.x) tile[t] = y[t0 + t];
    __syncthreads();
    float fz = 0.0f;
    for (int t = 0; t < cnt; ++t) {
      const float2 yj = tile[t];
      const float dx = yi.x - yj.x, dy = yi.y - yj.y;
      fz += 1.0f / (1.0f + (dx * dx + dy * dy));
    }
    z += fz;
  }
  if (i < n) zrow[i] = z - 1.0;  // remove the j == i term (q = 1 exactly)
}

// Exact repulsion of selected points against every point, partners split into gridDim.y slices:
// part[(slice * 3 + c) * n_rows + r] holds slice sums of -q^2 dx, -q^2 dy and q (c = 0, 1, 2) for
// the point y[inv[rows[r]]], excluding the point itself. FP32 pair terms, FP64 tile sums.
__global__ void __launch_bounds__(256)
exact_rows_kernel(const float2* __restrict__ y, int n, const int* __restrict__ rows, const int* __restrict__ inv,
                  int n_rows, int slice, double* __restrict__ part) {
  __shared__ float2 tile[kPairTile];
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  const int si = r < n_rows ? inv[rows[r]] : -1;
  const float2 yi = si >= 0 ? y[si] : make_float2(0.0f, 0.0f);
  const int j0 = blockIdx.y * slice, j1 = min(n, j0 + slice);
  double gx = 0.0, gy = 0.0, z = 0.0;
  for (int t0 = j0; t0 < j1; t0 += kPairTile) {
    const int cnt = min(kPairTile, j1 - t0);
    __syncthreads();
    for (int t = threadIdx.x; t < cnt; t += blockDim.x) tile[t] = y[t0 + t];
    __syncthreads();
    float fx = 0.0f, fy = 0.0f, fz = 0.0f;
    for (int t = 0; t < cnt; ++t) {
      const float2 yj = tile[t];
      const float dx = yi.x - yj.x, dy = yi.y - yj.y;
      const float q = 1.0f / (1.0f + (dx * dx + dy * dy));
      const float w = (t0 + t == si) ? 0.0f : 1.0f;
      fz += w * q;
      fx += w * q * q * dx;
      fy += w * q * q * dy;
    }
    gx += fx;
    gy += fy;
    z += fz;
  }
  if (r < n_rows) {
    const long long b = (long long)blockIdx.y * 3 * n_rows;
    part[b + r] = -gx;
    part[b + n_rows + r] = -gy;
    part[b + 2LL * n_rows + r] = z;
  }
}

// out[c * n_rows + r] = sum over slices (in slice order) of part.
__global__ void sum_slices_kernel(const double* __restrict__ part, int n_rows, int slices, double* __restrict__ out) {
  const long long m = 3LL * n_rows;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < m; t += (long long)gridDim.x * blockDim.x) {
    double acc = 0.0;
    for (int sl = 0; sl < slices; ++sl) acc += part[sl * m + t];
    out[t] = acc;
  }
}

__global__ void reduce_double_kernel(const double* __restrict__ v, int n, double* out) {
  __shared__ double part[1024];
  double s = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) s += v[i];
  part[threadIdx.x] = s;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) part[threadIdx.x] += part[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = part[0];
}

// KL = sum_CSR p log((p + 1e-9) / (q / Z + 1e-9)); Z rounded to float as the reference keeps it.
// Row i of P belongs to the point at y[inv[i]] (inv = nullptr: y is in row order); columns index y.
__global__ void __launch_bounds__(256)
kl_rows_kernel(const int* __restrict__ row_ptr, const int* __restrict__ col, const float* __restrict__ val,
               const float2* __restrict__ y, const float2* __restrict__ y_rows, const int* __restrict__ inv, int n,
               const double* __restrict__ zsum, double* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double z = (double)(float)fmax(*zsum, (double)FLT_MIN);
  const float2 yi = inv ? y[inv[i]] : y_rows[i];
  double acc = 0.0;
  for (int p = row_ptr[i]; p < row_ptr[i + 1]; ++p) {
    const float2 yj = y[col[p]];
    const float dx = yi.x - yj.x, dy = yi.y - yj.y;
    float d2 = 0.0f;
    d2 = __fadd_rn(d2, __fmul_rn(dx, dx));
    d2 = __fadd_rn(d2, __fmul_rn(dy, dy));
    const double pv = (double)val[p];
    const double q = (1.0 / (1.0 + (double)d2)) / z;
    acc += pv * log((pv + 1e-9) / (q + 1e-9));
  }
  out[i] = acc;
}

void exact_repulsion(const float* d_y, int n, double* d_rep, double* d_zrow, double* d_ztotal, cudaStream_t s) {
  exact_pairs_kernel<<<ceil_div(n, 256), 256, 0, s>>>(reinterpret_cast<const float2*>(d_y), n, d_rep, d_zrow);
  FE_LAUNCH("exact_pairs_kernel");
  reduce_double_kernel<<<1, 1024, 0, s>>>(d_zrow, n, d_ztotal);
  FE_LAUNCH("reduce_double_kernel");
}

int exact_rows_slices(int n, int n_rows) {
  const int row_blocks = ceil_div(n_rows, 256);
  const int want = std::max(1, ceil_div(8 * sm_count(), row_blocks));
  return std::min(want, std::max(1, ceil_div(n, kPairTile)));
}

void exact_repulsion_rows(const float* d_y, int n, const int* d_rows, const int* d_inv, int n_rows, double* d_part,
                          double* d_out, double* d_zrow, double* d_ztotal, cudaStream_t s) {
  const float2* y = reinterpret_cast<const float2*>(d_y);
  const int slices = exact_rows_slices(n, n_rows);
  const int slice = ceil_div(n, slices);
  exact_rows_kernel<<<dim3(ceil_div(n_rows, 256), slices), 256, 0, s>>>(y, n, d_rows, d_inv, n_rows, slice, d_part);
  FE_LAUNCH("exact_rows_kernel");
  sum_slices_kernel<<<std::max(1, std::min(ceil_div(3 * n_rows, 256), sm_count() * 4)), 256, 0, s>>>(
      d_part, n_rows, slices, d_out);
  FE_LAUNCH("sum_slices_kernel");
  sum_q_rows_kernel<<<ceil_div(n, 256), 256, 0, s>>>(y, n, d_zrow);
  FE_LAUNCH("sum_q_rows_kernel");
  reduce_double_kernel<<<1, 1024, 0, s>>>(d_zrow, n, d_ztotal);
  FE_LAUNCH("reduce_double_kernel");
}

void exact_kl(const DeviceCsr& P, const float* d_y, const int* d_inv, double* d_zrow, double* d_work,
              double* d_scalars, cudaStream_t s) {
  exact_kl_range(P.row_ptr, P.col, P.val, P.n, d_y, d_inv, 0, d_zrow, d_work, d_scalars, s);
}

void exact_kl_range(const int* row_ptr, const int* col, const float* val, int n, const float* d_y, const int* d_inv,
                    int y_begin, double* d_zrow, double* d_work, double* d_scalars, cudaStream_t s) {
  const float2* y = reinterpret_cast<const float2*>(d_y);
  sum_q_rows_kernel<<<ceil_div(n, 256), 256, 0, s>>>(y + y_begin, n, d_zrow);
  FE_LAUNCH("sum_q_rows_kernel");
  reduce_double_kernel<<<1, 1024, 0, s>>>(d_zrow, n, d_scalars);
  FE_LAUNCH("reduce_double_kernel");
  kl_rows_kernel<<<ceil_div(n, 256), 256, 0, s>>>(row_ptr, col, val, y, y + y_begin, d_inv, n, d_scalars, d_work);
  FE_LAUNCH("kl_rows_kernel");
  reduce_double_kernel<<<1, 1024, 0, s>>>(d_work, n, d_scalars + 1);
  FE_LAUNCH("reduce_double_kernel");
}

}  // namespace fe
