// PCA start of t-SNE on the GPU.
//
// The reference's device PCA initialisation (opentsne_fft_from_knn_impl,
// src/embedding_cuda_kernels.cpp:5860-5893) centres the columns of the data on the host
// (raft_tsvd_scores_to_device, :3379-3437: column means in double, float data minus float mean),
// calls RAPIDS RAFT's tsvd_fit_transform with the COV_EIG_DQ solver and sign flipping based on
// the scores (:3495-3525; RAFT is not vendored and the reference pins no version), then centres
// the two score columns and scales both by 1e-4 / the larger standard deviation
// (tsvd_scores_to_rowmajor_init_kernel :1337, finalize_tsne_pca_init_stats_kernel :1352,
// scale_tsne_pca_init_kernel :1411). The published algorithm of that solver: the Gram matrix
// C = Xc^T Xc, its symmetric eigendecomposition, components = eigenvectors of the largest
// eigenvalues, scores = Xc V, and each score column's sign chosen so that its entry of largest
// magnitude is positive.
//
// Here every step runs on the GPU: column means and centring, C accumulated in FP64 from exact
// float products (tiles of C x row slices, partials summed in a fixed order), a cyclic Jacobi
// eigendecomposition in FP64 on one block (round-robin ordering: the p/2 disjoint rotations of a
// step are applied together), scores in FP64, the sign rule, and the reference's scaling.
#include <algorithm>
#include <cfloat>
#include <cmath>

#include "pca.cuh"

namespace fe {
namespace {

constexpr int kGramTile = 16;
constexpr int kGramRows = 64;
constexpr int kGramSlices = 64;
constexpr int kJacobiThreads = 1024;
constexpr int kJacobiSweeps = 30;
constexpr int kPcaMaxFeatures = 1024;

__global__ void pca_mean_kernel(const float* __restrict__ X, int n, double* __restrict__ mean,
                                int* __restrict__ bad) {
  __shared__ double sm[32];
  const float* col = X + (long long)blockIdx.x * n;
  double s = 0.0;
  bool finite = true;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const float v = col[i];
    finite &= isfinite(v);
    s += (double)v;
  }
  if (!finite) atomicExch(bad, 1);
  s = warp_sum(s);
  if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += sm[w];
    mean[blockIdx.x] = t / (double)n;
  }
}

__global__ void pca_center_kernel(float* __restrict__ X, long long total, int n, const double* __restrict__ mean) {
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total; t += (long long)gridDim.x * blockDim.x)
    X[t] = X[t] - (float)mean[t / n];
}

// partial[slice][a][b] = sum over the slice's rows of Xc[r, a] Xc[r, b] for the block's 16 x 16
// tile of C (blockIdx.x = tile, blockIdx.y = row slice); products of floats are exact in FP64.
__global__ void __launch_bounds__(kGramTile * kGramTile)
pca_gram_kernel(const float* __restrict__ X, int n, int p, int tiles, double* __restrict__ partial) {
  __shared__ float sa[kGramTile][kGramRows + 1];
  __shared__ float sb[kGramTile][kGramRows + 1];
  const int ta = blockIdx.x / tiles, tb = blockIdx.x % tiles;
  const int la = threadIdx.x / kGramTile, lb = threadIdx.x % kGramTile;
  const int a = ta * kGramTile + la, b = tb * kGramTile + lb;
  double acc = 0.0;
  const long long chunks = (n + kGramRows - 1) / kGramRows;
  for (long long ch = blockIdx.y; ch < chunks; ch += gridDim.y) {
    const long long r0 = ch * kGramRows;
    __syncthreads();
    for (int t = threadIdx.x; t < kGramTile * kGramRows; t += blockDim.x) {
      const int c = t / kGramRows, r = t % kGramRows;
      const long long row = r0 + r;
      const int ca = ta * kGramTile + c, cb = tb * kGramTile + c;
      sa[c][r] = (row < n && ca < p) ? X[(long long)ca * n + row] : 0.0f;
      sb[c][r] = (row < n && cb < p) ? X[(long long)cb * n + row] : 0.0f;
    }
    __syncthreads();
#pragma unroll 8
    for (int r = 0; r < kGramRows; ++r) acc += (double)sa[la][r] * (double)sb[lb][r];
  }
  if (a < p && b < p) partial[((long long)blockIdx.y * p + a) * p + b] = acc;
}

__global__ void pca_gram_sum_kernel(const double* __restrict__ partial, int p, int slices, double* __restrict__ C) {
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < p * p; t += gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int y = 0; y < slices; ++y) s += partial[(long long)y * p * p + t];
    C[t] = s;
  }
}

// Cyclic Jacobi on the symmetric p x p matrix A (row-major, global memory), one block. V
// accumulates the rotations (A_final = V^T A V). Round-robin ordering over m = p rounded up to even
// (index m - 1 is a dummy when p is odd): step t pairs position 0 with position m - 1 and the
// others around a circle; the disjoint rotations of a step are applied together, columns first
// (A J, V J), then rows (J^T (A J)). Stops when the off-diagonal mass is below 1e-30 of the
// diagonal mass, or after kJacobiSweeps sweeps. order[0..1]: indices of the two largest
// eigenvalues.
__global__ void __launch_bounds__(kJacobiThreads)
pca_jacobi_kernel(double* __restrict__ A, double* __restrict__ V, int p, int* __restrict__ order) {
  __shared__ int s_i[kPcaMaxFeatures / 2], s_j[kPcaMaxFeatures / 2];
  __shared__ double s_c[kPcaMaxFeatures / 2], s_s[kPcaMaxFeatures / 2];
  __shared__ double s_red[2][kJacobiThreads / 32];
  __shared__ bool s_done;
  const int m = p + (p & 1), half = m / 2;
  for (int t = threadIdx.x; t < p * p; t += blockDim.x) V[t] = (t / p == t % p) ? 1.0 : 0.0;
  __syncthreads();
  for (int sweep = 0; sweep < kJacobiSweeps; ++sweep) {
    // convergence test on the current matrix
    double off = 0.0, dia = 0.0;
    for (int t = threadIdx.x; t < p * p; t += blockDim.x) {
      const double v = A[t];
      if (t / p == t % p) dia += v * v; else off += v * v;
    }
    off = warp_sum(off);
    dia = warp_sum(dia);
    if ((threadIdx.x & 31) == 0) {
      s_red[0][threadIdx.x >> 5] = off;
      s_red[1][threadIdx.x >> 5] = dia;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      double o = 0.0, d = 0.0;
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
        o += s_red[0][w];
        d += s_red[1][w];
      }
      s_done = !(o > 1e-30 * d);
    }
    __syncthreads();
    if (s_done) break;
    for (int step = 0; step < m - 1; ++step) {
      for (int k = threadIdx.x; k < half; k += blockDim.x) {
        const int u = k == 0 ? 0 : ((k - 1 + step) % (m - 1)) + 1;
        const int w = ((m - 2 - k + step) % (m - 1)) + 1;  // position m - 1 - k around the circle
        const int i = min(u, w), j = max(u, w);
        double c = 1.0, sn = 0.0;
        if (j < p) {
          const double aij = A[(long long)i * p + j];
          if (aij != 0.0) {
            const double tau = (A[(long long)j * p + j] - A[(long long)i * p + i]) / (2.0 * aij);
            const double t = (tau >= 0.0 ? 1.0 : -1.0) / (fabs(tau) + sqrt(1.0 + tau * tau));
            c = 1.0 / sqrt(1.0 + t * t);
            sn = t * c;
          }
        }
        s_i[k] = i;
        s_j[k] = j;
        s_c[k] = c;
        s_s[k] = sn;
      }
      __syncthreads();
      // columns: A <- A J, V <- V J
      for (int t = threadIdx.x; t < half * p; t += blockDim.x) {
        const int k = t / p, r = t % p;
        const int i = s_i[k], j = s_j[k];
        if (j >= p || s_s[k] == 0.0) continue;
        const double c = s_c[k], sn = s_s[k];
        const double ai = A[(long long)r * p + i], aj = A[(long long)r * p + j];
        A[(long long)r * p + i] = c * ai - sn * aj;
        A[(long long)r * p + j] = sn * ai + c * aj;
        const double vi = V[(long long)r * p + i], vj = V[(long long)r * p + j];
        V[(long long)r * p + i] = c * vi - sn * vj;
        V[(long long)r * p + j] = sn * vi + c * vj;
      }
      __syncthreads();
      // rows: A <- J^T A
      for (int t = threadIdx.x; t < half * p; t += blockDim.x) {
        const int k = t / p, col = t % p;
        const int i = s_i[k], j = s_j[k];
        if (j >= p || s_s[k] == 0.0) continue;
        const double c = s_c[k], sn = s_s[k];
        const double ai = A[(long long)i * p + col], aj = A[(long long)j * p + col];
        A[(long long)i * p + col] = c * ai - sn * aj;
        A[(long long)j * p + col] = sn * ai + c * aj;
      }
      __syncthreads();
    }
  }
  if (threadIdx.x == 0) {
    int b0 = 0, b1 = -1;
    for (int i = 1; i < p; ++i)
      if (A[(long long)i * p + i] > A[(long long)b0 * p + b0]) b0 = i;
    for (int i = 0; i < p; ++i)
      if (i != b0 && (b1 < 0 || A[(long long)i * p + i] > A[(long long)b1 * p + b1])) b1 = i;
    order[0] = b0;
    order[1] = b1;
  }
}

struct ArgMax {
  double v;
  long long i;
};

// scores (FP64 sums over the features) and block partial argmax |score| per component
__global__ void pca_scores_kernel(const float* __restrict__ X, int n, int p, const double* __restrict__ V,
                                  const int* __restrict__ order, double2* __restrict__ sc,
                                  ArgMax* __restrict__ part) {
  __shared__ ArgMax s_m[2][32];
  const int c0 = order[0], c1 = order[1];
  ArgMax m0{-1.0, 0}, m1{-1.0, 0};
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
    double x = 0.0, y = 0.0;
    for (int a = 0; a < p; ++a) {
      const double v = X[(long long)a * n + r];
      x += v * V[(long long)a * p + c0];
      y += v * V[(long long)a * p + c1];
    }
    sc[r] = make_double2(x, y);
    if (fabs(x) > m0.v) m0 = ArgMax{fabs(x), r};
    if (fabs(y) > m1.v) m1 = ArgMax{fabs(y), r};
  }
  // first index among equal maxima: compare (value desc, index asc)
  for (int o = 16; o > 0; o >>= 1) {
    const double v0 = __shfl_down_sync(0xffffffffu, m0.v, o), v1 = __shfl_down_sync(0xffffffffu, m1.v, o);
    const long long i0 = __shfl_down_sync(0xffffffffu, m0.i, o), i1 = __shfl_down_sync(0xffffffffu, m1.i, o);
    if (v0 > m0.v || (v0 == m0.v && i0 < m0.i)) m0 = ArgMax{v0, i0};
    if (v1 > m1.v || (v1 == m1.v && i1 < m1.i)) m1 = ArgMax{v1, i1};
  }
  if ((threadIdx.x & 31) == 0) {
    s_m[0][threadIdx.x >> 5] = m0;
    s_m[1][threadIdx.x >> 5] = m1;
  }
  __syncthreads();
  if (threadIdx.x < 2) {
    ArgMax best{-1.0, 0};
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
      const ArgMax q = s_m[threadIdx.x][w];
      if (q.v > best.v || (q.v == best.v && q.i < best.i)) best = q;
    }
    part[blockIdx.x * 2 + threadIdx.x] = best;
  }
}

// signs from the largest-magnitude scores, then the reference's t-SNE scaling (one block):
// sign, float scores (non-finite -> 0), moments, then (v - mean) * 1e-4 / max sd.
__global__ void pca_finish_kernel(const double2* __restrict__ sc, int n, const ArgMax* __restrict__ part, int nparts,
                                  float2* __restrict__ init) {
  __shared__ double s_sign[2];
  __shared__ double s_red[5][32];
  __shared__ double s_stat[3];
  if (threadIdx.x < 2) {
    ArgMax best{-1.0, 0};
    for (int b = 0; b < nparts; ++b) {
      const ArgMax q = part[b * 2 + threadIdx.x];
      if (q.v > best.v || (q.v == best.v && q.i < best.i)) best = q;
    }
    const double v = threadIdx.x == 0 ? sc[best.i].x : sc[best.i].y;
    s_sign[threadIdx.x] = v < 0.0 ? -1.0 : 1.0;
  }
  __syncthreads();
  double m[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
  for (int r = threadIdx.x; r < n; r += blockDim.x) {
    float x = (float)(s_sign[0] * sc[r].x), y = (float)(s_sign[1] * sc[r].y);
    if (!isfinite(x)) x = 0.0f;
    if (!isfinite(y)) y = 0.0f;
    init[r] = make_float2(x, y);
    const double dx = x, dy = y;
    m[0] += dx;
    m[1] += dy;
    m[2] += dx * dx;
    m[3] += dx * dy;
    m[4] += dy * dy;
  }
  for (int c = 0; c < 5; ++c) {
    const double v = warp_sum(m[c]);
    if ((threadIdx.x & 31) == 0) s_red[c][threadIdx.x >> 5] = v;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double t[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
    for (int c = 0; c < 5; ++c)
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t[c] += s_red[c][w];
    const double dn = (double)max(n, 1), den = (double)max(n - 1, 1);
    const double ssx = fmax(t[2] - t[0] * t[0] / dn, 0.0), ssy = fmax(t[4] - t[1] * t[1] / dn, 0.0);
    const double sd = fmax(sqrt(ssx / den), sqrt(ssy / den));
    s_stat[0] = t[0] / dn;
    s_stat[1] = t[1] / dn;
    s_stat[2] = (isfinite(sd) && sd > 0.0) ? 1.0e-4 / sd : 1.0;
  }
  __syncthreads();
  for (int r = threadIdx.x; r < n; r += blockDim.x) {
    const float2 v = init[r];
    init[r] = make_float2((float)(((double)v.x - s_stat[0]) * s_stat[2]), (float)(((double)v.y - s_stat[1]) * s_stat[2]));
  }
}

}  // namespace

void pca_tsne_start(float* X, int n, int p, float2* init, cudaStream_t s) {
  if (n < 2 || p < 2) throw Error("invalid dimensions in device PCA initialization");
  if (p > kPcaMaxFeatures)
    throw Error("device PCA initialization supports at most 1024 features; reduce the dimension first");
  const int tiles = ceil_div(p, kGramTile);
  const int slices = std::max(1, std::min(kGramSlices, ceil_div(n, kGramRows)));
  const int sblocks = std::max(1, std::min(ceil_div(n, 256), sm_count() * 4));
  double *mean = nullptr, *partial = nullptr, *C = nullptr, *V = nullptr;
  double2* sc = nullptr;
  ArgMax* am = nullptr;
  int *bad = nullptr, *order = nullptr;
  Arena w;
  w.reserve(&mean, p);
  w.reserve(&partial, (std::size_t)slices * p * p);
  w.reserve(&C, (std::size_t)p * p);
  w.reserve(&V, (std::size_t)p * p);
  w.reserve(&sc, n);
  w.reserve(&am, 2 * (std::size_t)sblocks);
  w.reserve(&bad, 1);
  w.reserve(&order, 2);
  w.commit("device PCA initialization");
  FE_CUDA(cudaMemsetAsync(bad, 0, sizeof(int), s));
  pca_mean_kernel<<<p, 256, 0, s>>>(X, n, mean, bad);
  FE_LAUNCH("pca_mean_kernel");
  int h_bad = 0;
  FE_CUDA(cudaMemcpyAsync(&h_bad, bad, sizeof(int), cudaMemcpyDeviceToHost, s));
  FE_CUDA(cudaStreamSynchronize(s));
  if (h_bad) throw Error("PCA input must contain only finite values");
  const long long total = (long long)n * p;
  pca_center_kernel<<<std::max(1, (int)std::min<long long>(ceil_div(total, 256), sm_count() * 8)), 256, 0, s>>>(
      X, total, n, mean);
  FE_LAUNCH("pca_center_kernel");
  pca_gram_kernel<<<dim3(tiles * tiles, slices), kGramTile * kGramTile, 0, s>>>(X, n, p, tiles, partial);
  FE_LAUNCH("pca_gram_kernel");
  pca_gram_sum_kernel<<<std::max(1, std::min(ceil_div(p * p, 256), sm_count())), 256, 0, s>>>(partial, p, slices, C);
  FE_LAUNCH("pca_gram_sum_kernel");
  pca_jacobi_kernel<<<1, kJacobiThreads, 0, s>>>(C, V, p, order);
  FE_LAUNCH("pca_jacobi_kernel");
  pca_scores_kernel<<<sblocks, 256, 0, s>>>(X, n, p, V, order, sc, am);
  FE_LAUNCH("pca_scores_kernel");
  pca_finish_kernel<<<1, 1024, 0, s>>>(sc, n, am, sblocks, init);
  FE_LAUNCH("pca_finish_kernel");
  FE_CUDA(cudaStreamSynchronize(s));
}

}  // namespace fe
