// Spectral start of UMAP on the GPU.
//
// Restates initialize_layout_csr (src/fast_knn_umap.cpp:2231-2528), as optimize_layout_csr
// (:3088-3205) calls it for spectral_knn_init(backend = "cpu") / umap_init: the symmetric
// normalised adjacency D^-1/2 W D^-1/2 of the fuzzy graph, a block of 8 vectors drawn from the
// reference's std::mt19937 / normal(0, 1e-4) x 1e4 stream, spectral_n_iter rounds of
// multiply + modified Gram-Schmidt against the trivial eigenvector sqrt(deg) / |sqrt(deg)| and
// the earlier columns, a Rayleigh-Ritz step (the 8 x 8 projected matrix, diagonalised by the
// reference's largest-off-diagonal Jacobi rotations), the two leading Ritz vectors centred,
// scaled to max |y| = 10 and jittered by the stream's normal(0, 1e-4) draws
// (scale_embedding_max_abs_and_jitter, :2705-2730), then the optional scale_embedding_sdev
// (:2681-2703).
//
// The random draws are made on the host in the reference's order (the column redraw of a
// vanishing Gram-Schmidt column included) and uploaded; every arithmetic step runs on the GPU in
// FP64 with the reference's operation order and no contraction (__d*_rn). Sums over points are
// reduced in a fixed block order, so results are deterministic and differ from the sequential
// CPU sums by rounding only.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <future>
#include <random>
#include <vector>

#include "umap_spectral.cuh"

namespace fe {
namespace {

constexpr int kSpThreads = 256;
constexpr int kSpMaxBlocks = 1024;
constexpr int kSpBlock = 8;                           // block size of the reference for 2 components
constexpr int kSpPairs = kSpBlock * (kSpBlock + 1) / 2;  // upper triangle of the projected matrix

int sp_blocks(int n) { return std::max(1, std::min(ceil_div(n, kSpThreads), kSpMaxBlocks)); }

// Fixed-order sum of `count` partials, valid in every thread of the block (all threads call). The
// loads go to L2: the partials may come from other blocks of the same launch.
__device__ double sum_partials(const double* __restrict__ part, int count) {
  __shared__ double s_total;
  if (threadIdx.x < 32) {
    double s = 0.0;
    int b = threadIdx.x;
    // the lane's partials in order; eight loads are issued before their adds
    for (; b + 7 * 32 < count; b += 8 * 32) {
      double v[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) v[u] = __ldcg(part + b + u * 32);
#pragma unroll
      for (int u = 0; u < 8; ++u) s = __dadd_rn(s, v[u]);
    }
    for (; b < count; b += 32) s = __dadd_rn(s, __ldcg(part + b));
    s = warp_sum(s);
    if (threadIdx.x == 0) s_total = s;
  }
  __syncthreads();
  const double r = s_total;
  __syncthreads();
  return r;
}

// The total of sum_partials computed by one full warp (every lane gets it).
__device__ double warp_total(const double* __restrict__ part, int count) {
  const int lane = threadIdx.x & 31;
  double s = 0.0;
  int b = lane;
  for (; b + 7 * 32 < count; b += 8 * 32) {
    double v[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) v[u] = __ldcg(part + b + u * 32);
#pragma unroll
    for (int u = 0; u < 8; ++u) s = __dadd_rn(s, v[u]);
  }
  for (; b < count; b += 32) s = __dadd_rn(s, __ldcg(part + b));
  return warp_sum(s);
}

// Block sum of v into *dst (fixed order: warp trees, then warps in order).
__device__ void block_partial_at(double v, double* __restrict__ dst) {
  __shared__ double s_w[kSpThreads / 32];
  v = warp_sum(v);
  if ((threadIdx.x & 31) == 0) s_w[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t = __dadd_rn(t, s_w[w]);
    *dst = t;
  }
}

__device__ void block_partial(double v, double* __restrict__ part) { block_partial_at(v, part + blockIdx.x); }

// deg[r] = float(sum of row r's weights in double)
__global__ void sp_degree_kernel(const int* __restrict__ offsets, const float* __restrict__ w, int n,
                                 float* __restrict__ deg) {
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int p = offsets[r]; p < offsets[r + 1]; ++p) s = __dadd_rn(s, (double)w[p]);
    deg[r] = (float)s;
  }
}

// nw[p] = float(w / sqrt(max(deg_r deg_j, 1e-24))): one warp per row, lanes over its entries.
__global__ void __launch_bounds__(kSpThreads)
sp_adjacency_kernel(const int* __restrict__ offsets, const int* __restrict__ nb, const float* __restrict__ w,
                    const float* __restrict__ deg, int n, float* __restrict__ nw) {
  const int lane = threadIdx.x & 31;
  const int warps = gridDim.x * (blockDim.x >> 5);
  for (int r = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); r < n; r += warps) {
    const double dr = (double)deg[r];
    for (int p = offsets[r] + lane; p < offsets[r + 1]; p += 32) {
      const double den = __dsqrt_rn(fmax(__dmul_rn(dr, (double)deg[nb[p]]), 1e-24));
      nw[p] = (float)__ddiv_rn((double)w[p], den);
    }
  }
}

// triv[r] = sqrt(max(deg_r, 0)); block partials of sum triv^2 (one thread per row, grid-stride
// with a fixed row-to-block assignment).
__global__ void __launch_bounds__(kSpThreads)
sp_trivial_kernel(const float* __restrict__ deg, int n, double* __restrict__ triv, double* __restrict__ part) {
  double acc = 0.0;
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
    const double t = __dsqrt_rn(fmax((double)deg[r], 0.0));
    triv[r] = t;
    acc = __dadd_rn(acc, __dmul_rn(t, t));
  }
  block_partial(acc, part);
}

__global__ void sp_normalise_trivial_kernel(double* __restrict__ triv, int n, const double* __restrict__ part,
                                            int nparts) {
  const double nrm = __dsqrt_rn(fmax(sum_partials(part, nparts), 1e-12));
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x)
    triv[r] = __ddiv_rn(triv[r], nrm);
}

// ---------------------------------------------------------------- subspace iteration
//
// The block subspace iteration runs as one cooperative launch: all rounds of multiply and modified
// Gram-Schmidt, with a grid barrier between dependent steps. Every sum over points keeps the
// partial structure of a grid of `nparts` = sp_blocks(n) blocks of kSpThreads threads ("virtual
// blocks": thread t of virtual block vb covers points vb * kSpThreads + t + k * nparts *
// kSpThreads), whatever the number of resident blocks that run them, so its value does not depend
// on the launch. Vectors written during the launch are read through L2 (__ldcg): another block
// may have written them, and L1 is not coherent.

constexpr long long kSpBarrierCycles = 4000000000LL;  // about 2 s at the SM clock

struct SpGrid {
  unsigned count, gen;  // barrier arrivals, barrier generation
  int error;            // 1: a barrier wait gave up
  int status;           // -1, or 16 * (round + 1) + column of a vanished Gram-Schmidt column
};

// Grid barrier number `bar` (0, 1, ... within a launch) of a cooperative launch (all blocks
// resident). Arrivals count up without reset, so barrier `bar` is complete at count G * (bar + 1).
// The last block to arrive first sums the partial arrays of the columns in `mask` (part + c *
// nparts) into totals[c], the sums the next step needs, then releases the others by writing the
// generation bar + 1. A wait is bounded: after kSpBarrierCycles the block records the error and
// returns false, and later barriers return false at once, so every block leaves the kernel.
__device__ bool sp_grid_sync(SpGrid* g, unsigned bar, unsigned mask, const double* part, int nparts,
                             double* totals) {
  __shared__ int s_ok, s_last;
  __syncthreads();
  if (threadIdx.x == 0) {
    s_ok = *(volatile int*)&g->error == 0;
    s_last = 0;
    if (s_ok) {
      __threadfence();
      s_last = atomicAdd(&g->count, 1u) == gridDim.x * (bar + 1) - 1;
    }
  }
  __syncthreads();
  if (!s_ok) return false;
  if (s_last) {
    __threadfence();
    const int w = threadIdx.x >> 5;
    if (w < kSpBlock && ((mask >> w) & 1u)) {
      const double t = warp_total(part + (long long)w * nparts, nparts);
      if ((threadIdx.x & 31) == 0) totals[w] = t;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      __threadfence();
      *(volatile unsigned*)&g->gen = bar + 1;
    }
  } else if (threadIdx.x == 0) {
    const long long t0 = clock64();
    while (*(volatile unsigned*)&g->gen < bar + 1) {
      if (clock64() - t0 > kSpBarrierCycles) {
        atomicExch(&g->error, 1);
        s_ok = 0;
        break;
      }
      __nanosleep(32);
    }
    __threadfence();
  }
  __syncthreads();
  return s_ok != 0;
}

// y[:, c] = A x[:, c] for the B columns. A warp works on four rows at once, eight lanes per row
// (lane = 8 * slot + column): per group of 8 entries of its row the slot's lanes load the
// entries' neighbours and weights (one each, the next group's loads issued ahead), pass them
// round by shuffles, and every lane gathers its column's 8 values and adds the products in CSR
// order. Each (row, column) sum is the sequential FP64 sum of the row, and all 32 lanes of a
// warp instruction on the FP64 pipe carry work.
__device__ void sp_multiply_rows(const int* __restrict__ offsets, const int* __restrict__ nb,
                                 const float* __restrict__ nw, int n, int B, const double* x, double* y) {
  const int lane = threadIdx.x & 31, slot = lane >> 3, c = lane & 7;
  const unsigned gmask = 0xffu << (slot * 8);
  const int slots = gridDim.x * (blockDim.x >> 5) * 4;
  const double* xc = x + (long long)(c < B ? c : 0) * n;
  for (int r = (blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5)) * 4 + slot; r < n; r += slots) {
    const int p0 = offsets[r], p1 = offsets[r + 1];
    double acc = 0.0;
    int j = 0;
    double w = 0.0;
    if (p0 + c < p1) {
      j = nb[p0 + c];
      w = (double)nw[p0 + c];
    }
    for (int base = p0; base < p1; base += 8) {
      const int cnt = min(8, p1 - base);
      int jn = 0;
      double wn = 0.0;
      if (base + 8 + c < p1) {
        jn = nb[base + 8 + c];
        wn = (double)nw[base + 8 + c];
      }
      double v[8];
#pragma unroll
      for (int t = 0; t < 8; ++t) {
        const int jt = __shfl_sync(gmask, j, t, 8);
        v[t] = t < cnt ? __ldcg(xc + jt) : 0.0;
      }
#pragma unroll
      for (int t = 0; t < 8; ++t) {
        const double wt = __shfl_sync(gmask, w, t, 8);
        if (t < cnt) acc = __dadd_rn(acc, __dmul_rn(wt, v[t]));
      }
      j = jn;
      w = wn;
    }
    if (c < B) y[(long long)c * n + r] = acc;
  }
}

__global__ void __launch_bounds__(kSpThreads)
sp_multiply_kernel(const int* __restrict__ offsets, const int* __restrict__ nb, const float* __restrict__ nw,
                   int n, int B, const double* __restrict__ x, double* __restrict__ y) {
  sp_multiply_rows(offsets, nb, nw, n, B, x, y);
}

// Block partials of acc[c] for the columns in `mask` into part[c * nparts + vb]: per column the
// order of block_partial_at (warp trees, then warps in order).
__device__ void sp_block_partials(const double (&acc)[kSpBlock], unsigned mask, double* part, int nparts, int vb) {
  __shared__ double s_red[kSpBlock][kSpThreads / 32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int c = 0; c < kSpBlock; ++c)
    if ((mask >> c) & 1u) {
      const double v = warp_sum(acc[c]);
      if (lane == 0) s_red[c][w] = v;
    }
  __syncthreads();
  if (threadIdx.x < kSpBlock && ((mask >> threadIdx.x) & 1u)) {
    double t = 0.0;
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) t = __dadd_rn(t, s_red[threadIdx.x][k]);
    part[(long long)threadIdx.x * nparts + vb] = t;
  }
  __syncthreads();
}

// Modified Gram-Schmidt of the columns from..B-1 of m against the trivial vector and the columns
// before them (columns below `from` are final), as a wavefront. Column c's step j (j = 0..c)
// subtracts its last dot times u_j (u_0 = triv, u_j = q_{j-1}) and forms the partials of its dot
// with v_j = q_j, or of its squared norm when j = c; a column is divided by its norm at the start
// of the step after its norm step. Step j needs q_j final, so every column whose next step has
// its v final advances in the same grid step: the pass takes 2 (B - from) + 1 grid steps instead
// of one per projection, and each column sees exactly the operations of the column-by-column
// order. The columns' post-multiply values are copied to `backup` first (restored by the host
// before a redraw resumes the pass). Returns 0 when done, 1 + c when column c vanished, -1 when a
// barrier gave up.
__device__ int sp_orthonormalise(double* m, double* backup, const double* __restrict__ triv, int n, int B, int from,
                                 int nparts, double* part, double* totals, SpGrid* grid, unsigned& bar) {
  // the first projection of every column, which the earlier columns do not change
  const unsigned all = ((1u << B) - 1u) & ~((1u << from) - 1u);
  for (int vb = blockIdx.x; vb < nparts; vb += gridDim.x) {
    double acc[kSpBlock];
#pragma unroll
    for (int c = 0; c < kSpBlock; ++c) acc[c] = 0.0;
    for (int i = vb * blockDim.x + threadIdx.x; i < n; i += nparts * blockDim.x) {
      const double t = triv[i];
#pragma unroll
      for (int c = 0; c < kSpBlock; ++c)
        if ((all >> c) & 1u) {
          const double x = __ldcg(m + (long long)c * n + i);
          backup[(long long)c * n + i] = x;
          acc[c] = __dadd_rn(acc[c], __dmul_rn(x, t));
        }
    }
    sp_block_partials(acc, all, part, nparts, vb);
  }
  if (!sp_grid_sync(grid, bar++, all, part, nparts, totals)) return -1;
  int jn[kSpBlock];  // next step of each column (block-uniform)
#pragma unroll
  for (int c = 0; c < kSpBlock; ++c) jn[c] = 0;
  int nfinal = from, pending = -1;
  while (nfinal < B) {
    double nrm = 0.0;
    const int fin = pending;
    if (fin >= 0) {
      nrm = __dsqrt_rn(__ldcg(totals + fin));
      if (nrm < 1e-10) return 1 + fin;
      nfinal = fin + 1;
    }
    // ready columns: not final, next step's v final (or the norm step); all share one step j
    int j = kSpBlock;
#pragma unroll
    for (int c = 0; c < kSpBlock; ++c)
      if (c >= nfinal && c < B && (jn[c] == c || jn[c] < nfinal)) j = min(j, jn[c]);
    unsigned ready = 0u;
#pragma unroll
    for (int c = 0; c < kSpBlock; ++c)
      if (c >= nfinal && c < B && jn[c] == j && (j == c || j < nfinal)) ready |= 1u << c;
    double d[kSpBlock];
#pragma unroll
    for (int c = 0; c < kSpBlock; ++c) d[c] = ((ready >> c) & 1u) ? __ldcg(totals + c) : 0.0;
    const double* u = j == 0 ? triv : m + (long long)(j - 1) * n;
    double* qf = fin >= 0 ? m + (long long)fin * n : nullptr;
    const double* qv = m + (long long)(j < kSpBlock ? j : 0) * n;
    for (int vb = blockIdx.x; vb < nparts; vb += gridDim.x) {
      double acc[kSpBlock];
#pragma unroll
      for (int c = 0; c < kSpBlock; ++c) acc[c] = 0.0;
      for (int i = vb * blockDim.x + threadIdx.x; i < n; i += nparts * blockDim.x) {
        double xf = 0.0;
        if (qf) {
          xf = __ddiv_rn(__ldcg(qf + i), nrm);
          qf[i] = xf;
        }
        if (ready) {
          const double ui = __ldcg(u + i);
          const double vi = j == fin ? xf : __ldcg(qv + i);
#pragma unroll
          for (int c = 0; c < kSpBlock; ++c)
            if ((ready >> c) & 1u) {
              double* qc = m + (long long)c * n;
              const double x = __dsub_rn(__ldcg(qc + i), __dmul_rn(d[c], ui));
              qc[i] = x;
              acc[c] = __dadd_rn(acc[c], __dmul_rn(x, j < c ? vi : x));
            }
        }
      }
      if (ready) sp_block_partials(acc, ready, part, nparts, vb);
    }
    pending = -1;
#pragma unroll
    for (int c = 0; c < kSpBlock; ++c)
      if ((ready >> c) & 1u) {
        if (jn[c] == c) pending = c;
        jn[c] += 1;
      }
    if (!sp_grid_sync(grid, bar++, ready, part, nparts, totals)) return -1;
  }
  return 0;
}

// Rounds round_begin..round_end-1 of the subspace iteration over the two blocks buf0 / buf1 (n x B
// column-major): round r multiplies buf[r % 2] into buf[(r + 1) % 2] and orthonormalises the
// result (round -1: orthonormalise buf0 only); buf[r % 2] then holds the post-multiply copy. The
// first round starts at column first_from and multiplies only when first_multiply is set. A
// column whose norm vanishes stops every block at the same step (they all read the same norm);
// block 0 records round and column in grid->status for the host's redraw.
__global__ void __launch_bounds__(kSpThreads, 3)
sp_rounds_kernel(const int* __restrict__ offsets, const int* __restrict__ nbr, const float* __restrict__ nw,
                 const double* __restrict__ triv, int n, int B, int nparts, double* buf0, double* buf1, double* part,
                 double* totals, int round_begin, int round_end, int first_from, int first_multiply, SpGrid* grid) {
  unsigned bar = 0;
  for (int r = round_begin; r < round_end; ++r) {
    double* m = ((r + 1) & 1) ? buf1 : buf0;
    double* other = (r & 1) ? buf1 : buf0;
    const bool first = r == round_begin;
    if (!first || first_multiply) {
      sp_multiply_rows(offsets, nbr, nw, n, B, other, m);
      if (!sp_grid_sync(grid, bar++, 0u, part, nparts, totals)) return;
    }
    const int st = sp_orthonormalise(m, other, triv, n, B, first ? first_from : 0, nparts, part, totals, grid, bar);
    if (st > 0) {
      if (blockIdx.x == 0 && threadIdx.x == 0) grid->status = 16 * (r + 1) + (st - 1);
      return;
    }
    if (st < 0) return;
  }
}

// Block partials of q[:, a] . z[:, b] for a <= b (pair index in row-major upper-triangle order).
__global__ void __launch_bounds__(kSpThreads)
sp_project_kernel(const double* __restrict__ q, const double* __restrict__ z, int n, int B,
                  double* __restrict__ part) {
  __shared__ double s_w[kSpThreads / 32][kSpPairs];
  double acc[kSpPairs];
#pragma unroll
  for (int t = 0; t < kSpPairs; ++t) acc[t] = 0.0;
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
    int t = 0;
#pragma unroll
    for (int a = 0; a < kSpBlock; ++a) {
      const double qv = a < B ? q[(long long)a * n + r] : 0.0;
#pragma unroll
      for (int b = a; b < kSpBlock; ++b, ++t)
        if (b < B) acc[t] = __dadd_rn(acc[t], __dmul_rn(qv, z[(long long)b * n + r]));
    }
  }
#pragma unroll
  for (int t = 0; t < kSpPairs; ++t) {
    const double v = warp_sum(acc[t]);
    if ((threadIdx.x & 31) == 0) s_w[threadIdx.x >> 5][t] = v;
  }
  __syncthreads();
  if ((int)threadIdx.x < kSpPairs) {
    double s = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s = __dadd_rn(s, s_w[w][threadIdx.x]);
    part[(long long)blockIdx.x * kSpPairs + threadIdx.x] = s;
  }
}

// One thread: the projected matrix from the partials, the reference's Jacobi rotations (at most
// 80, each on the largest off-diagonal entry), Ritz values sorted descending; coef[c * 8 + b]
// = component c's coefficients on the basis.
__global__ void sp_ritz_kernel(const double* __restrict__ part, int nparts, int B, double* __restrict__ coef) {
  __shared__ double s_pair[kSpPairs];
  if (blockIdx.x != 0) return;
  if ((int)threadIdx.x < kSpPairs) {
    // entry t of the upper triangle: its block partials in block order, loads issued ahead
    const int t = threadIdx.x;
    double s = 0.0;
    int k = 0;
    for (; k + 7 < nparts; k += 8) {
      double v[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) v[u] = part[(long long)(k + u) * kSpPairs + t];
#pragma unroll
      for (int u = 0; u < 8; ++u) s = __dadd_rn(s, v[u]);
    }
    for (; k < nparts; ++k) s = __dadd_rn(s, part[(long long)k * kSpPairs + t]);
    s_pair[t] = s;
  }
  __syncthreads();
  if (threadIdx.x != 0) return;
  double P[kSpBlock][kSpBlock], V[kSpBlock][kSpBlock];
  int t = 0;
  for (int a = 0; a < kSpBlock; ++a)
    for (int b = a; b < kSpBlock; ++b, ++t) {
      P[a][b] = s_pair[t];
      P[b][a] = s_pair[t];
    }
  for (int i = 0; i < kSpBlock; ++i)
    for (int j = 0; j < kSpBlock; ++j) V[i][j] = i == j ? 1.0 : 0.0;
  for (int sweep = 0; sweep < 80; ++sweep) {
    int p = 0, q = 1;
    double mx = 0.0;
    for (int i = 0; i < B; ++i)
      for (int j = i + 1; j < B; ++j) {
        const double v = fabs(P[i][j]);
        if (v > mx) {
          mx = v;
          p = i;
          q = j;
        }
      }
    if (mx < 1e-10) break;
    const double app = P[p][p], aqq = P[q][q], apq = P[p][q];
    const double tau = __ddiv_rn(__dsub_rn(aqq, app), __dmul_rn(2.0, apq));
    const double tt = __ddiv_rn(tau >= 0.0 ? 1.0 : -1.0,
                                __dadd_rn(fabs(tau), __dsqrt_rn(__dadd_rn(1.0, __dmul_rn(tau, tau)))));
    const double cs = __ddiv_rn(1.0, __dsqrt_rn(__dadd_rn(1.0, __dmul_rn(tt, tt))));
    const double sn = __dmul_rn(tt, cs);
    for (int k = 0; k < B; ++k) {
      if (k == p || k == q) continue;
      const double akp = P[k][p], akq = P[k][q];
      P[k][p] = __dsub_rn(__dmul_rn(cs, akp), __dmul_rn(sn, akq));
      P[p][k] = P[k][p];
      P[k][q] = __dadd_rn(__dmul_rn(sn, akp), __dmul_rn(cs, akq));
      P[q][k] = P[k][q];
    }
    const double cc = __dmul_rn(cs, cs), ss = __dmul_rn(sn, sn);
    const double cross = __dmul_rn(__dmul_rn(__dmul_rn(2.0, sn), cs), apq);
    P[p][p] = __dadd_rn(__dsub_rn(__dmul_rn(cc, app), cross), __dmul_rn(ss, aqq));
    P[q][q] = __dadd_rn(__dadd_rn(__dmul_rn(ss, app), cross), __dmul_rn(cc, aqq));
    P[p][q] = 0.0;
    P[q][p] = 0.0;
    for (int k = 0; k < B; ++k) {
      const double vp = V[k][p], vq = V[k][q];
      V[k][p] = __dsub_rn(__dmul_rn(cs, vp), __dmul_rn(sn, vq));
      V[k][q] = __dadd_rn(__dmul_rn(sn, vp), __dmul_rn(cs, vq));
    }
  }
  int order[kSpBlock];
  for (int i = 0; i < B; ++i) {
    int j = i;
    while (j > 0 && P[i][i] > P[order[j - 1]][order[j - 1]]) {
      order[j] = order[j - 1];
      --j;
    }
    order[j] = i;
  }
  for (int c = 0; c < 2; ++c)
    for (int b = 0; b < kSpBlock; ++b) coef[c * kSpBlock + b] = b < B ? V[b][order[c]] : 0.0;
}

// emb[:, c] = q coef_c (basis order), with block partials of each column's sum.
__global__ void __launch_bounds__(kSpThreads)
sp_embed_kernel(const double* __restrict__ q, const double* __restrict__ coef, int n, int B,
                double* __restrict__ emb, double* __restrict__ part) {
  double acc0 = 0.0, acc1 = 0.0;
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
    double v0 = 0.0, v1 = 0.0;
    for (int b = 0; b < B; ++b) {
      const double x = q[(long long)b * n + r];
      v0 = __dadd_rn(v0, __dmul_rn(x, coef[b]));
      v1 = __dadd_rn(v1, __dmul_rn(x, coef[kSpBlock + b]));
    }
    emb[r] = v0;
    emb[(long long)n + r] = v1;
    acc0 = __dadd_rn(acc0, v0);
    acc1 = __dadd_rn(acc1, v1);
  }
  block_partial(acc0, part);
  __syncthreads();
  block_partial(acc1, part + gridDim.x);
}

// emb[:, c] -= mean_c (sums in part[c * nparts ...]); block maxima of |emb| into pmax.
__global__ void __launch_bounds__(kSpThreads)
sp_centre_kernel(double* __restrict__ emb, int n, const double* __restrict__ part, int nparts,
                 double* __restrict__ pmax) {
  __shared__ double s_w[kSpThreads / 32];
  const double m0 = __ddiv_rn(sum_partials(part, nparts), (double)n);
  const double m1 = __ddiv_rn(sum_partials(part + nparts, nparts), (double)n);
  double mx = 0.0;
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
    const double a = __dsub_rn(emb[r], m0), b = __dsub_rn(emb[(long long)n + r], m1);
    emb[r] = a;
    emb[(long long)n + r] = b;
    if (isfinite(a)) mx = fmax(mx, fabs(a));
    if (isfinite(b)) mx = fmax(mx, fabs(b));
  }
  mx = warp_max(mx);
  if ((threadIdx.x & 31) == 0) s_w[threadIdx.x >> 5] = mx;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t = fmax(t, s_w[w]);
    pmax[blockIdx.x] = t;
  }
}

// emb = emb * (10 / max|emb|) + jitter, unless the maximum is zero or not finite.
__global__ void sp_expand_kernel(double* __restrict__ emb, int n, const double* __restrict__ pmax, int nparts,
                                 const double* __restrict__ jitter) {
  __shared__ double s_mx;
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int b = 0; b < nparts; ++b) t = fmax(t, pmax[b]);
    s_mx = t;
  }
  __syncthreads();
  const double mx = s_mx;
  if (!isfinite(mx) || mx <= 0.0) return;
  const double ex = __ddiv_rn(10.0, mx);
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < 2LL * n;
       t += (long long)gridDim.x * blockDim.x)
    emb[t] = __dadd_rn(__dmul_rn(emb[t], ex), jitter[t]);
}

// scale_embedding_sdev: column c -> (x - mean) * (target / sd), sd over n - 1.
__global__ void __launch_bounds__(kSpThreads)
sp_column_sum_kernel(const double* __restrict__ col, int n, const double* __restrict__ mean_part, int nparts,
                     double* __restrict__ part) {
  const double mean = mean_part ? __ddiv_rn(sum_partials(mean_part, nparts), (double)n) : 0.0;
  double acc = 0.0;
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
    if (mean_part) {
      const double d = __dsub_rn(col[r], mean);
      acc = __dadd_rn(acc, __dmul_rn(d, d));
    } else {
      acc = __dadd_rn(acc, col[r]);
    }
  }
  block_partial(acc, part);
}

__global__ void sp_rescale_kernel(double* __restrict__ col, int n, const double* __restrict__ mean_part,
                                  const double* __restrict__ ss_part, int nparts, double target) {
  const double mean = __ddiv_rn(sum_partials(mean_part, nparts), (double)n);
  const double sd = __dsqrt_rn(__ddiv_rn(sum_partials(ss_part, nparts), (double)(n - 1)));
  if (!isfinite(sd) || sd <= 0.0) return;
  const double sc = __ddiv_rn(target, sd);
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x)
    col[r] = __dmul_rn(__dsub_rn(col[r], mean), sc);
}

}  // namespace

SpectralDraws spectral_draws(int n, int seed) {
  SpectralDraws d;
  d.rng.seed((std::uint32_t)seed);
  const int B = std::min(n - 1, kSpBlock);
  if (B < 2) return d;
  d.block.resize((std::size_t)n * B);
  d.normal.fill(d.rng, d.block.data(), d.block.size(), 10000.0);
  d.jitter = std::async(std::launch::async, [ahead = d.rng, n]() mutable {
               NormalStream jitter(0.0, 1e-4);
               std::vector<double> v(2 * (std::size_t)n);
               jitter.fill(ahead, v.data(), v.size(), 1.0);
               return v;
             }).share();
  return d;
}

void umap_spectral_start(const int* offsets, const int* neighbors, const float* weights, int n, long long nnz,
                         int spectral_n_iter, double init_scale, int seed, double* out, cudaStream_t s,
                         SpectralDraws* pre) {
  if (n < 1 || spectral_n_iter < 1) throw Error("invalid spectral initialization parameters");
  std::mt19937 rng((std::uint32_t)seed);
  std::uniform_real_distribution<double> uniform(-10.0, 10.0);
  const int B = std::min(n - 1, kSpBlock);
  const int nb = sp_blocks(n);
  const int gb = std::max(1, std::min(ceil_div(n, kSpThreads), sm_count() * 8));
  const int gw = std::max(1, std::min(ceil_div(n, kSpThreads / 32), sm_count() * 8));  // warp per row
  const int gm = std::max(1, std::min(ceil_div(n, kSpThreads / 8), sm_count() * 8));   // 8 lanes per row
  std::vector<double> host;
  if (nnz < 1 || B < 2) {
    // the reference's fallback: uniform(-10, 10) coordinates, column after column
    host.resize(2 * (std::size_t)n);
    for (double& v : host) v = uniform(rng);
    FE_CUDA(cudaMemcpyAsync(out, host.data(), sizeof(double) * host.size(), cudaMemcpyHostToDevice, s));
  } else {
    float *deg = nullptr, *nw = nullptr;
    double *triv = nullptr, *q = nullptr, *z = nullptr, *pa = nullptr, *pb = nullptr, *pc = nullptr;
    double *coef = nullptr, *jit = nullptr;
    SpGrid* grid = nullptr;
    double* totals = nullptr;
    Arena w;
    w.reserve(&deg, n);
    w.reserve(&nw, (std::size_t)nnz);
    w.reserve(&triv, n);
    w.reserve(&q, (std::size_t)n * B);
    w.reserve(&z, (std::size_t)n * B);
    w.reserve(&pa, kSpMaxBlocks * kSpPairs);
    w.reserve(&pb, kSpMaxBlocks * 2);
    w.reserve(&pc, kSpMaxBlocks * 2);
    w.reserve(&coef, 2 * kSpBlock);
    w.reserve(&jit, 2 * (std::size_t)n);
    w.reserve(&grid, 1);
    w.reserve(&totals, kSpBlock);
    w.commit("UMAP spectral start");
    sp_degree_kernel<<<gb, kSpThreads, 0, s>>>(offsets, weights, n, deg);
    FE_LAUNCH("sp_degree_kernel");
    sp_adjacency_kernel<<<gw, kSpThreads, 0, s>>>(offsets, neighbors, weights, deg, n, nw);
    FE_LAUNCH("sp_adjacency_kernel");
    sp_trivial_kernel<<<nb, kSpThreads, 0, s>>>(deg, n, triv, pa);
    FE_LAUNCH("sp_trivial_kernel");
    sp_normalise_trivial_kernel<<<gb, kSpThreads, 0, s>>>(triv, n, pa, nb);
    FE_LAUNCH("sp_normalise_trivial_kernel");
    SpGrid g0{0u, 0u, 0, -1};
    FE_CUDA(cudaMemcpyAsync(grid, &g0, sizeof(SpGrid), cudaMemcpyHostToDevice, s));
    SpectralDraws local;
    SpectralDraws* dr = pre;
    if (!dr || dr->block.size() != (std::size_t)n * B) {
      local = spectral_draws(n, seed);
      dr = &local;
    }
    bool redrawn = false;

    // The subspace iteration as cooperative launches of every resident block (at most one per
    // partial slot): the initial orthonormalisation (round -1) and spectral_n_iter rounds. A
    // launch that stops at a vanished column is resumed from it after the host redraws the
    // column from the stream, as the reference redraws and repeats it.
    int per_sm = 0;
    FE_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, sp_rounds_kernel, kSpThreads, 0));
    const int G = std::min(nb, per_sm * sm_count());
    if (G < 1) throw Error("the spectral start's subspace iteration cannot be made resident");
    int dev = 0, coop = 0;
    FE_CUDA(cudaGetDevice(&dev));
    FE_CUDA(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev));
    if (!coop) throw Error("the device does not support cooperative launches");
    FE_CUDA(cudaMemcpyAsync(q, dr->block.data(), sizeof(double) * dr->block.size(), cudaMemcpyHostToDevice, s));
    int r0 = -1, from = 0, mult = 0;
    for (;;) {
      int nparts = nb, r_end = spectral_n_iter;
      void* args[] = {(void*)&offsets, (void*)&neighbors, (void*)&nw, (void*)&triv, (void*)&n, (void*)&B,
                      (void*)&nparts, (void*)&q, (void*)&z, (void*)&pa, (void*)&totals, (void*)&r0, (void*)&r_end,
                      (void*)&from, (void*)&mult, (void*)&grid};
      FE_CUDA(cudaLaunchCooperativeKernel((const void*)sp_rounds_kernel, dim3(G), dim3(kSpThreads), args, 0, s));
      FE_LAUNCH("sp_rounds_kernel");
      SpGrid g1;
      FE_CUDA(cudaMemcpyAsync(&g1, grid, sizeof(SpGrid), cudaMemcpyDeviceToHost, s));
      FE_CUDA(cudaStreamSynchronize(s));
      if (g1.error) throw Error("spectral start: a grid barrier of the subspace iteration timed out");
      if (g1.status < 0) break;
      const int rr = g1.status / 16 - 1, f = g1.status % 16;
      if (rr < -1 || rr >= spectral_n_iter || f < 0 || f >= B) throw Error("spectral start: invalid redraw status");
      redrawn = true;
      host.resize(n);
      dr->normal.fill(dr->rng, host.data(), host.size(), 10000.0);
      // the later columns back to their post-multiply values (the pass had started on them), then
      // the redrawn column
      double* m = ((rr + 1) & 1) ? z : q;
      const double* bk = (rr & 1) ? z : q;
      if (f + 1 < B)
        FE_CUDA(cudaMemcpyAsync(m + (std::size_t)(f + 1) * n, bk + (std::size_t)(f + 1) * n,
                                sizeof(double) * (std::size_t)(B - f - 1) * n, cudaMemcpyDeviceToDevice, s));
      FE_CUDA(cudaMemcpyAsync(m + (std::size_t)f * n, host.data(), sizeof(double) * n, cudaMemcpyHostToDevice, s));
      FE_CUDA(cudaMemcpyAsync(grid, &g0, sizeof(SpGrid), cudaMemcpyHostToDevice, s));
      r0 = rr;
      from = f;
      mult = 0;
    }
    // after round r the block is in buf[(r + 1) % 2]: the last round leaves it in buf[n_iter % 2]
    if (spectral_n_iter & 1) std::swap(q, z);
    sp_multiply_kernel<<<gm, kSpThreads, 0, s>>>(offsets, neighbors, nw, n, B, q, z);
    FE_LAUNCH("sp_multiply_kernel");
    sp_project_kernel<<<nb, kSpThreads, 0, s>>>(q, z, n, B, pa);
    FE_LAUNCH("sp_project_kernel");
    sp_ritz_kernel<<<1, 64, 0, s>>>(pa, nb, B, coef);
    FE_LAUNCH("sp_ritz_kernel");
    sp_embed_kernel<<<nb, kSpThreads, 0, s>>>(q, coef, n, B, out, pb);
    FE_LAUNCH("sp_embed_kernel");
    sp_centre_kernel<<<nb, kSpThreads, 0, s>>>(out, n, pb, nb, pc);
    FE_LAUNCH("sp_centre_kernel");
    // jitter: a fresh normal(0, 1e-4) distribution on the same stream, column after column (drawn
    // ahead unless a redraw moved the stream on)
    std::vector<double> fresh;
    if (redrawn) {
      NormalStream jitter(0.0, 1e-4);
      fresh.resize(2 * (std::size_t)n);
      jitter.fill(dr->rng, fresh.data(), fresh.size(), 1.0);
    }
    const std::vector<double>& jv = redrawn ? fresh : dr->jitter.get();
    FE_CUDA(cudaMemcpyAsync(jit, jv.data(), sizeof(double) * jv.size(), cudaMemcpyHostToDevice, s));
    sp_expand_kernel<<<gb, kSpThreads, 0, s>>>(out, n, pc, nb, jit);
    FE_LAUNCH("sp_expand_kernel");
    FE_CUDA(cudaStreamSynchronize(s));
  }
  if (std::isfinite(init_scale) && init_scale > 0.0 && n >= 2) {
    double *pm = nullptr, *ps = nullptr;
    Arena w;
    w.reserve(&pm, kSpMaxBlocks);
    w.reserve(&ps, kSpMaxBlocks);
    w.commit("UMAP start rescale");
    for (int c = 0; c < 2; ++c) {
      double* col = out + (std::size_t)c * n;
      sp_column_sum_kernel<<<nb, kSpThreads, 0, s>>>(col, n, nullptr, nb, pm);
      FE_LAUNCH("sp_column_sum_kernel");
      sp_column_sum_kernel<<<nb, kSpThreads, 0, s>>>(col, n, pm, nb, ps);
      FE_LAUNCH("sp_column_sum_kernel");
      sp_rescale_kernel<<<gb, kSpThreads, 0, s>>>(col, n, pm, ps, nb, init_scale);
      FE_LAUNCH("sp_rescale_kernel");
    }
    FE_CUDA(cudaStreamSynchronize(s));
  }
}

}  // namespace fe
