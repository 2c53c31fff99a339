// Per-iteration kernels of the t-SNE gradient loop on the GPU.
//
// Reference algorithm (fastEmbedR src/tsne_neighbors.cpp:1152-1260 on the CPU,
// src/embedding_cuda_kernels.cpp:2472-2886 on CUDA): bound the layout by a square,
// interpolate charges {1, x, y} onto a uniform grid, convolve with the kernels
// q = 1/(1 + d^2) and q^2 by FFT on the zero-padded 2G x 2G torus, interpolate the potentials
// back, combine with the sparse attractive term and apply the gains/momentum update.
//
// GB300 layout of one iteration (6 launches, two streams, captured in a CUDA graph):
//   side stream:  attractive_kernel        warp-per-row CSR attractive force, rows in storage
//                                          (spatial) order (stream of P + L1/L2 gathers of y)
//   main stream:  scatter_kernel           points -> 64-bit fixed-point charges (deterministic)
//                 rows_forward_kernel      row FFTs of the charges (x + i y plane, paired mass
//                                          rows as half spectra) and of the kernel rows; the top
//                                          stages run in registers on the values as loaded
//                 columns_convolve_kernel  column FFTs per conjugate column pair, Z by Parseval,
//                                          multiply, inverse column FFTs in shared memory; the
//                                          passes next to global memory and to the product run
//                                          in registers
//                 rows_inverse_kernel      inverse row FFTs -> float4 potentials, Z finalised
//   join:         update_kernel            potential gather + gains/momentum/step clip +
//                                          recentring; epilogue reduces the new bounding box and
//                                          mean into the next iteration's grid
// The attractive pass (load-latency-bound) runs beside the grid stage (shared-memory bound).
// Interpolation: the reference bilinear splat on G shared nodes (default), or 3 equispaced
// Lagrange nodes per box over floor(G / 3) boxes, as in FIt-SNE-style interpolation.
#include <cfloat>
#include <climits>
#include <cmath>
#include <algorithm>
#include <vector>

#include "tsne_grid.cuh"

namespace fe {

constexpr int kStepThreads = 256;
constexpr int kFftThreads = 256;
constexpr int kColThreads = 256;  // the column pass holds 4 x M complex values of shared memory
                                  // (70 KB at M = 2048: 3 blocks per SM)

// ---------------------------------------------------------------- stencils
template <int TAPS>
struct Stencil {
  int base;
  float w[TAPS];
};

// Bilinear (TAPS = 2): bilinear_grid_value_t / the scatter of src/tsne_neighbors.cpp:1194-1213.
// Lagrange (TAPS = 3): nodes at x0 + (3b + j + 0.5) h, j = 0..2, of box b.
template <int TAPS>
__device__ __forceinline__ Stencil<TAPS> make_stencil(float x, float x0, float inv_h, float inv_box, int nodes) {
  Stencil<TAPS> s;
  if constexpr (TAPS == 2) {
    const float raw = (x - x0) * inv_h;
    const float c = fmaxf(0.0f, fminf((float)(nodes - 1), raw));
    int u0 = (int)floorf(c);
    u0 = max(0, min(nodes - 2, u0));
    const float f = c - (float)u0;
    s.base = u0;
    s.w[0] = 1.0f - f;
    s.w[1] = f;
  } else {
    const int nbox = nodes / 3;
    int b = (int)floorf((x - x0) * inv_box);
    b = max(0, min(nbox - 1, b));
    const float t = (x - x0) * inv_h - (float)(3 * b) - 0.5f;
    s.base = 3 * b;
    s.w[0] = 0.5f * (t - 1.0f) * (t - 2.0f);
    s.w[1] = t * (2.0f - t);
    s.w[2] = 0.5f * t * (t - 1.0f);
  }
  return s;
}

// ---------------------------------------------------------------- layout statistics
// Fixed-order reduction of the per-block partials into the grid of the next iteration
// (the bounding-square rule of src/tsne_neighbors.cpp:1168-1184).
__device__ void finish_layout_stats(const StepPartial* __restrict__ part, int nblocks, int n, int grid, int mode,
                                    GridState* __restrict__ next) {
  __shared__ float s_min_x[kStepThreads], s_max_x[kStepThreads], s_min_y[kStepThreads], s_max_y[kStepThreads];
  __shared__ double s_sx[kStepThreads], s_sy[kStepThreads];
  float mnx = FLT_MAX, mxx = -FLT_MAX, mny = FLT_MAX, mxy = -FLT_MAX;
  double sx = 0.0, sy = 0.0;
  // partials written by the other blocks of this launch: read through L2, eight loads in flight
#pragma unroll 8
  for (int b = threadIdx.x; b < nblocks; b += blockDim.x) {
    const float4 mm = __ldcg(reinterpret_cast<const float4*>(part + b));
    const double2 ss = __ldcg(reinterpret_cast<const double2*>(part + b) + 1);
    mnx = fminf(mnx, mm.x);
    mxx = fmaxf(mxx, mm.y);
    mny = fminf(mny, mm.z);
    mxy = fmaxf(mxy, mm.w);
    sx += ss.x;
    sy += ss.y;
  }
  s_min_x[threadIdx.x] = mnx;
  s_max_x[threadIdx.x] = mxx;
  s_min_y[threadIdx.x] = mny;
  s_max_y[threadIdx.x] = mxy;
  s_sx[threadIdx.x] = sx;
  s_sy[threadIdx.x] = sy;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) {
      s_min_x[threadIdx.x] = fminf(s_min_x[threadIdx.x], s_min_x[threadIdx.x + w]);
      s_max_x[threadIdx.x] = fmaxf(s_max_x[threadIdx.x], s_max_x[threadIdx.x + w]);
      s_min_y[threadIdx.x] = fminf(s_min_y[threadIdx.x], s_min_y[threadIdx.x + w]);
      s_max_y[threadIdx.x] = fmaxf(s_max_y[threadIdx.x], s_max_y[threadIdx.x + w]);
      s_sx[threadIdx.x] += s_sx[threadIdx.x + w];
      s_sy[threadIdx.x] += s_sy[threadIdx.x + w];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    const float min_x = s_min_x[0], max_x = s_max_x[0], min_y = s_min_y[0], max_y = s_max_y[0];
    GridState g;
    g.cx = 0.5f * (min_x + max_x);
    g.cy = 0.5f * (min_y + max_y);
    float span = fmaxf(max_x - min_x, max_y - min_y);
    if (!isfinite(span) || span <= 0.0f) span = 1.0f;
    const float half = 0.55f * span + 1.0e-3f;
    g.x0 = g.cx - half;
    g.y0 = g.cy - half;
    if (mode == kInterpBilinear) {
      g.nodes = grid;
      g.h = (2.0f * half) / (float)(grid - 1);
      g.box = g.h;
    } else {
      const int nbox = grid / 3;
      g.nodes = 3 * nbox;
      g.box = (2.0f * half) / (float)nbox;
      g.h = g.box / 3.0f;
    }
    g.inv_h = 1.0f / g.h;
    g.inv_box = 1.0f / g.box;
    g.mean_x = s_sx[0] / (double)n;
    g.mean_y = s_sy[0] / (double)n;
    g.z = 0.0;
    g.inv_z = 0.0f;
    // |mass| and |mass * d| summed over any subset of points stay below 1.5625 n max(half, 1)
    // (stencil weights sum to 1 in absolute value for bilinear, 1.5625 for Lagrange; |d| <= half):
    // scale so that bound stays below 2^62.
    float bound = 2.0f * (float)n * fmaxf(half, 1.0f);
    if (!(bound < 1.0e30f)) bound = 1.0e30f;
    int e = 0;
    frexpf(bound, &e);  // bound < 2^e
    g.qscale = ldexpf(1.0f, 62 - e);
    g.inv_qscale = ldexpf(1.0f, e - 62);
    // the same bound over the points of one block (at most kPointBlock), below 2^30
    float tbound = 2.0f * (float)min(n, kPointBlock) * fmaxf(half, 1.0f);
    if (!(tbound < 1.0e30f)) tbound = 1.0e30f;
    int et = 0;
    frexpf(tbound, &et);
    g.tile_shift = (62 - e) - (30 - et);  // >= 0: et <= e
    g.tscale = ldexpf(1.0f, 30 - et);
    *next = g;
  }
}

__device__ __forceinline__ void block_partial(float mnx, float mxx, float mny, float mxy, double sx, double sy,
                                              StepPartial* out) {
  __shared__ StepPartial s_part[kStepThreads / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  mnx = warp_min(mnx);
  mxx = warp_max(mxx);
  mny = warp_min(mny);
  mxy = warp_max(mxy);
  sx = warp_sum(sx);
  sy = warp_sum(sy);
  if (lane == 0) s_part[warp] = StepPartial{mnx, mxx, mny, mxy, sx, sy};
  __syncthreads();
  if (threadIdx.x == 0) {
    StepPartial p = s_part[0];
    for (int w = 1; w < (int)(blockDim.x / 32); ++w) {
      p.min_x = fminf(p.min_x, s_part[w].min_x);
      p.max_x = fmaxf(p.max_x, s_part[w].max_x);
      p.min_y = fminf(p.min_y, s_part[w].min_y);
      p.max_y = fmaxf(p.max_y, s_part[w].max_y);
      p.sum_x += s_part[w].sum_x;
      p.sum_y += s_part[w].sum_y;
    }
    *out = p;
  }
}

// Returns true in exactly one of the `blocks` blocks sharing `counter`: the last one to finish
// (counter reset for reuse).
__device__ __forceinline__ bool last_block_done(unsigned* counter, int blocks) {
  __shared__ bool s_last;
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) {
    const unsigned prev = atomicAdd(counter, 1u);
    s_last = prev == (unsigned)blocks - 1u;
    if (s_last) *counter = 0u;
  }
  __syncthreads();
  if (s_last) __threadfence();
  return s_last;
}

// Initial statistics of ynew (setup, and after an external layout write). One point per thread;
// each instance's last block finishes that instance's grid.
__global__ void __launch_bounds__(kStepThreads)
layout_stats_kernel(const float2* __restrict__ ynew, const TsneInstance* __restrict__ inst,
                    const int2* __restrict__ blocks, int mode, StepPartial* __restrict__ part,
                    unsigned* __restrict__ counter, GridState* __restrict__ next) {
  const int2 bl = blocks[blockIdx.x];
  const TsneInstance I = inst[bl.x];
  const int i = bl.y + threadIdx.x;
  float mnx = FLT_MAX, mxx = -FLT_MAX, mny = FLT_MAX, mxy = -FLT_MAX;
  double sx = 0.0, sy = 0.0;
  if (i < I.pt_begin + I.n) {
    const float2 p = ynew[i];
    mnx = mxx = p.x;
    mny = mxy = p.y;
    sx = p.x;
    sy = p.y;
  }
  block_partial(mnx, mxx, mny, mxy, sx, sy, part + blockIdx.x);
  if (last_block_done(counter + bl.x, I.blocks))
    finish_layout_stats(part + I.block_begin, I.blocks, I.n, I.grid, mode, next + bl.x);
}

// ---------------------------------------------------------------- scatter
// Each point adds (w, w*(x - cx), w*(y - cy)) to its TAPS x TAPS stencil nodes of its instance's
// grid; the first block of every instance also promotes the grid computed by the previous update
// (`next`) to `cur`.
// Points are stored in spatial (Morton) order and every block takes 256 consecutive points of one
// instance, so a block covers a compact patch of the grid even when clusters collapse onto a few
// cells:
//   1. runs of equal stencil anchors inside a warp are summed by a segmented shuffle reduction
//      (a fixed tree: the same inputs give the same float sums);
//   2. run heads accumulate into a kTile x kTile node tile in shared memory anchored at the block's
//      lowest anchor, in 32-bit fixed point (the run sums rounded to a multiple of 1 / tscale,
//      about 2^-30 of the largest sum a block can make; native 32-bit shared atomics); heads
//      outside the tile add to the grid directly in 64-bit fixed point (x qscale);
//   3. the tile is flushed with one 64-bit integer atomic per touched node and value, the tile sum
//      shifted up to the grid's scale (exact: both scales are powers of two).
// Integer sums do not depend on the order in which atomics arrive, so the charges (and the
// whole iteration) are deterministic.
constexpr int kScatterTile = 32;

__device__ __forceinline__ void red_add_i64(long long* p, long long v) {
  atomicAdd(reinterpret_cast<unsigned long long*>(p), static_cast<unsigned long long>(v));
}

template <int TAPS>
__global__ void __launch_bounds__(256)
scatter_kernel(const float2* __restrict__ y, const TsneInstance* __restrict__ inst, const int2* __restrict__ blocks,
               GridState* __restrict__ cur, const GridState* __restrict__ next) {
  constexpr int NV = TAPS * TAPS * 3;
  __shared__ int tile[kScatterTile * kScatterTile * 3];
  __shared__ int s_box[4];
  const int2 bl = blocks[blockIdx.x];
  const TsneInstance I = inst[bl.x];
  const int grid = I.grid;
  long long* __restrict__ charges = I.charges;
  const GridState g = next[bl.x];
  if (bl.y == I.pt_begin && threadIdx.x == 0) cur[bl.x] = g;
  const int lane = threadIdx.x & 31;
  for (int t = threadIdx.x; t < kScatterTile * kScatterTile * 3; t += blockDim.x) tile[t] = 0;
  if (threadIdx.x == 0) {
    s_box[0] = INT_MAX;
    s_box[1] = INT_MAX;
    s_box[2] = -1;
    s_box[3] = -1;
  }
  const int i = bl.y + threadIdx.x;
  const bool valid = i < I.pt_begin + I.n;
  const float2 p = valid ? y[i] : make_float2(g.cx, g.cy);
  const Stencil<TAPS> sx = make_stencil<TAPS>(p.x, g.x0, g.inv_h, g.inv_box, g.nodes);
  const Stencil<TAPS> sy = make_stencil<TAPS>(p.y, g.y0, g.inv_h, g.inv_box, g.nodes);
  const float dx = p.x - g.cx, dy = p.y - g.cy;
  float v[NV];
#pragma unroll
  for (int a = 0; a < TAPS; ++a)
#pragma unroll
    for (int b = 0; b < TAPS; ++b) {
      const float w = valid ? sy.w[a] * sx.w[b] : 0.0f;
      v[(a * TAPS + b) * 3 + 0] = w;
      v[(a * TAPS + b) * 3 + 1] = w * dx;
      v[(a * TAPS + b) * 3 + 2] = w * dy;
    }
  const int key = valid ? sy.base * grid + sx.base : -1 - lane;
  const int prev = __shfl_up_sync(0xffffffffu, key, 1);
  const unsigned heads = __ballot_sync(0xffffffffu, lane == 0 || prev != key);
  if (heads != 0xffffffffu) {
    // suffix sums restricted to contiguous runs [lane, next head)
    const unsigned above = heads & ~((2u << lane) - 1u);
    const int run_end = above ? __ffs(above) - 1 : 32;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
      const bool take = lane + off < run_end;
#pragma unroll
      for (int c = 0; c < NV; ++c) {
        const float o = __shfl_down_sync(0xffffffffu, v[c], off);
        if (take) v[c] += o;
      }
    }
  }
  const bool head = valid && ((heads >> lane) & 1u);
  __syncthreads();
  if (head) {
    atomicMin(&s_box[0], sx.base);
    atomicMin(&s_box[1], sy.base);
    atomicMax(&s_box[2], sx.base);
    atomicMax(&s_box[3], sy.base);
  }
  __syncthreads();
  const int ox = s_box[0], oy = s_box[1];
  if (head) {
    const int tx = sx.base - ox, ty = sy.base - oy;
    if (tx + TAPS <= kScatterTile && ty + TAPS <= kScatterTile) {
#pragma unroll
      for (int a = 0; a < TAPS; ++a)
#pragma unroll
        for (int b = 0; b < TAPS; ++b) {
          int* t = tile + ((ty + a) * kScatterTile + tx + b) * 3;
          const int c = (a * TAPS + b) * 3;
          atomicAdd(t, __float2int_rn(v[c] * g.tscale));
          atomicAdd(t + 1, __float2int_rn(v[c + 1] * g.tscale));
          atomicAdd(t + 2, __float2int_rn(v[c + 2] * g.tscale));
        }
    } else {
#pragma unroll
      for (int a = 0; a < TAPS; ++a) {
        long long* row = charges + ((long long)(sy.base + a) * grid + sx.base) * kChargeStride;
#pragma unroll
        for (int b = 0; b < TAPS; ++b) {
          const int c = (a * TAPS + b) * 3;
          red_add_i64(row + b * kChargeStride, __float2ll_rn(v[c] * g.qscale));
          red_add_i64(row + b * kChargeStride + 1, __float2ll_rn(v[c + 1] * g.qscale));
          red_add_i64(row + b * kChargeStride + 2, __float2ll_rn(v[c + 2] * g.qscale));
        }
      }
    }
  }
  __syncthreads();
  if (s_box[2] < 0) return;  // no valid point in this block
  const int wu = min(kScatterTile, s_box[2] - ox + TAPS);
  const int hu = min(kScatterTile, s_box[3] - oy + TAPS);
  for (int t = threadIdx.x; t < wu * hu; t += blockDim.x) {
    const int r = t / wu, c = t - r * wu;
    const int* src = tile + (r * kScatterTile + c) * 3;
    const int a0 = src[0], a1 = src[1], a2 = src[2];
    if (a0 != 0 || a1 != 0 || a2 != 0) {
      long long* dst = charges + ((long long)(oy + r) * grid + ox + c) * kChargeStride;
      const int sh = g.tile_shift;
      red_add_i64(dst, (long long)((unsigned long long)(long long)a0 << sh));
      red_add_i64(dst + 1, (long long)((unsigned long long)(long long)a1 << sh));
      red_add_i64(dst + 2, (long long)((unsigned long long)(long long)a2 << sh));
    }
  }
}

// ---------------------------------------------------------------- shared-memory FFT
__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
// Shared-memory index with one pad slot after every 16 complex values: the radix-2^4 passes with
// small butterfly strides (1, 16) touch elements 16 or 256 apart from consecutive threads, which
// would otherwise land on the same banks (with this padding every pass of M = 512 .. 2048 is
// free of bank conflicts for 64-bit accesses).
__device__ __forceinline__ int sidx(int i) { return i + (i >> 4); }
__host__ __device__ constexpr int padded(int count) { return count + count / 16; }

// Radix-2 FFTs over `count` sequences of length M = 2^logm stored at buf + seq * M, with R
// consecutive radix-2 stages fused per shared-memory pass (R <= MAXR <= 4; with 4, M = 2048 takes
// three passes): each work item keeps the 2^R elements i0 + t * 2^s of one butterfly group in
// registers. tw[t] = exp(-2 pi i t / M). The forward row pass uses MAXR = 3.
__device__ __forceinline__ float2 twiddle(const float2* __restrict__ tw, int x, int shift, bool inverse) {
  float2 w = tw[x << shift];
  if (inverse) w.y = -w.y;
  return w;
}

// Radix-2 butterflies of one work item held in registers: v[e] is element i0 + e * h of its
// sequence, h = 2^s, j = i0 mod h. Decimation in time: stages s .. s + R - 1 (input of the FFT
// in bit-reversed order).
template <int R>
__device__ __forceinline__ void dit_regs(float2 (&v)[1 << R], int j, int s, int logm, const float2* __restrict__ tw,
                                         bool inverse) {
  constexpr int E = 1 << R;
  const int h = 1 << s;
#pragma unroll
  for (int st = 0; st < R; ++st) {
    const int span = 1 << st;               // partner distance in units of h
    const int shift = logm - 1 - (s + st);  // twiddle stride for block length 2^(s+st+1)
#pragma unroll
    for (int e = 0; e < E; ++e) {
      if (e & span) continue;
      const float2 w = twiddle(tw, j + (e & (span - 1)) * h, shift, inverse);
      const float2 x = cmul(v[e + span], w);
      const float2 u = v[e];
      v[e] = make_float2(u.x + x.x, u.y + x.y);
      v[e + span] = make_float2(u.x - x.x, u.y - x.y);
    }
  }
}

// Decimation in frequency: stages s + R - 1 down to s (output in bit-reversed order).
template <int R>
__device__ __forceinline__ void dif_regs(float2 (&v)[1 << R], int j, int s, int logm, const float2* __restrict__ tw,
                                         bool inverse) {
  constexpr int E = 1 << R;
  const int h = 1 << s;
#pragma unroll
  for (int st = R - 1; st >= 0; --st) {
    const int span = 1 << st;
    const int shift = logm - 1 - (s + st);
#pragma unroll
    for (int e = 0; e < E; ++e) {
      if (e & span) continue;
      const float2 w = twiddle(tw, j + (e & (span - 1)) * h, shift, inverse);
      const float2 u = v[e], x = v[e + span];
      v[e] = make_float2(u.x + x.x, u.y + x.y);
      v[e + span] = cmul(make_float2(u.x - x.x, u.y - x.y), w);
    }
  }
}

// One shared-memory pass of R stages starting at stage s over `count` sequences.
template <int R>
__device__ __forceinline__ void dit_pass(float2* buf, int count, int logm, int s, const float2* __restrict__ tw,
                                         bool inverse) {
  constexpr int E = 1 << R;
  const int h = 1 << s;
  const int items = count << (logm - R);
  for (int t = threadIdx.x; t < items; t += blockDim.x) {
    const int seq = t >> (logm - R);
    const int rem = t & ((1 << (logm - R)) - 1);
    const int j = rem & (h - 1);
    const int i0 = (seq << logm) + ((rem >> s) << (s + R)) + j;
    float2 v[E];
#pragma unroll
    for (int e = 0; e < E; ++e) v[e] = buf[sidx(i0 + e * h)];
    dit_regs<R>(v, j, s, logm, tw, inverse);
#pragma unroll
    for (int e = 0; e < E; ++e) buf[sidx(i0 + e * h)] = v[e];
  }
}

template <int R>
__device__ __forceinline__ void dif_pass(float2* buf, int count, int logm, int s, const float2* __restrict__ tw,
                                         bool inverse) {
  constexpr int E = 1 << R;
  const int h = 1 << s;
  const int items = count << (logm - R);
  for (int t = threadIdx.x; t < items; t += blockDim.x) {
    const int seq = t >> (logm - R);
    const int rem = t & ((1 << (logm - R)) - 1);
    const int j = rem & (h - 1);
    const int i0 = (seq << logm) + ((rem >> s) << (s + R)) + j;
    float2 v[E];
#pragma unroll
    for (int e = 0; e < E; ++e) v[e] = buf[sidx(i0 + e * h)];
    dif_regs<R>(v, j, s, logm, tw, inverse);
#pragma unroll
    for (int e = 0; e < E; ++e) buf[sidx(i0 + e * h)] = v[e];
  }
}

// Stages lo .. hi - 1 (decimation in time) or top down to lo (decimation in frequency), at most
// MAXR per shared-memory pass; each pass ends with a barrier.
template <int MAXR = 4>
__device__ void fft_dit(float2* buf, int count, int logm, const float2* __restrict__ tw, bool inverse, int lo = 0,
                        int hi = -1) {
  if (hi < 0) hi = logm;
  for (int s = lo; s < hi;) {
    const int r = min(MAXR, hi - s);
    if (r == 4) dit_pass<4>(buf, count, logm, s, tw, inverse);
    else if (r == 3) dit_pass<3>(buf, count, logm, s, tw, inverse);
    else if (r == 2) dit_pass<2>(buf, count, logm, s, tw, inverse);
    else dit_pass<1>(buf, count, logm, s, tw, inverse);
    __syncthreads();
    s += r;
  }
}

template <int MAXR = 4>
__device__ void fft_dif(float2* buf, int count, int logm, const float2* __restrict__ tw, bool inverse, int top = -1,
                        int lo = 0) {
  if (top < 0) top = logm - 1;
  while (top >= lo) {
    const int r = min(MAXR, top - lo + 1);
    const int s = top - r + 1;
    if (r == 4) dif_pass<4>(buf, count, logm, s, tw, inverse);
    else if (r == 3) dif_pass<3>(buf, count, logm, s, tw, inverse);
    else if (r == 2) dif_pass<2>(buf, count, logm, s, tw, inverse);
    else dif_pass<1>(buf, count, logm, s, tw, inverse);
    __syncthreads();
    top = s - 1;
  }
}

// Forward transforms are decimation in frequency (natural order in, bit-reversed order out) and
// inverse transforms decimation in time (bit-reversed in, natural out); spectra are stored in
// natural frequency order between the passes (written from, and loaded into, bit-reversed
// shared-memory positions), and the column pass multiplies its spectra element by element in
// the bit-reversed order both of its operands share.
//
// Real-input savings (the three charge planes and the kernel are real):
//   * the x and y charges travel as one complex plane A = x-charge + i y-charge (all M columns);
//   * the mass plane B is real, so its row spectra are Hermitian: B^[r][M - f] = conj(B^[r][f]),
//     and only f = 0 .. M/2 is kept. Rows are transformed in pairs (r, r + npairs): one complex
//     FFT of m_r + i m_r2 gives both half spectra;
//   * the kernel rows q + i q^2 are real and even in x: their spectra Kq + i Kq2 have real parts,
//     and K^[dy][M - f] = K^[dy][f], so f = 0 .. M/2 is kept;
//   * the column pass takes frequency columns in conjugate pairs (c, M - c): A_c, A_(M-c), B_c and
//     one kernel column (K_(M-c) = K_c) are transformed, B_(M-c) being conj(B_c) row by row;
//     the Parseval sum of the pair is twice that of column c (once for c = 0 and c = M/2);
//   * the inverse row pass rebuilds each B row's full spectrum from its half and transforms two
//     rows in one complex FFT (real parts: row r, imaginary parts: row r2).
// Per pair of rows and pair of columns that is 3 + 4 + 3 + 3 transforms of length M where the
// plain complex scheme needs 4 + 6 + 4 + 4 (and the kernel rows once per row in both).
__device__ __forceinline__ int bitrev(int f, int logm) { return (int)(__brev((unsigned)f) >> (32 - logm)); }
__device__ __forceinline__ float2 conjf2(float2 a) { return make_float2(a.x, -a.y); }

// The row pass's top forward pass (stages logm - 1 .. logm - kRowTop) runs on values loaded or
// computed straight into registers rather than staged in shared memory first; the butterflies
// are those of dif_pass.
constexpr int kRowTop = 3;

// Charge rows: the fixed-point charges of nodes j + e h of rows r1 (c1) and r2 (c2) are read,
// cleared for the next scatter and converted, then transformed as A_r1, A_r2 and m_r1 + i m_r2.
template <int R>
__device__ __forceinline__ void rows_charges_dif_top(float2* sbuf, longlong2* __restrict__ c1,
                                                     longlong2* __restrict__ c2, bool has2, int nodes, float inv_q,
                                                     int logm, const float2* __restrict__ tw) {
  constexpr int E = 1 << R;
  const int m = 1 << logm, s = logm - R, h = 1 << s;
  for (int j = threadIdx.x; j < h; j += blockDim.x) {
    float2 a[E];
    float mx[E], my[E];
#pragma unroll
    for (int e = 0; e < E; ++e) {
      const int c = j + e * h;
      a[e] = make_float2(0.0f, 0.0f);
      mx[e] = 0.0f;
      if (c < nodes) {
        const longlong2 p0 = c1[2 * c], p1 = c1[2 * c + 1];
        c1[2 * c] = make_longlong2(0, 0);
        c1[2 * c + 1] = make_longlong2(0, 0);
        a[e] = make_float2((float)p0.y * inv_q, (float)p1.x * inv_q);
        mx[e] = (float)p0.x * inv_q;
      }
    }
    dif_regs<R>(a, j, s, logm, tw, false);
#pragma unroll
    for (int e = 0; e < E; ++e) sbuf[sidx(j + e * h)] = a[e];
#pragma unroll
    for (int e = 0; e < E; ++e) {
      const int c = j + e * h;
      a[e] = make_float2(0.0f, 0.0f);
      my[e] = 0.0f;
      if (has2 && c < nodes) {
        const longlong2 p0 = c2[2 * c], p1 = c2[2 * c + 1];
        c2[2 * c] = make_longlong2(0, 0);
        c2[2 * c + 1] = make_longlong2(0, 0);
        a[e] = make_float2((float)p0.y * inv_q, (float)p1.x * inv_q);
        my[e] = (float)p0.x * inv_q;
      }
    }
    dif_regs<R>(a, j, s, logm, tw, false);
#pragma unroll
    for (int e = 0; e < E; ++e) sbuf[sidx(m + j + e * h)] = a[e];
#pragma unroll
    for (int e = 0; e < E; ++e) a[e] = make_float2(mx[e], my[e]);
    dif_regs<R>(a, j, s, logm, tw, false);
#pragma unroll
    for (int e = 0; e < E; ++e) sbuf[sidx(2 * m + j + e * h)] = a[e];
  }
}

// Kernel rows dy1 and dy2 (offsets yo1, yo2): (q, q^2) of columns j + e h, q = 1 / (1 + d^2),
// zero beyond +-(nodes - 1) columns.
template <int R>
__device__ __forceinline__ void rows_kernel_dif_top(float2* sbuf, int nodes, float h_node, float yo1, float yo2,
                                                    int logm, const float2* __restrict__ tw) {
  constexpr int E = 1 << R;
  const int m = 1 << logm, hm = m >> 1, s = logm - R, h = 1 << s;
  for (int j = threadIdx.x; j < h; j += blockDim.x) {
    float2 v1[E], v2[E];
#pragma unroll
    for (int e = 0; e < E; ++e) {
      const int c = j + e * h;
      const int dx = c < hm ? c : c - m;
      v1[e] = make_float2(0.0f, 0.0f);
      v2[e] = v1[e];
      if (dx <= nodes - 1 && dx >= -(nodes - 1)) {
        const float xo = (float)dx * h_node;
        const float q1 = 1.0f / (1.0f + (xo * xo + yo1 * yo1));
        const float q2 = 1.0f / (1.0f + (xo * xo + yo2 * yo2));
        v1[e] = make_float2(q1, q1 * q1);
        v2[e] = make_float2(q2, q2 * q2);
      }
    }
    dif_regs<R>(v1, j, s, logm, tw, false);
    dif_regs<R>(v2, j, s, logm, tw, false);
#pragma unroll
    for (int e = 0; e < E; ++e) {
      sbuf[sidx(j + e * h)] = v1[e];
      sbuf[sidx(m + j + e * h)] = v2[e];
    }
  }
}

// Row pass. Blocks [0, npairs): charge rows r1 = p and r2 = p + npairs (r2 < nodes or absent):
// forward FFTs of A_r1, A_r2 and m_r1 + i m_r2; A spectra to arow (natural order, all M),
// separated B half spectra to brow (f = 0 .. M/2); the charge rows are cleared for the next
// scatter. Blocks [npairs, 2 npairs): kernel rows dy1 = p and dy2 = p + npairs -> forward FFTs of
// (q + i q^2), f = 0 .. M/2 kept. blockIdx.y selects the instance members[blockIdx.y] of the grid
// class.
#ifndef FE_ROW_MIN_BLOCKS
#define FE_ROW_MIN_BLOCKS 4
#endif
__global__ void __launch_bounds__(kFftThreads, FE_ROW_MIN_BLOCKS)
rows_forward_kernel(const TsneInstance* __restrict__ inst, const int* __restrict__ members, int grid, int nodes,
                    int logm, const float2* __restrict__ tw, const GridState* __restrict__ cur,
                    float2* __restrict__ arow, float2* __restrict__ brow, float2* __restrict__ krow) {
  extern __shared__ float2 sbuf[];
  const int m = 1 << logm, hm = m >> 1;
  const int npairs = (nodes + 1) >> 1;
  const int b = members[blockIdx.y];
  long long* __restrict__ charges = inst[b].charges;
  cur += b;
  arow += (long long)blockIdx.y * nodes * m;
  brow += (long long)blockIdx.y * nodes * (hm + 1);
  krow += (long long)blockIdx.y * nodes * (hm + 1);
  if ((int)blockIdx.x < npairs) {
    const int r1 = blockIdx.x, r2 = blockIdx.x + npairs;
    const bool has2 = r2 < nodes;
    const float inv_q = cur->inv_qscale;
    longlong2* c1 = reinterpret_cast<longlong2*>(charges + (long long)r1 * grid * kChargeStride);
    longlong2* c2 = reinterpret_cast<longlong2*>(charges + (long long)(has2 ? r2 : r1) * grid * kChargeStride);
    rows_charges_dif_top<kRowTop>(sbuf, c1, c2, has2, nodes, inv_q, logm, tw);
    __syncthreads();
    fft_dif<3>(sbuf, 3, logm, tw, false, logm - kRowTop - 1, 0);
    float2* o1 = arow + (long long)r1 * m;
    float2* o2 = arow + (long long)r2 * m;
    for (int f = threadIdx.x; f < m; f += blockDim.x) {
      const int p = bitrev(f, logm);
      o1[f] = sbuf[sidx(p)];
      if (has2) o2[f] = sbuf[sidx(m + p)];
    }
    float2* b1 = brow + (long long)r1 * (hm + 1);
    float2* b2 = brow + (long long)r2 * (hm + 1);
    for (int f = threadIdx.x; f <= hm; f += blockDim.x) {
      const float2 z = sbuf[sidx(2 * m + bitrev(f, logm))];
      const float2 zc = conjf2(sbuf[sidx(2 * m + bitrev((m - f) & (m - 1), logm))]);
      b1[f] = make_float2(0.5f * (z.x + zc.x), 0.5f * (z.y + zc.y));
      if (has2) b2[f] = make_float2(0.5f * (z.y - zc.y), -0.5f * (z.x - zc.x));
    }
  } else {
    const int k1 = blockIdx.x - npairs, k2 = k1 + npairs;
    const bool has2 = k2 < nodes;
    const float h = cur->h;
    const float yo1 = (float)k1 * h, yo2 = (float)k2 * h;
    rows_kernel_dif_top<kRowTop>(sbuf, nodes, h, yo1, yo2, logm, tw);
    __syncthreads();
    fft_dif<3>(sbuf, 2, logm, tw, false, logm - kRowTop - 1, 0);
    float2* o1 = krow + (long long)k1 * (hm + 1);
    float2* o2 = krow + (long long)k2 * (hm + 1);
    for (int f = threadIdx.x; f <= hm; f += blockDim.x) {
      const int p = bitrev(f, logm);
      o1[f] = sbuf[sidx(p)];
      if (has2) o2[f] = sbuf[sidx(m + p)];
    }
  }
}

// Column pass for the conjugate pair (c, c') = (j, M - j), j = 0 .. M/2 (c' = c for j = 0 and
// M/2): column FFTs of A_c, A_c', B_c and the kernel column K_c (giving the real spectra
// Kq + i Kq2), the Parseval sum of |B^|^2 Kq over both columns of the pair (Z + n up to the
// 1 / M^2 scale), the products with Kq2 and their inverse column FFTs; rows < nodes of the
// results go back to arow / brow.
//
// Three shared-memory round trips of the plain scheme are kept in registers, with the same
// radix-2 butterflies: the top forward pass takes its inputs straight from global memory, the
// last forward pass (stages 2 .. 0, groups of 8 consecutive positions), the products and the
// first inverse pass (stages 0 .. 2, the same groups) run in one pass, and the top inverse pass
// writes its outputs straight to global memory.
constexpr int kColBottom = 3;

template <int R>
__device__ __forceinline__ void col_load_dif_top(float2* sbuf, const float2* __restrict__ arow,
                                                 const float2* __restrict__ brow, const float2* __restrict__ krow,
                                                 int c, int c2, int nodes, int logm, const float2* __restrict__ tw) {
  constexpr int E = 1 << R;
  const int m = 1 << logm, hm = m >> 1;
  const int s = logm - R, h = 1 << s;
  const int items = 4 << s;
  for (int t = threadIdx.x; t < items; t += blockDim.x) {
    const int seq = t >> s, j = t & (h - 1);
    float2 v[E];
#pragma unroll
    for (int e = 0; e < E; ++e) {
      const int r = j + e * h;
      float2 x = make_float2(0.0f, 0.0f);
      if (seq == 3) {
        const int dy = r < hm ? r : m - r;
        if (dy <= nodes - 1) x = krow[(long long)dy * (hm + 1) + c];
      } else if (r < nodes) {
        x = seq == 2 ? brow[(long long)r * (hm + 1) + c] : arow[(long long)r * m + (seq == 0 ? c : c2)];
      }
      v[e] = x;
    }
    dif_regs<R>(v, j, s, logm, tw, false);
#pragma unroll
    for (int e = 0; e < E; ++e) sbuf[sidx((seq << logm) + j + e * h)] = v[e];
  }
}

template <int R>
__device__ __forceinline__ void col_dit_top_store(const float2* sbuf, float2* __restrict__ arow,
                                                  float2* __restrict__ brow, int c, int c2, int nodes, int logm,
                                                  const float2* __restrict__ tw) {
  constexpr int E = 1 << R;
  const int m = 1 << logm, hm = m >> 1;
  const int s = logm - R, h = 1 << s;
  const int items = 3 << s;
  for (int t = threadIdx.x; t < items; t += blockDim.x) {
    const int seq = t >> s, j = t & (h - 1);
    if (seq == 1 && c2 == c) continue;
    float2 v[E];
#pragma unroll
    for (int e = 0; e < E; ++e) v[e] = sbuf[sidx((seq << logm) + j + e * h)];
    dit_regs<R>(v, j, s, logm, tw, true);
#pragma unroll
    for (int e = 0; e < E; ++e) {
      const int r = j + e * h;
      if (r < nodes) {
        if (seq == 2) brow[(long long)r * (hm + 1) + c] = v[e];
        else arow[(long long)r * m + (seq == 0 ? c : c2)] = v[e];
      }
    }
  }
}

// 3 blocks per SM, as the 4 x M complex shared-memory buffer allows at M = 2048
#ifndef FE_COL_MIN_BLOCKS
#define FE_COL_MIN_BLOCKS 3
#endif
__global__ void __launch_bounds__(kColThreads, FE_COL_MIN_BLOCKS)
columns_convolve_kernel(float2* __restrict__ arow, float2* __restrict__ brow, const float2* __restrict__ krow,
                        int nodes, int logm, const float2* __restrict__ tw, double* __restrict__ zpart) {
  extern __shared__ float2 sbuf[];  // [A_c][A_c'][B_c][K_c]
  __shared__ double s_z[kColThreads / 32];
  const int m = 1 << logm, hm = m >> 1;
  const int j = blockIdx.x;
  const int c = j, c2 = (m - j) & (m - 1);
  arow += (long long)blockIdx.y * nodes * m;
  brow += (long long)blockIdx.y * nodes * (hm + 1);
  krow += (long long)blockIdx.y * nodes * (hm + 1);
  zpart += (long long)blockIdx.y * gridDim.x;
  // logm >= 4 (M >= 16): the top pass has 1 .. 4 stages above the fused bottom three
  const int rt = min(4, logm - kColBottom);
  if (rt == 4) col_load_dif_top<4>(sbuf, arow, brow, krow, c, c2, nodes, logm, tw);
  else if (rt == 3) col_load_dif_top<3>(sbuf, arow, brow, krow, c, c2, nodes, logm, tw);
  else if (rt == 2) col_load_dif_top<2>(sbuf, arow, brow, krow, c, c2, nodes, logm, tw);
  else col_load_dif_top<1>(sbuf, arow, brow, krow, c, c2, nodes, logm, tw);
  __syncthreads();
  fft_dif(sbuf, 4, logm, tw, false, logm - rt - 1, kColBottom);
  double zl = 0.0;
  constexpr int E = 1 << kColBottom;
  for (int g = threadIdx.x; g < (m >> kColBottom); g += blockDim.x) {
    const int i0 = g << kColBottom;
    float2 kv[E];
#pragma unroll
    for (int e = 0; e < E; ++e) kv[e] = sbuf[sidx(3 * m + i0 + e)];
    dif_regs<kColBottom>(kv, 0, 0, logm, tw, false);
#pragma unroll
    for (int seq = 0; seq < 3; ++seq) {
      float2 v[E];
#pragma unroll
      for (int e = 0; e < E; ++e) v[e] = sbuf[sidx(seq * m + i0 + e)];
      dif_regs<kColBottom>(v, 0, 0, logm, tw, false);
#pragma unroll
      for (int e = 0; e < E; ++e) {
        if (seq == 2) zl += ((double)v[e].x * v[e].x + (double)v[e].y * v[e].y) * (double)kv[e].x;
        v[e].x *= kv[e].y;
        v[e].y *= kv[e].y;
      }
      dit_regs<kColBottom>(v, 0, 0, logm, tw, true);
#pragma unroll
      for (int e = 0; e < E; ++e) sbuf[sidx(seq * m + i0 + e)] = v[e];
    }
  }
  __syncthreads();
  fft_dit(sbuf, 3, logm, tw, true, kColBottom, logm - rt);
  if (rt == 4) col_dit_top_store<4>(sbuf, arow, brow, c, c2, nodes, logm, tw);
  else if (rt == 3) col_dit_top_store<3>(sbuf, arow, brow, c, c2, nodes, logm, tw);
  else if (rt == 2) col_dit_top_store<2>(sbuf, arow, brow, c, c2, nodes, logm, tw);
  else col_dit_top_store<1>(sbuf, arow, brow, c, c2, nodes, logm, tw);
  zl = warp_sum(zl);
  if ((threadIdx.x & 31) == 0) s_z[threadIdx.x >> 5] = zl;
  __syncthreads();
  if (threadIdx.x == 0) {
    double z = 0.0;
    for (int w = 0; w < (int)(blockDim.x / 32); ++w) z += s_z[w];
    zpart[blockIdx.x] = c2 != c ? 2.0 * z : z;
  }
}

// Inverse row pass for the row pair (r1, r2) -> potentials (phi_q2, phi_x, phi_y) per node; block
// 0 also finalises Z = sum_k |F_mass|^2 Kq / M^2 - n (the reference's sum_i q_grid(y_i) - n).
__global__ void __launch_bounds__(kFftThreads, 4)
rows_inverse_kernel(const float2* __restrict__ arow, const float2* __restrict__ brow,
                    const TsneInstance* __restrict__ inst, const int* __restrict__ members, int grid, int nodes,
                    int logm, const float2* __restrict__ tw, const double* __restrict__ zpart, int zblocks,
                    GridState* __restrict__ cur) {
  extern __shared__ float2 sbuf[];
  const int m = 1 << logm, hm = m >> 1;
  const int npairs = (nodes + 1) >> 1;
  const int r1 = blockIdx.x, r2 = blockIdx.x + npairs;
  const bool has2 = r2 < nodes;
  const int b = members[blockIdx.y];
  const TsneInstance& I = inst[b];
  float4* __restrict__ potential = I.potential;
  const int n = I.n;
  cur += b;
  arow += (long long)blockIdx.y * nodes * m;
  brow += (long long)blockIdx.y * nodes * (hm + 1);
  zpart += (long long)blockIdx.y * zblocks;
  const float2* a1 = arow + (long long)r1 * m;
  const float2* a2 = arow + (long long)r2 * m;
  const float2* b1 = brow + (long long)r1 * (hm + 1);
  const float2* b2 = brow + (long long)r2 * (hm + 1);
  for (int f = threadIdx.x; f < m; f += blockDim.x) {
    const int p = bitrev(f, logm);
    sbuf[sidx(p)] = a1[f];
    sbuf[sidx(m + p)] = has2 ? a2[f] : make_float2(0.0f, 0.0f);
    // full spectra of the two real B rows from their halves, packed as X1 + i X2
    const float2 x1 = f <= hm ? b1[f] : conjf2(b1[m - f]);
    const float2 x2 = has2 ? (f <= hm ? b2[f] : conjf2(b2[m - f])) : make_float2(0.0f, 0.0f);
    sbuf[sidx(2 * m + p)] = make_float2(x1.x - x2.y, x1.y + x2.x);
  }
  __syncthreads();
  fft_dit(sbuf, 3, logm, tw, true);
  const float scale = 1.0f / ((float)m * (float)m);
  float4* o1 = potential + (long long)r1 * grid;
  float4* o2 = potential + (long long)r2 * grid;
  for (int c = threadIdx.x; c < nodes; c += blockDim.x) {
    const float2 q1 = sbuf[sidx(c)], pb = sbuf[sidx(2 * m + c)];
    o1[c] = make_float4(pb.x * scale, q1.x * scale, q1.y * scale, 0.0f);
    if (has2) {
      const float2 q2 = sbuf[sidx(m + c)];
      o2[c] = make_float4(pb.y * scale, q2.x * scale, q2.y * scale, 0.0f);
    }
  }
  if (r1 == 0) {
    __shared__ double s_z[kFftThreads];
    double z = 0.0;
    for (int t = threadIdx.x; t < zblocks; t += blockDim.x) z += zpart[t];
    s_z[threadIdx.x] = z;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
      if ((int)threadIdx.x < w) s_z[threadIdx.x] += s_z[threadIdx.x + w];
      __syncthreads();
    }
    if (threadIdx.x == 0) {
      const double zz = s_z[0] / ((double)m * (double)m) - (double)n;
      cur->z = zz;
      cur->inv_z = (float)(1.0 / fmax(zz, (double)FLT_MIN));
    }
  }
}

// ---------------------------------------------------------------- attractive pass
// a_i = exag * sum_j p_ij q_ij (y_i - y_j), q = 1 / (1 + d^2)
// (add_sparse_attractive_gradient_f, src/tsne_neighbors.cpp:1061-1088).
// Rows are taken in storage (spatial) order: slot_rows[s] = (begin, end) of the CSR row of the
// point in slot s (rebuilt at every reorder), so a row is one contiguous segment of P and
// consecutive rows of a warp belong to neighbouring points, whose neighbour sets overlap: their
// y gathers hit L1. Warp w first takes chunk w of `chunk` consecutive slots, then further
// chunks from a counter (the last warp to finish resets it for the next launch), which keeps
// every SM busy to the end whatever the row lengths of a region. The chunk size and the number of
// resident blocks are launch parameters chosen at run time by timing (tsne_tune_attractive): the
// result does not depend on them. A row is read with 128-bit loads: lane l takes entries
// c0 + 4 l .. + 3 of each 128-entry round (c0 = the row's first entry rounded down to a multiple
// of 4; entries outside the row are masked), kAttrRounds rounds loaded before their gathers.
// Lane 0 keeps a bulk L2 prefetch (cp.async.bulk.prefetch) of the row kAttrAhead rows ahead.
// Each lane sums its entries in a fixed order, the rounds of a row longer than one group are
// added with Kahan compensation, and the warp sum is a fixed butterfly: the force depends only
// on the row and its entries' positions modulo 4, not on the schedule.
constexpr int kAttrThreads = 256;
constexpr int kAttrWarps = kAttrThreads / 32;
constexpr int kAttrAhead = 2;
// Compile-time shape of the pass (measured alternatives in the attractive-pass variants profile):
// 128-entry rounds loaded together (1: 40 registers) and the register cap that allows six
// resident blocks per SM.
#ifndef FE_ATTR_ROUNDS
#define FE_ATTR_ROUNDS 1
#endif
constexpr int kAttrRounds = FE_ATTR_ROUNDS;

__device__ __forceinline__ void prefetch_l2_range(const void* base, long long first, long long last, int elem) {
  // [first, last) elements of a 4-byte array, widened to 16-byte boundaries (the arena pads
  // every buffer to 256 bytes, so the widened range stays inside the allocation)
  if (last <= first) return;
  const unsigned long long a = (unsigned long long)base + (unsigned long long)(first * elem);
  const unsigned long long e = (unsigned long long)base + (unsigned long long)(last * elem);
  const unsigned long long a16 = a & ~15ull, e16 = (e + 15ull) & ~15ull;
  asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(a16), "r"((unsigned)(e16 - a16)) : "memory");
}

__device__ __forceinline__ int int4_at(const int4& v, int c) { return c == 0 ? v.x : c == 1 ? v.y : c == 2 ? v.z : v.w; }
__device__ __forceinline__ float float4_at(const float4& v, int c) {
  return c == 0 ? v.x : c == 1 ? v.y : c == 2 ? v.z : v.w;
}

// Butterfly of lane partials (x, y): the warp's x sum ends in lanes 0-15, its y sum in lanes
// 16-31 (fixed order).
__device__ __forceinline__ float butterfly_xy(float x, float y, int lane) {
  const bool upper = lane >= 16;
  float keep = upper ? y : x;
  const float send = upper ? x : y;
  keep += __shfl_xor_sync(0xffffffffu, send, 16);
  keep += __shfl_xor_sync(0xffffffffu, keep, 8);
  keep += __shfl_xor_sync(0xffffffffu, keep, 4);
  keep += __shfl_xor_sync(0xffffffffu, keep, 2);
  keep += __shfl_xor_sync(0xffffffffu, keep, 1);
  return keep;
}

__device__ __forceinline__ void prefetch_row(const int2* __restrict__ slot_rows, const int* col, const float* val,
                                             int s) {
  const int2 se = __ldg(slot_rows + s);
  prefetch_l2_range(col, se.x, se.y, 4);
  prefetch_l2_range(val, se.x, se.y, 4);
}

#ifndef FE_ATTR_MIN_BLOCKS
#define FE_ATTR_MIN_BLOCKS 6
#endif
__global__ void __launch_bounds__(kAttrThreads, FE_ATTR_MIN_BLOCKS)
attractive_kernel(const int2* __restrict__ slot_rows, const int* __restrict__ col, const float* __restrict__ val,
                  const float2* __restrict__ y, int n, float exag, float2* __restrict__ attr,
                  unsigned* __restrict__ ctr, int chunk) {
  const int lane = threadIdx.x & 31;
  const unsigned nchunks = (unsigned)((n + chunk - 1) / chunk);
  const unsigned nwarps = gridDim.x * kAttrWarps;
  // chunk gw first, then chunks nwarps, nwarps + 1, ... from the counter
  unsigned c = blockIdx.x * kAttrWarps + (threadIdx.x >> 5), next = 0;
  if (lane == 0) next = nwarps + atomicAdd(ctr, 1u);
  next = __shfl_sync(0xffffffffu, next, 0);
  // slot at position t of chunk c (positions past the chunk run into chunk `next`), or -1
  auto slot_at = [&](int t) -> int {
    const unsigned ch = t < chunk ? c : next;
    if (ch >= nchunks) return -1;
    const int sl = (int)ch * chunk + (t < chunk ? t : t - chunk);
    return sl < n ? sl : -1;
  };
  if (lane == 0)
    for (int a = 0; a < kAttrAhead; ++a) {
      const int t = slot_at(a);
      if (t >= 0) prefetch_row(slot_rows, col, val, t);
    }
  while (c < nchunks) {
    for (int t = 0; t < chunk; ++t) {
      const int s = slot_at(t);
      if (s < 0) break;
      if (lane == 0) {
        const int pf = slot_at(t + kAttrAhead);
        if (pf >= 0) prefetch_row(slot_rows, col, val, pf);
      }
      const int2 se = __ldg(slot_rows + s);
      const float2 yi = __ldg(y + s);
      const int b = se.x, e = se.y;
      float ax = 0.0f, ay = 0.0f, kx = 0.0f, ky = 0.0f;
      for (int c0 = b & ~3; c0 < e; c0 += 128 * kAttrRounds) {
        int4 ci[kAttrRounds];
        float4 vv[kAttrRounds];
#pragma unroll
        for (int u = 0; u < kAttrRounds; ++u) {
          const int p = c0 + 128 * u + 4 * lane;
          if (p < e) {
            ci[u] = __ldcs(reinterpret_cast<const int4*>(col + p));
            vv[u] = __ldcs(reinterpret_cast<const float4*>(val + p));
          } else {
            ci[u] = make_int4(s, s, s, s);
            vv[u] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
          }
        }
        float rx = 0.0f, ry = 0.0f;
#pragma unroll
        for (int u = 0; u < kAttrRounds; ++u) {
#pragma unroll
          for (int cc = 0; cc < 4; ++cc) {
            const int p = c0 + 128 * u + 4 * lane + cc;
            const bool ok = p >= b && p < e;
            const float w = ok ? float4_at(vv[u], cc) : 0.0f;
            const float2 yj = ok ? __ldg(y + int4_at(ci[u], cc)) : yi;
            const float dx = yi.x - yj.x, dy = yi.y - yj.y;
            // fast reciprocal (within 2 ulp; 1 + d^2 >= 1 is never denormal or huge): the IEEE
            // division's instruction sequence cost 5 % of this issue-limited pass
            const float q = __fdividef(1.0f, 1.0f + (dx * dx + dy * dy));
            const float cq = w * q;
            rx += cq * dx;
            ry += cq * dy;
          }
        }
        const float tx = rx - kx, ty = ry - ky;
        const float nx = ax + tx, ny = ay + ty;
        kx = (nx - ax) - tx;
        ky = (ny - ay) - ty;
        ax = nx;
        ay = ny;
      }
      const float keep = butterfly_xy(ax, ay, lane);
      const float sy = __shfl_sync(0xffffffffu, keep, 16);
      if (lane == 0) attr[s] = make_float2(exag * keep, exag * sy);
    }
    c = next;
    if (c < nchunks) {
      if (lane == 0) next = nwarps + atomicAdd(ctr, 1u);
      next = __shfl_sync(0xffffffffu, next, 0);
    }
  }
  if (lane == 0) {
    __threadfence();
    const unsigned done = atomicAdd(ctr + 1, 1u);
    if (done == gridDim.x * kAttrWarps - 1u) {
      atomicExch(ctr, 0u);
      atomicExch(ctr + 1, 0u);
    }
  }
}

// slot_rows[t] = CSR segment of the point stored in slot t.
__global__ void bind_rows_kernel(const int* __restrict__ perm, const int* __restrict__ row_ptr, int n,
                                 int2* __restrict__ slot_rows) {
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
    const int o = perm[t];
    slot_rows[t] = make_int2(row_ptr[o], row_ptr[o + 1]);
  }
}

// ---------------------------------------------------------------- update
template <int TAPS>
__device__ __forceinline__ float pick(const float (&w)[TAPS], int a) {
  float v = w[0];
#pragma unroll
  for (int t = 1; t < TAPS; ++t) v = a == t ? w[t] : v;
  return v;
}

__device__ __forceinline__ int sign3(float v) { return (v > 0.0f) - (v < 0.0f); }

// One thread per point: interpolate the potentials, form the gradient
//   g_i = a_i - ((y_i - c) phi_q2 - phi_xy) / Z     (src/tsne_neighbors.cpp:1247-1259)
// and apply gains / momentum / step clip (apply_open_tsne_update_f, :1297-1336) with the
// recentring of zero_mean_f (:1280-1291) folded in by subtracting the previous mean. The
// epilogue reduces bounding box and mean of the new layout into `next`. DIAG writes the
// repulsive force instead of updating.
template <int TAPS, bool DIAG>
__global__ void __launch_bounds__(kStepThreads)
update_kernel(float2* __restrict__ y, const float2* __restrict__ attr, float2* __restrict__ gains,
              float2* __restrict__ update, const TsneInstance* __restrict__ inst, const int2* __restrict__ blocks,
              const GridState* __restrict__ cur, GridState* __restrict__ next, StepPartial* __restrict__ part,
              unsigned* __restrict__ counter, int mode, float lr, float mom, float min_gain, float max_step,
              float2* __restrict__ out_rep) {
  const int2 bl = blocks[blockIdx.x];
  const TsneInstance I = inst[bl.x];
  const GridState g = cur[bl.x];
  const float4* __restrict__ pot = I.potential;
  const int grid = I.grid;
  const float lr_i = lr * I.lr_mult;
  const bool clip = isfinite(max_step) && max_step > 0.0f;
  const float max2 = max_step * max_step;
  float mnx = FLT_MAX, mxx = -FLT_MAX, mny = FLT_MAX, mxy = -FLT_MAX;
  double sx = 0.0, sy = 0.0;
  const int i = bl.y + threadIdx.x;
  if (i < I.pt_begin + I.n) {
    const float2 p = y[i];
    const Stencil<TAPS> stx = make_stencil<TAPS>(p.x, g.x0, g.inv_h, g.inv_box, g.nodes);
    const Stencil<TAPS> sty = make_stencil<TAPS>(p.y, g.y0, g.inv_h, g.inv_box, g.nodes);
    float r0 = 0.0f, r1 = 0.0f, r2 = 0.0f;
#pragma unroll
    for (int a = 0; a < TAPS; ++a) {
      const float4* row = pot + (long long)(sty.base + a) * grid + stx.base;
#pragma unroll
      for (int b = 0; b < TAPS; ++b) {
        const float w = sty.w[a] * stx.w[b];
        const float4 f = __ldg(row + b);
        r0 += w * f.x;
        r1 += w * f.y;
        r2 += w * f.z;
      }
    }
    const float repx = -((p.x - g.cx) * r0 - r1) * g.inv_z;
    const float repy = -((p.y - g.cy) * r0 - r2) * g.inv_z;
    if constexpr (DIAG) {
      out_rep[i] = make_float2(repx, repy);
    } else {
      const float2 a = attr[i];
      const float gx = repx + a.x, gy = repy + a.y;
      const float2 ga = gains[i], up = update[i];
      float gnx = sign3(up.x) != sign3(gx) ? ga.x + 0.2f : ga.x * 0.8f + min_gain;
      float gny = sign3(up.y) != sign3(gy) ? ga.y + 0.2f : ga.y * 0.8f + min_gain;
      if (gnx < min_gain) gnx = min_gain;
      if (gny < min_gain) gny = min_gain;
      float ux = mom * up.x - lr_i * gnx * gx;
      float uy = mom * up.y - lr_i * gny * gy;
      const float s2 = ux * ux + uy * uy;
      if (clip && s2 > max2) {
        const float sc = max_step / sqrtf(fmaxf(s2, FLT_MIN));
        ux *= sc;
        uy *= sc;
      }
      const float nx = (p.x - (float)g.mean_x) + ux;
      const float ny = (p.y - (float)g.mean_y) + uy;
      gains[i] = make_float2(gnx, gny);
      update[i] = make_float2(ux, uy);
      y[i] = make_float2(nx, ny);
      mnx = mxx = nx;
      mny = mxy = ny;
      sx = nx;
      sy = ny;
    }
  }
  if constexpr (!DIAG) {
    block_partial(mnx, mxx, mny, mxy, sx, sy, part + blockIdx.x);
    if (last_block_done(counter + bl.x, I.blocks))
      finish_layout_stats(part + I.block_begin, I.blocks, I.n, I.grid, mode, next + bl.x);
  }
}

__global__ void fill_state_kernel(float2* __restrict__ gains, float2* __restrict__ update, int n) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    gains[i] = make_float2(1.0f, 1.0f);
    update[i] = make_float2(0.0f, 0.0f);
  }
}

__global__ void finalize_kernel(const float2* __restrict__ y, const TsneInstance* __restrict__ inst,
                                const int2* __restrict__ blocks, const GridState* __restrict__ next,
                                const int* __restrict__ perm, float2* __restrict__ out) {
  const int2 bl = blocks[blockIdx.x];
  const TsneInstance& I = inst[bl.x];
  const float mx = (float)next[bl.x].mean_x, my = (float)next[bl.x].mean_y;
  const int i = bl.y + threadIdx.x;
  if (i < I.pt_begin + I.n) {
    const float2 p = y[i];
    out[perm ? perm[i] : i] = make_float2(p.x - mx, p.y - my);
  }
}

// ---------------------------------------------------------------- spatial reorder
__device__ __forceinline__ unsigned spread_bits(unsigned v) {
  v &= 0xffffu;
  v = (v | (v << 8)) & 0x00ff00ffu;
  v = (v | (v << 4)) & 0x0f0f0f0fu;
  v = (v | (v << 2)) & 0x33333333u;
  v = (v | (v << 1)) & 0x55555555u;
  return v;
}

// Sort key: instance index above the Morton code of the stencil anchor, so a stable sort keeps
// every instance inside its slot range.
template <int TAPS>
__global__ void anchor_keys_kernel(const float2* __restrict__ y, const TsneInstance* __restrict__ inst,
                                   const int2* __restrict__ blocks, const GridState* __restrict__ next,
                                   int morton_bits, unsigned* __restrict__ keys, int* __restrict__ order) {
  const int2 bl = blocks[blockIdx.x];
  const TsneInstance& I = inst[bl.x];
  const GridState g = next[bl.x];
  const int i = bl.y + threadIdx.x;
  if (i < I.pt_begin + I.n) {
    const float2 p = y[i];
    const int bx = make_stencil<TAPS>(p.x, g.x0, g.inv_h, g.inv_box, g.nodes).base;
    const int by = make_stencil<TAPS>(p.y, g.y0, g.inv_h, g.inv_box, g.nodes).base;
    keys[i] = ((unsigned)bl.x << morton_bits) | spread_bits((unsigned)bx) | (spread_bits((unsigned)by) << 1);
    order[i] = i;
  }
}

__global__ void gather_points_kernel(const int* __restrict__ order, int n, const float2* __restrict__ y,
                                     const float2* __restrict__ gains, const float2* __restrict__ update,
                                     const int* __restrict__ perm, float2* __restrict__ scratch,
                                     int* __restrict__ perm_tmp, int* __restrict__ delta) {
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
    const int o = order[r];
    scratch[r] = y[o];
    scratch[n + r] = gains[o];
    scratch[2 * (long long)n + r] = update[o];
    perm_tmp[r] = perm[o];
    delta[o] = r;
  }
}

__global__ void scatter_points_kernel(const float2* __restrict__ scratch, const int* __restrict__ perm_tmp, int n,
                                      const int* __restrict__ row_ptr, float2* __restrict__ y,
                                      float2* __restrict__ gains, float2* __restrict__ update, int* __restrict__ perm,
                                      int* __restrict__ inv, int2* __restrict__ slot_rows) {
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
    y[r] = scratch[r];
    gains[r] = scratch[n + r];
    update[r] = scratch[2 * (long long)n + r];
    const int o = perm_tmp[r];
    perm[r] = o;
    inv[o] = r;
    slot_rows[r] = make_int2(row_ptr[o], row_ptr[o + 1]);
  }
}

__global__ void relabel_cols_kernel(int* __restrict__ col, long long nnz, const int* __restrict__ delta) {
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < nnz; p += (long long)gridDim.x * blockDim.x)
    col[p] = __ldg(delta + __ldcs(col + p));
}

__global__ void identity_kernel(int* __restrict__ perm, int* __restrict__ inv, int n) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    perm[i] = i;
    inv[i] = i;
  }
}

// ---------------------------------------------------------------- host side
namespace {
int point_blocks(int n) { return std::max(1, std::min(ceil_div(n, 256), sm_count() * 8)); }

template <typename K>
int persistent_blocks(K kernel, int threads, long long warps_needed) {
  int per_sm = 0;
  FE_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, 0));
  per_sm = std::max(1, per_sm);
  return std::max(1, (int)std::min<long long>((long long)per_sm * sm_count(), (warps_needed + threads / 32 - 1) /
                                                                                   (threads / 32)));
}

int log2_ceil(int v) {
  int b = 0;
  while ((1 << b) < v) ++b;
  return b;
}
}  // namespace

TsneDevice::~TsneDevice() {
  if (fork) cudaEventDestroy(fork);
  if (join) cudaEventDestroy(join);
  if (side) cudaStreamDestroy(side);
}

int default_grid_size(int n, int /*mode*/) { return cuda_fft_grid_size(n); }

void tsne_device_alloc(TsneDevice& d, int n, int grid, int mode) {
  tsne_batch_alloc(d, std::vector<int>{n}, std::vector<int>{grid}, std::vector<float>{1.0f}, mode);
}

namespace {
// Group instances by grid size, allocate the class workspaces in d.grid_arena and point the
// instance table at them (host copy; the caller uploads it).
void build_grid_classes(TsneDevice& d, const std::vector<int>& grids) {
  const int ninst = (int)d.inst.size();
  std::vector<int> distinct(grids.begin(), grids.end());
  std::sort(distinct.begin(), distinct.end());
  distinct.erase(std::unique(distinct.begin(), distinct.end()), distinct.end());
  d.classes.assign(distinct.size(), GridClass{});
  std::vector<std::vector<int>> members(distinct.size());
  for (int b = 0; b < ninst; ++b) {
    const int g = grids[b];
    if (g < 8 || g > 2048 || (g & (g - 1)) != 0) throw Error("`grid_size` must be a power of two between 8 and 2048.");
    const int c = (int)(std::lower_bound(distinct.begin(), distinct.end(), g) - distinct.begin());
    members[c].push_back(b);
  }
  d.grid_arena.release();
  int* d_members = nullptr;
  d.grid_arena.reserve(&d_members, ninst);
  for (std::size_t c = 0; c < distinct.size(); ++c) {
    GridClass& k = d.classes[c];
    k.grid = distinct[c];
    k.nodes = d.mode == kInterpBilinear ? k.grid : 3 * (k.grid / 3);
    k.fft = 2 * k.grid;
    k.log_fft = log2_ceil(k.fft);
    k.count = (int)members[c].size();
    k.col_blocks = k.fft / 2 + 1;
    const std::size_t m = k.fft;
    d.grid_arena.reserve(&k.charges, (std::size_t)k.count * k.grid * k.grid * kChargeStride);
    d.grid_arena.reserve(&k.potential, (std::size_t)k.count * k.grid * k.grid);
    d.grid_arena.reserve(&k.arow, (std::size_t)k.count * k.nodes * m);
    d.grid_arena.reserve(&k.brow, (std::size_t)k.count * k.nodes * (m / 2 + 1));
    d.grid_arena.reserve(&k.krow, (std::size_t)k.count * k.nodes * (m / 2 + 1));
    d.grid_arena.reserve(&k.twiddle, m / 2);
    d.grid_arena.reserve(&k.zpart, (std::size_t)k.count * k.col_blocks);
  }
  d.grid_arena.commit("t-SNE grid workspaces");
  std::vector<int> flat;
  int max_m = 0, max_grid = 0;
  for (std::size_t c = 0; c < distinct.size(); ++c) {
    GridClass& k = d.classes[c];
    k.members = d_members + flat.size();
    const int m = k.fft;
    max_m = std::max(max_m, m);
    max_grid = std::max(max_grid, k.grid);
    for (int j = 0; j < k.count; ++j) {
      const int b = members[c][j];
      flat.push_back(b);
      TsneInstance& I = d.inst[b];
      I.grid = k.grid;
      I.nodes = k.nodes;
      I.charges = k.charges + (std::size_t)j * k.grid * k.grid * kChargeStride;
      I.potential = k.potential + (std::size_t)j * k.grid * k.grid;
    }
    std::vector<float2> tw(m / 2);
    for (int t = 0; t < m / 2; ++t) {
      const double ang = -2.0 * M_PI * (double)t / (double)m;
      tw[t] = make_float2((float)std::cos(ang), (float)std::sin(ang));
    }
    FE_CUDA(cudaMemcpy(k.twiddle, tw.data(), sizeof(float2) * tw.size(), cudaMemcpyHostToDevice));
    FE_CUDA(cudaMemset(k.charges, 0, sizeof(long long) * kChargeStride * (std::size_t)k.count * k.grid * k.grid));
    FE_CUDA(cudaMemset(k.potential, 0, sizeof(float4) * (std::size_t)k.count * k.grid * k.grid));
  }
  FE_CUDA(cudaMemcpy(d_members, flat.data(), sizeof(int) * ninst, cudaMemcpyHostToDevice));
  d.grid = d.inst[0].grid;
  d.nodes = d.inst[0].nodes;
  d.key_bits = 2 * log2_ceil(max_grid);
  d.sort_bits = d.key_bits + log2_ceil(ninst);
  if (d.sort_bits > 32) throw Error("t-SNE batch: too many instances for the spatial sort key");
  const int big = padded(4 * max_m) * (int)sizeof(float2);
  FE_CUDA(cudaFuncSetAttribute(columns_convolve_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, big));
  const int rowb = padded(3 * max_m) * (int)sizeof(float2);
  FE_CUDA(cudaFuncSetAttribute(rows_forward_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, rowb));
  FE_CUDA(cudaFuncSetAttribute(rows_inverse_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, rowb));
}
}  // namespace

void tsne_batch_alloc(TsneDevice& d, const std::vector<int>& sizes, const std::vector<int>& grids,
                      const std::vector<float>& lr_mult, int mode) {
  const int ninst = (int)sizes.size();
  if (ninst < 1 || grids.size() != sizes.size() || lr_mult.size() != sizes.size())
    throw Error("t-SNE batch: one size, grid and learning-rate multiplier per instance");
  d.mode = mode;
  d.inst.assign(ninst, TsneInstance{});
  long long total = 0;
  int nblocks = 0;
  for (int b = 0; b < ninst; ++b) {
    if (sizes[b] < 2) throw Error("t-SNE batch: every instance needs at least two points");
    TsneInstance& I = d.inst[b];
    I.pt_begin = (int)total;
    I.n = sizes[b];
    I.block_begin = nblocks;
    I.blocks = ceil_div(sizes[b], kPointBlock);
    I.lr_mult = lr_mult[b];
    total += sizes[b];
    nblocks += I.blocks;
  }
  if (total > INT_MAX / 2) throw Error("t-SNE batch: too many points");
  const int n = (int)total;
  d.n = n;
  d.nblocks = nblocks;
  d.attr_blocks = persistent_blocks(attractive_kernel, kAttrThreads, n);
  d.arena.release();
  d.arena.reserve(&d.d_inst, ninst);
  d.arena.reserve(&d.blocks, nblocks);
  d.arena.reserve(&d.y, n);
  d.arena.reserve(&d.attr, n);
  d.arena.reserve(&d.gains, n);
  d.arena.reserve(&d.update, n);
  d.arena.reserve(&d.cur, ninst);
  d.arena.reserve(&d.next, ninst);
  d.arena.reserve(&d.partial, nblocks);
  d.arena.reserve(&d.counter, ninst);
  const int nb = radix_sort_blocks(n);
  d.arena.reserve(&d.perm, n);
  d.arena.reserve(&d.inv, n);
  d.arena.reserve(&d.slot_rows, n);
  d.arena.reserve(&d.attr_ctr, 2);
  d.arena.reserve(&d.keys, n);
  d.arena.reserve(&d.keys_tmp, n);
  d.arena.reserve(&d.order, n);
  d.arena.reserve(&d.order_tmp, n);
  d.arena.reserve(&d.delta, n);
  d.arena.reserve(&d.perm_tmp, n);
  d.arena.reserve(&d.scratch, 3 * (std::size_t)n);
  d.arena.reserve(&d.radix.hist, 256 * (std::size_t)nb);
  d.arena.reserve(&d.radix.offs, 256 * (std::size_t)nb + 1);
  d.arena.reserve(&d.radix.scan_tmp, ceil_div(256LL * nb, 1024));
  d.arena.commit("t-SNE optimizer state");
  d.reordered = false;
  build_grid_classes(d, grids);
  std::vector<int2> blk(nblocks);
  for (int b = 0; b < ninst; ++b)
    for (int t = 0; t < d.inst[b].blocks; ++t)
      blk[d.inst[b].block_begin + t] = make_int2(b, d.inst[b].pt_begin + t * kPointBlock);
  FE_CUDA(cudaMemcpy(d.d_inst, d.inst.data(), sizeof(TsneInstance) * ninst, cudaMemcpyHostToDevice));
  FE_CUDA(cudaMemcpy(d.blocks, blk.data(), sizeof(int2) * nblocks, cudaMemcpyHostToDevice));
  FE_CUDA(cudaMemset(d.counter, 0, sizeof(unsigned) * ninst));
  FE_CUDA(cudaMemset(d.attr_ctr, 0, sizeof(unsigned) * 2));
  FE_CUDA(cudaMemset(d.cur, 0, sizeof(GridState) * ninst));
  if (!d.side) FE_CUDA(cudaStreamCreateWithFlags(&d.side, cudaStreamNonBlocking));
  if (!d.fork) FE_CUDA(cudaEventCreateWithFlags(&d.fork, cudaEventDisableTiming));
  if (!d.join) FE_CUDA(cudaEventCreateWithFlags(&d.join, cudaEventDisableTiming));
  // the synchronous setup above ran on the legacy stream, which the job's non-blocking streams
  // do not wait for
  FE_CUDA(cudaDeviceSynchronize());
}

void tsne_regrid(TsneDevice& d, const std::vector<int>& grids, cudaStream_t s) {
  if (grids.size() != d.inst.size()) throw Error("t-SNE regrid: one grid size per instance");
  FE_CUDA(cudaStreamSynchronize(s));
  build_grid_classes(d, grids);
  FE_CUDA(cudaMemcpy(d.d_inst, d.inst.data(), sizeof(TsneInstance) * d.inst.size(), cudaMemcpyHostToDevice));
  FE_CUDA(cudaDeviceSynchronize());
  // `next` of every instance was laid out for its old grid: recompute it from the layout
  layout_stats_kernel<<<d.nblocks, kStepThreads, 0, s>>>(d.y, d.d_inst, d.blocks, d.mode, d.partial, d.counter,
                                                          d.next);
  FE_LAUNCH("layout_stats_kernel");
}

std::vector<float> tsne_grid_extents(TsneDevice& d, cudaStream_t s) {
  std::vector<GridState> g(d.inst.size());
  FE_CUDA(cudaMemcpyAsync(g.data(), d.next, sizeof(GridState) * g.size(), cudaMemcpyDeviceToHost, s));
  FE_CUDA(cudaStreamSynchronize(s));
  std::vector<float> ext(g.size());
  for (std::size_t b = 0; b < g.size(); ++b) ext[b] = g[b].h * (float)(g[b].nodes - 1);
  return ext;
}

void tsne_device_init(TsneDevice& d, const float* d_init, cudaStream_t s) {
  FE_CUDA(cudaMemcpyAsync(d.y, d_init, sizeof(float2) * d.n, cudaMemcpyDeviceToDevice, s));
  identity_kernel<<<point_blocks(d.n), 256, 0, s>>>(d.perm, d.inv, d.n);
  FE_LAUNCH("identity_kernel");
  fill_state_kernel<<<point_blocks(d.n), 256, 0, s>>>(d.gains, d.update, d.n);
  FE_LAUNCH("fill_state_kernel");
  layout_stats_kernel<<<d.nblocks, kStepThreads, 0, s>>>(d.y, d.d_inst, d.blocks, d.mode, d.partial, d.counter,
                                                          d.next);
  FE_LAUNCH("layout_stats_kernel");
}

void tsne_grid_stage(TsneDevice& d, cudaStream_t s) {
  if (d.mode == kInterpBilinear)
    scatter_kernel<2><<<d.nblocks, kPointBlock, 0, s>>>(d.y, d.d_inst, d.blocks, d.cur, d.next);
  else
    scatter_kernel<3><<<d.nblocks, kPointBlock, 0, s>>>(d.y, d.d_inst, d.blocks, d.cur, d.next);
  FE_LAUNCH("scatter_kernel");
  for (const GridClass& c : d.classes) {
    const int m = c.fft;
    const int npairs = (c.nodes + 1) / 2;
    rows_forward_kernel<<<dim3(2 * npairs, c.count), kFftThreads, padded(3 * m) * sizeof(float2), s>>>(
        d.d_inst, c.members, c.grid, c.nodes, c.log_fft, c.twiddle, d.cur, c.arow, c.brow, c.krow);
    FE_LAUNCH("rows_forward_kernel");
    columns_convolve_kernel<<<dim3(c.col_blocks, c.count), kColThreads, padded(4 * m) * sizeof(float2), s>>>(
        c.arow, c.brow, c.krow, c.nodes, c.log_fft, c.twiddle, c.zpart);
    FE_LAUNCH("columns_convolve_kernel");
    rows_inverse_kernel<<<dim3(npairs, c.count), kFftThreads, padded(3 * m) * sizeof(float2), s>>>(
        c.arow, c.brow, d.d_inst, c.members, c.grid, c.nodes, c.log_fft, c.twiddle, c.zpart, c.col_blocks, d.cur);
    FE_LAUNCH("rows_inverse_kernel");
  }
}

void tsne_bind_rows(TsneDevice& d, const DeviceCsr& P, cudaStream_t s) {
  if (P.n != d.n) throw Error("t-SNE: P and the optimizer state have different sizes");
  bind_rows_kernel<<<point_blocks(d.n), 256, 0, s>>>(d.perm, P.row_ptr, d.n, d.slot_rows);
  FE_LAUNCH("bind_rows_kernel");
}

void tsne_attractive_stage(TsneDevice& d, const DeviceCsr& P, float exag, cudaStream_t s) {
  attractive_kernel<<<d.attr_blocks, kAttrThreads, 0, s>>>(d.slot_rows, P.col, P.val, d.y, d.n, exag, d.attr,
                                                           d.attr_ctr, d.attr_chunk);
  FE_LAUNCH("attractive_kernel");
}

// Run-time tuning of the attractive pass's launch: every (chunk, resident blocks per SM)
// candidate is launched once as warm-up and timed over `reps` launches with CUDA events on s, on
// the current layout (the pass only writes the attractive force, which the next iteration
// overwrites, so the optimizer state is untouched); the fastest is kept. Returns true when the
// choice changed (captured graphs hold the old launch).
bool tsne_tune_attractive(TsneDevice& d, const DeviceCsr& P, float exag, cudaStream_t s) {
  int per_sm = 0;
  FE_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, attractive_kernel, kAttrThreads, 0));
  per_sm = std::max(1, per_sm);
  const int chunks[] = {4, 8, 16};
  const int old_chunk = d.attr_chunk, old_blocks = d.attr_blocks;
  cudaEvent_t e0, e1;
  FE_CUDA(cudaEventCreate(&e0));
  FE_CUDA(cudaEventCreate(&e1));
  constexpr int reps = 2;
  float best = -1.0f;
  int best_chunk = old_chunk, best_blocks = old_blocks;
  d.tuning.clear();
  for (int per = per_sm; per >= std::max(1, per_sm - 1); --per) {
    const int blocks = std::max(1, std::min(per * sm_count(), ceil_div(d.n, kAttrThreads / 32)));
    for (int chunk : chunks) {
      d.attr_chunk = chunk;
      d.attr_blocks = blocks;
      tsne_attractive_stage(d, P, exag, s);
      FE_CUDA(cudaEventRecord(e0, s));
      for (int r = 0; r < reps; ++r) tsne_attractive_stage(d, P, exag, s);
      FE_CUDA(cudaEventRecord(e1, s));
      FE_CUDA(cudaEventSynchronize(e1));
      float ms = 0.0f;
      FE_CUDA(cudaEventElapsedTime(&ms, e0, e1));
      ms /= reps;
      d.tuning.push_back({chunk, blocks, ms});
      if (best < 0.0f || ms < best) {
        best = ms;
        best_chunk = chunk;
        best_blocks = blocks;
      }
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  d.attr_chunk = best_chunk;
  d.attr_blocks = best_blocks;
  d.tuned = true;
  return best_chunk != old_chunk || best_blocks != old_blocks;
}

void tsne_update_stage(TsneDevice& d, float lr, float mom, float min_gain, float max_step, cudaStream_t s) {
  if (d.mode == kInterpBilinear)
    update_kernel<2, false><<<d.nblocks, kStepThreads, 0, s>>>(d.y, d.attr, d.gains, d.update, d.d_inst, d.blocks,
                                                                d.cur, d.next, d.partial, d.counter, d.mode, lr, mom,
                                                                min_gain, max_step, nullptr);
  else
    update_kernel<3, false><<<d.nblocks, kStepThreads, 0, s>>>(d.y, d.attr, d.gains, d.update, d.d_inst, d.blocks,
                                                                d.cur, d.next, d.partial, d.counter, d.mode, lr, mom,
                                                                min_gain, max_step, nullptr);
  FE_LAUNCH("update_kernel");
}

void tsne_iteration(TsneDevice& d, const DeviceCsr& P, float exag, float lr, float mom, float min_gain,
                    float max_step, cudaStream_t s) {
  FE_CUDA(cudaEventRecord(d.fork, s));
  FE_CUDA(cudaStreamWaitEvent(d.side, d.fork, 0));
  tsne_attractive_stage(d, P, exag, d.side);
  FE_CUDA(cudaEventRecord(d.join, d.side));
  tsne_grid_stage(d, s);
  FE_CUDA(cudaStreamWaitEvent(s, d.join, 0));
  tsne_update_stage(d, lr, mom, min_gain, max_step, s);
}

void tsne_forces(TsneDevice& d, const DeviceCsr& P, float exag, float* d_attr, float* d_rep, cudaStream_t s) {
  tsne_attractive_stage(d, P, exag, s);
  tsne_grid_stage(d, s);
  FE_CUDA(cudaMemcpyAsync(d_attr, d.attr, sizeof(float2) * d.n, cudaMemcpyDeviceToDevice, s));
  float2* r = reinterpret_cast<float2*>(d_rep);
  if (d.mode == kInterpBilinear)
    update_kernel<2, true><<<d.nblocks, kStepThreads, 0, s>>>(d.y, d.attr, d.gains, d.update, d.d_inst, d.blocks,
                                                               d.cur, d.next, d.partial, d.counter, d.mode, 0.0f,
                                                               0.0f, 0.0f, 0.0f, r);
  else
    update_kernel<3, true><<<d.nblocks, kStepThreads, 0, s>>>(d.y, d.attr, d.gains, d.update, d.d_inst, d.blocks,
                                                               d.cur, d.next, d.partial, d.counter, d.mode, 0.0f,
                                                               0.0f, 0.0f, 0.0f, r);
  FE_LAUNCH("update_kernel(diagnostic)");
}

void tsne_finalize(TsneDevice& d, float* d_out, cudaStream_t s) {
  finalize_kernel<<<d.nblocks, kPointBlock, 0, s>>>(d.y, d.d_inst, d.blocks, d.next, d.perm,
                                                     reinterpret_cast<float2*>(d_out));
  FE_LAUNCH("finalize_kernel");
}

void tsne_reorder(TsneDevice& d, DeviceCsr& P, cudaStream_t s) {
  const int n = d.n;
  if (d.mode == kInterpBilinear)
    anchor_keys_kernel<2><<<d.nblocks, kPointBlock, 0, s>>>(d.y, d.d_inst, d.blocks, d.next, d.key_bits, d.keys,
                                                            d.order);
  else
    anchor_keys_kernel<3><<<d.nblocks, kPointBlock, 0, s>>>(d.y, d.d_inst, d.blocks, d.next, d.key_bits, d.keys,
                                                            d.order);
  FE_LAUNCH("anchor_keys_kernel");
  radix_sort_pairs(d.keys, d.order, d.keys_tmp, d.order_tmp, n, d.sort_bits, d.radix, s);
  gather_points_kernel<<<point_blocks(n), 256, 0, s>>>(d.order, n, d.y, d.gains, d.update, d.perm, d.scratch,
                                                       d.perm_tmp, d.delta);
  FE_LAUNCH("gather_points_kernel");
  scatter_points_kernel<<<point_blocks(n), 256, 0, s>>>(d.scratch, d.perm_tmp, n, P.row_ptr, d.y, d.gains, d.update,
                                                        d.perm, d.inv, d.slot_rows);
  FE_LAUNCH("scatter_points_kernel");
  relabel_cols_kernel<<<std::max(1, std::min(ceil_div(P.nnz, 256), sm_count() * 16)), 256, 0, s>>>(P.col, P.nnz,
                                                                                                   d.delta);
  FE_LAUNCH("relabel_cols_kernel");
  d.reordered = true;
}

int tsne_reorder_launches(const TsneDevice& d) {
  // keys, radix passes x (histogram + 3-kernel scan + scatter), gather, scatter, relabel
  return 1 + ceil_div(d.sort_bits, 8) * 5 + 3;
}

int tsne_launches_per_iteration(const TsneDevice& d) { return 3 + 3 * (int)d.classes.size(); }

}  // namespace fe
