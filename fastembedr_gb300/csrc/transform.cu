// Fixed-reference t-SNE transform on the GPU: places query points into an existing layout.
//
// Reference behaviour followed: transform_tsne_cpp (fastEmbedR src/tsne_neighbors.cpp:2124-2373)
// for two-dimensional layouts -
//   - query rows P by the FP64 min-shifted bisection of compute_row_probabilities_flat (:452-530);
//   - initialisation: supplied, median, inverse-distance weighted or random
//     (initialize_tsne_transform, :1384-1452);
//   - gradient of compute_tsne_transform_gradient_2d_flat (:1552-1648): exact repulsion against
//     the whole reference (n_ref <= threshold) or n_negatives references drawn from the per-query,
//     per-iteration xorshift32 stream seeded by mix_uint32((seed + 65537 (iter + 1)) ^
//     (query + 1) 0x9e3779b9), normalised by the query's own sum of q; attractive term over the
//     k neighbours;
//   - update of :2316-2347: gradient clip, gains (+0.2 / x0.8 + 0.01, floor 0.01), momentum,
//     step clip, y += update.
// This is the CUDA transform that R's transform_tsne(backend = "cuda") calls
// (R/transform_tsne.R:272-289), which the reference declares but never defines.
//
// Precision: pair terms, sums, gains and momentum in FP32; the layout is a two-float
// (compensated) value so 250 small steps keep their low bits; P in FP64, stored as FP32.
#include "transform.cuh"

#include <cfloat>
#include <climits>
#include <cmath>
#include <cstring>
#include <mutex>
#include <random>
#include <string>
#include <vector>

#include "../../include/fastembedr_cuda.h"

namespace fe {

// mix_uint32 / xorshift32 of src/tsne_neighbors.cpp:67-83
__host__ __device__ __forceinline__ std::uint32_t mix_u32(std::uint32_t v) {
  v ^= v >> 16u;
  v *= 0x7feb352du;
  v ^= v >> 15u;
  v *= 0x846ca68bu;
  v ^= v >> 16u;
  return v == 0u ? 0x6d2b79f5u : v;
}
__host__ __device__ __forceinline__ std::uint32_t xorshift32_step(std::uint32_t s) {
  s ^= s << 13u;
  s ^= s >> 17u;
  s ^= s << 5u;
  return s;
}

// ------------------------------------------------------------------ xorshift jump-ahead
namespace {
std::uint32_t gf2_apply_host(const std::uint32_t* m, std::uint32_t v) {
  std::uint32_t r = 0;
  for (int b = 0; b < 32; ++b)
    if ((v >> b) & 1u) r ^= m[b];
  return r;
}
void gf2_mul(const std::uint32_t* a, const std::uint32_t* b, std::uint32_t* out) {  // a after b
  std::uint32_t tmp[32];
  for (int c = 0; c < 32; ++c) tmp[c] = gf2_apply_host(a, b[c]);
  std::memcpy(out, tmp, sizeof(tmp));
}
void gf2_power(long long n, std::uint32_t* out) {
  std::uint32_t p[32], r[32];
  for (int b = 0; b < 32; ++b) {
    p[b] = xorshift32_step(1u << b);
    r[b] = 1u << b;
  }
  while (n > 0) {
    if (n & 1) gf2_mul(p, r, r);
    gf2_mul(p, p, p);
    n >>= 1;
  }
  std::memcpy(out, r, sizeof(r));
}
}  // namespace

XorshiftJump xorshift_jump_table(int n_negatives) {
  XorshiftJump t;
  for (int lane = 0; lane < 32; ++lane) gf2_power((long long)lane * n_negatives / 32, t.col[lane]);
  return t;
}

std::size_t transform_query_bytes(int k) {
  return (std::size_t)k * (sizeof(float2) + sizeof(float)) + 2 * sizeof(float4) + 2 * sizeof(double) + 64;
}

// ------------------------------------------------------------------ kernels
__device__ __forceinline__ int find_segment(const TransformSegment* segs, int nseg, long long q) {
  int lo = 0, hi = nseg - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (segs[mid].query_begin <= q) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

__device__ __forceinline__ double seg_dist(const TransformSegment& sg, int j, int i) {
  const long long pos = (long long)j * sg.nq + i;
  return sg.dist_f ? (double)sg.dist_f[pos] : sg.dist_d[pos];
}

__global__ void transform_reference_kernel(const double* __restrict__ ref_cm, int n_ref, float2* __restrict__ ref,
                                           double2* __restrict__ ref_d) {
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n_ref; r += gridDim.x * blockDim.x) {
    const double x = ref_cm[r], y = ref_cm[(long long)n_ref + r];
    ref[r] = make_float2((float)x, (float)y);
    ref_d[r] = make_double2(x, y);
  }
}

// Warp per query: FP64 bisection of compute_row_probabilities_flat, P stored as FP32 [query][k].
__global__ void transform_row_p_kernel(const TransformSegment* __restrict__ segs, int nseg, long long total_q,
                                       double perplexity) {
  const int lane = threadIdx.x & 31;
  const long long q = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (q >= total_q) return;
  const TransformSegment& sg = segs[find_segment(segs, nseg, q)];
  const int i = (int)(q - sg.query_begin), k = sg.k;
  float* prow = sg.p + (long long)i * k;
  double mn = DBL_MAX, mx = 0.0;
  for (int j = lane; j < k; j += 32) {
    const double d = seg_dist(sg, j, i);
    mn = fmin(mn, d * d);
    mx = fmax(mx, d * d);
  }
  mn = warp_min(mn);
  mx = warp_max(mx);
  if (mx - mn <= DBL_EPSILON * fmax(1.0, mx)) {
    for (int j = lane; j < k; j += 32) prow[j] = (float)(1.0 / (double)k);
    return;
  }
  const double target = log(perplexity);
  double beta = 1.0, bmin = -DBL_MAX, bmax = DBL_MAX, beta_eval = 1.0, sum_p = DBL_MIN;
  for (int it = 0; it < 200; ++it) {
    double sp = 0.0, ent = 0.0;
    for (int j = lane; j < k; j += 32) {
      const double d = seg_dist(sg, j, i);
      const double s = d * d - mn;
      const double pv = exp(-beta * s);
      sp += pv;
      ent += beta * (s * pv);
    }
    sp = warp_sum(sp);
    ent = warp_sum(ent);
    beta_eval = beta;
    sum_p = DBL_MIN + sp;
    const double diff = ent / sum_p + log(sum_p) - target;
    if (fabs(diff) < 1e-5) break;
    if (diff > 0.0) {
      bmin = beta;
      beta = (bmax == DBL_MAX || bmax == -DBL_MAX) ? beta * 2.0 : (beta + bmax) / 2.0;
    } else {
      bmax = beta;
      beta = (bmin == -DBL_MAX || bmin == DBL_MAX) ? beta / 2.0 : (beta + bmin) / 2.0;
    }
    if (!isfinite(beta)) break;
  }
  if (!isfinite(sum_p) || sum_p <= DBL_MIN) {
    // every term underflowed: uniform over the neighbours tied at the minimum distance
    const double tol = DBL_EPSILON * fmax(1.0, mn);
    double tied = 0.0;
    for (int j = lane; j < k; j += 32) {
      const double d = seg_dist(sg, j, i);
      tied += fabs(d * d - mn) <= tol ? 1.0 : 0.0;
    }
    tied = fmax(warp_sum(tied), 1.0);
    for (int j = lane; j < k; j += 32) {
      const double d = seg_dist(sg, j, i);
      prow[j] = fabs(d * d - mn) <= tol ? (float)(1.0 / tied) : 0.0f;
    }
    return;
  }
  const double inv = 1.0 / sum_p;
  for (int j = lane; j < k; j += 32) {
    const double d = seg_dist(sg, j, i);
    prow[j] = (float)(exp(-beta_eval * (d * d - mn)) * inv);
  }
}

// Warp per query: neighbour coordinates, initial layout and optimizer state.
// init_mode 0 = supplied y_init, 1 = median, 2 = inverse-distance weighted; a segment that
// carries y_init uses it whatever the mode.
__global__ void transform_init_kernel(const float2* __restrict__ ref, const double2* __restrict__ ref_d,
                                      const TransformSegment* __restrict__ segs, int nseg, long long total_q,
                                      int init_mode) {
  const int lane = threadIdx.x & 31;
  const long long q = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (q >= total_q) return;
  const TransformSegment& sg = segs[find_segment(segs, nseg, q)];
  const int i = (int)(q - sg.query_begin), k = sg.k, nq = sg.nq;
  float2* nrow = sg.nb + (long long)i * k;
  for (int j = lane; j < k; j += 32) nrow[j] = ref[sg.idx[(long long)j * nq + i] - sg.offset];
  double y[2];
  if (sg.y_init) {
    y[0] = sg.y_init[i];
    y[1] = sg.y_init[(long long)nq + i];
  } else if (init_mode == 2) {
    double nx = 0.0, ny = 0.0, den = 0.0;
    for (int j = lane; j < k; j += 32) {
      const double2 r = ref_d[sg.idx[(long long)j * nq + i] - sg.offset];
      const double w = 1.0 / (fmax(0.0, seg_dist(sg, j, i)) + 1e-6);
      nx += w * r.x;
      ny += w * r.y;
      den += w;
    }
    den = DBL_MIN + warp_sum(den);
    y[0] = warp_sum(nx) / den;
    y[1] = warp_sum(ny) / den;
  } else {
    // median per dimension: the values of rank k/2 (and k/2 - 1 for even k), by counting ranks
    const int mid = k / 2;
    for (int d = 0; d < 2; ++d) {
      double hi_v = -DBL_MAX, lo_v = -DBL_MAX;
      for (int j = lane; j < k; j += 32) {
        const double2 rv = ref_d[sg.idx[(long long)j * nq + i] - sg.offset];
        const double v = d ? rv.y : rv.x;
        int less = 0, equal = 0;
        for (int u = 0; u < k; ++u) {
          const double2 ru = ref_d[sg.idx[(long long)u * nq + i] - sg.offset];
          const double w = d ? ru.y : ru.x;
          less += w < v;
          equal += w == v;
        }
        if (less <= mid && mid < less + equal) hi_v = v;
        if (less <= mid - 1 && mid - 1 < less + equal) lo_v = v;
      }
      hi_v = warp_max(hi_v);
      lo_v = warp_max(lo_v);
      y[d] = (k & 1) ? hi_v : 0.5 * (hi_v + lo_v);
    }
  }
  if (lane == 0) {
    const float hx = (float)y[0], hy = (float)y[1];
    sg.state[i] = make_float4(hx, hy, (float)(y[0] - (double)hx), (float)(y[1] - (double)hy));
    sg.opt[i] = make_float4(1.0f, 1.0f, 0.0f, 0.0f);
  }
}

__device__ __forceinline__ std::uint32_t gf2_apply(const std::uint32_t (*cols)[32], int lane, std::uint32_t v) {
  std::uint32_t r = 0;
#pragma unroll
  for (int b = 0; b < 32; ++b) r ^= ((v >> b) & 1u) ? cols[b][lane] : 0u;
  return r;
}

__device__ __forceinline__ void two_sum_add(float& hi, float& lo, float u) {
  const float s = __fadd_rn(hi, u);
  const float bp = __fsub_rn(s, hi);
  const float err = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bp)), __fsub_rn(u, bp));
  const float l = __fadd_rn(lo, err);
  const float t = __fadd_rn(s, l);
  lo = __fsub_rn(l, __fsub_rn(t, s));
  hi = t;
}

__device__ __forceinline__ float sign_f(float v) { return v == 0.0f ? 0.0f : (v < 0.0f ? -1.0f : 1.0f); }

// One repulsion pair: q, q^2 (y - r) with the compensated query position.
__device__ __forceinline__ void repulse(float2 rr, float yhx, float yhy, float ylx, float yly, float& fz, float& fx,
                                        float& fy) {
  const float dx = (yhx - rr.x) + ylx, dy = (yhy - rr.y) + yly;
  const float qv = __frcp_rn(1.0f + dx * dx + dy * dy);
  const float q2 = qv * qv;
  fz += qv;
  fx += q2 * dx;
  fy += q2 * dy;
}

// MODE 0: sampled repulsion; 1: exact, whole reference staged in shared memory once;
// 2: exact, reference streamed through shared memory in tiles every iteration.
constexpr int kTransformWarps = 8;
constexpr int kTransformTile = 4096;

template <int MODE>
__global__ void __launch_bounds__(kTransformWarps * 32)
transform_iterate_kernel(const float2* __restrict__ ref, const TransformSegment* __restrict__ segs, int nseg,
                         long long total_q, TransformParams tp, const XorshiftJump* __restrict__ jump, int it_begin,
                         int it_end) {
  extern __shared__ float2 sref[];
  __shared__ std::uint32_t sjump[32][32];  // [bit][lane]
  const int lane = threadIdx.x & 31;
  const long long q = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const bool active = q < total_q;
  if (MODE == 0) {
    for (int t = threadIdx.x; t < 32 * 32; t += blockDim.x) sjump[t & 31][t >> 5] = jump->col[t >> 5][t & 31];
    __syncthreads();
  } else if (MODE == 1) {
    for (int t = threadIdx.x; t < tp.n_ref; t += blockDim.x) sref[t] = ref[t];
    __syncthreads();
  }
  // MODE 2 keeps inactive warps alive: they take part in every tile's barriers.
  if (MODE != 2 && !active) return;
  const TransformSegment* sgp = &segs[active ? find_segment(segs, nseg, q) : 0];
  const int i = active ? (int)(q - sgp->query_begin) : 0;
  const int k = active ? sgp->k : 0;
  const float2* nrow = sgp->nb + (long long)i * sgp->k;
  const float* prow = sgp->p + (long long)i * sgp->k;
  const float4 st = active ? sgp->state[i] : make_float4(0.f, 0.f, 0.f, 0.f);
  const float4 op = active ? sgp->opt[i] : make_float4(1.f, 1.f, 0.f, 0.f);
  float yhx = st.x, yhy = st.y, ylx = st.z, yly = st.w;
  float gnx = op.x, gny = op.y, upx = op.z, upy = op.w;
  const int s_begin = (int)(((long long)lane * tp.n_negatives) >> 5);
  const int s_end = (int)(((long long)(lane + 1) * tp.n_negatives) >> 5);
  const std::uint32_t salt = (std::uint32_t)(i + 1) * 0x9e3779b9u;
  for (int it = it_begin; it < it_end; ++it) {
    const bool early = it < tp.early_iter;
    const float exg = early ? tp.early_exag : tp.exag;
    const float mom = early ? tp.m0 : tp.m1;
    float fz = 0.0f, fx = 0.0f, fy = 0.0f;
    if (MODE == 0 && tp.hash_sampler) {
      // landmark_reference_sample of the reference's landmark transform
      // (src/embedding_cuda_kernels.cpp:511-521): an independent hash per sample
      const std::uint32_t base = (std::uint32_t)tp.seed ^ ((std::uint32_t)(it + 1) * 0x9e3779b9u) ^
                                 ((std::uint32_t)(i + 1) * 0x85ebca6bu);
#pragma unroll 4
      for (int m = lane; m < tp.n_negatives; m += 32) {
        std::uint32_t x = base ^ ((std::uint32_t)(m + 1) * 0xc2b2ae35u);
        x ^= x >> 16u;
        x *= 0x7feb352du;
        x ^= x >> 15u;
        x *= 0x846ca68bu;
        x ^= x >> 16u;
        repulse(__ldg(&ref[x % (std::uint32_t)tp.n_ref]), yhx, yhy, ylx, yly, fz, fx, fy);
      }
    } else if (MODE == 0) {
      const std::uint32_t iter_seed = (std::uint32_t)tp.seed + 65537u * (std::uint32_t)(it + 1);
      std::uint32_t s = gf2_apply(sjump, lane, mix_u32(iter_seed ^ salt));
#pragma unroll 4
      for (int m = s_begin; m < s_end; ++m) {
        s = xorshift32_step(s);
        const int r = (int)(((unsigned long long)s * (unsigned long long)tp.n_ref) >> 32);
        repulse(__ldg(&ref[r]), yhx, yhy, ylx, yly, fz, fx, fy);
      }
    } else if (MODE == 1) {
      for (int t = lane; t < tp.n_ref; t += 32) repulse(sref[t], yhx, yhy, ylx, yly, fz, fx, fy);
    } else {
      for (int t0 = 0; t0 < tp.n_ref; t0 += kTransformTile) {
        const int cnt = min(kTransformTile, tp.n_ref - t0);
        __syncthreads();
        for (int t = threadIdx.x; t < cnt; t += blockDim.x) sref[t] = ref[t0 + t];
        __syncthreads();
        for (int t = lane; t < cnt; t += 32) repulse(sref[t], yhx, yhy, ylx, yly, fz, fx, fy);
      }
    }
    float ax = 0.0f, ay = 0.0f;
    for (int j = lane; j < k; j += 32) {
      const float2 nb = nrow[j];
      const float pj = prow[j];
      const float dx = (yhx - nb.x) + ylx, dy = (yhy - nb.y) + yly;
      const float c = pj * __frcp_rn(1.0f + dx * dx + dy * dy);
      ax += c * dx;
      ay += c * dy;
    }
    fz = warp_sum(fz);
    fx = warp_sum(fx);
    fy = warp_sum(fy);
    ax = warp_sum(ax);
    ay = warp_sum(ay);
    const float zq = fmaxf(fz, FLT_MIN);
    float gx = exg * ax - fx / zq;
    float gy = exg * ay - fy / zq;
    const float g2 = gx * gx + gy * gy;
    if (g2 > tp.max_grad * tp.max_grad) {
      const float sc = tp.max_grad / (sqrtf(g2) + 1e-12f);
      gx *= sc;
      gy *= sc;
    }
    gnx = sign_f(upx) != sign_f(gx) ? gnx + 0.2f : gnx * 0.8f + 0.01f;
    gny = sign_f(upy) != sign_f(gy) ? gny + 0.2f : gny * 0.8f + 0.01f;
    gnx = fmaxf(gnx, 0.01f);
    gny = fmaxf(gny, 0.01f);
    upx = mom * upx - tp.lr * gnx * gx;
    upy = mom * upy - tp.lr * gny * gy;
    const float s2 = upx * upx + upy * upy;
    if (s2 > tp.max_step * tp.max_step) {
      const float sc = tp.max_step / (sqrtf(s2) + 1e-12f);
      upx *= sc;
      upy *= sc;
    }
    two_sum_add(yhx, ylx, upx);
    two_sum_add(yhy, yly, upy);
  }
  if (!active || lane != 0) return;
  if (it_end >= tp.iter_total) {
    sgp->out[i] = (double)yhx + (double)ylx;
    sgp->out[(long long)sgp->nq + i] = (double)yhy + (double)yly;
  } else {
    sgp->state[i] = make_float4(yhx, yhy, ylx, yly);
    sgp->opt[i] = make_float4(gnx, gny, upx, upy);
  }
}

// ------------------------------------------------------------------ host launchers
void transform_prepare(const float2* ref, const double2* ref_d, const TransformSegment* segs, int nseg,
                       long long total_q, const TransformParams& tp, cudaStream_t s) {
  const int blocks = ceil_div(total_q * 32, 256);
  transform_row_p_kernel<<<blocks, 256, 0, s>>>(segs, nseg, total_q, tp.perplexity);
  FE_LAUNCH("transform_row_p_kernel");
  transform_init_kernel<<<blocks, 256, 0, s>>>(ref, ref_d, segs, nseg, total_q, tp.init_mode);
  FE_LAUNCH("transform_init_kernel");
}

void transform_iterate(const float2* ref, const TransformSegment* segs, int nseg, long long total_q,
                       const TransformParams& tp, const XorshiftJump* jump, int it_begin, int it_end,
                       cudaStream_t s) {
  static std::once_flag attr_once;
  std::call_once(attr_once, [] {
    cudaFuncSetAttribute(transform_iterate_kernel<1>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)(kTransformSmemRefs * sizeof(float2)));
  });
  const int blocks = ceil_div(total_q, kTransformWarps);
  const int threads = kTransformWarps * 32;
  if (!tp.exact) {
    transform_iterate_kernel<0><<<blocks, threads, 0, s>>>(ref, segs, nseg, total_q, tp, jump, it_begin, it_end);
  } else if (tp.n_ref <= kTransformSmemRefs) {
    transform_iterate_kernel<1><<<blocks, threads, tp.n_ref * sizeof(float2), s>>>(ref, segs, nseg, total_q, tp,
                                                                                   jump, it_begin, it_end);
  } else {
    transform_iterate_kernel<2><<<blocks, threads, kTransformTile * sizeof(float2), s>>>(ref, segs, nseg, total_q,
                                                                                        tp, jump, it_begin, it_end);
  }
  FE_LAUNCH("transform_iterate_kernel");
}

}  // namespace fe

namespace fe {

TransformParams transform_params(int n_ref, int n_negatives, int exact_repulsion_threshold, double perplexity,
                                 int n_iter, int early_iter, double learning_rate, double early_exaggeration,
                                 double exaggeration, double initial_momentum, double final_momentum,
                                 double max_grad_norm, double max_step_norm, int init_mode, int seed) {
  if (n_ref < 1) throw Error("`reference_layout` must be a non-empty matrix.");
  if (!(perplexity > 0.0) || !std::isfinite(perplexity)) throw Error("`perplexity` must be a positive number.");
  if (n_iter < 0 || early_iter < 0 || n_iter + early_iter < 1)
    throw Error("Transform iteration counts must be non-negative and sum to at least one.");
  if (n_negatives < 1) throw Error("`n_negatives` must be NULL or a positive integer.");
  if (exact_repulsion_threshold < 1) exact_repulsion_threshold = 1;
  if (n_negatives > n_ref) n_negatives = n_ref;
  TransformParams tp;
  tp.n_ref = n_ref;
  tp.exact = (n_ref <= exact_repulsion_threshold || n_negatives >= n_ref) ? 1 : 0;
  tp.n_negatives = n_negatives;
  tp.iter_total = n_iter + early_iter;
  tp.early_iter = early_iter;
  tp.init_mode = init_mode;
  tp.seed = seed == INT_MIN ? 5489 : seed;  // R's NA_integer_
  tp.perplexity = perplexity;
  tp.lr = (float)learning_rate;
  tp.early_exag = (float)early_exaggeration;
  tp.exag = (float)exaggeration;
  tp.m0 = (float)initial_momentum;
  tp.m1 = (float)final_momentum;
  tp.max_grad = (max_grad_norm > 0.0 && std::isfinite(max_grad_norm)) ? (float)max_grad_norm : INFINITY;
  tp.max_step = (max_step_norm > 0.0 && std::isfinite(max_step_norm)) ? (float)max_step_norm : INFINITY;
  return tp;
}

// initialize_tsne_transform's "random" start (src/tsne_neighbors.cpp:1398-1413): per query a
// std::mt19937 seeded with mix_uint32(seed ^ (query + 1) 0x9e3779b9) and two draws of
// N(0, 1e-4^2). Two draws per query consume exactly one polar pair, so a fresh distribution per
// query gives the reference's values. Host work of n_query x 2 draws; column-major output.
void transform_random_init(int seed, int query_begin, int n_query, double* out) {
  for (int i = 0; i < n_query; ++i) {
    std::normal_distribution<double> normal(0.0, 1.0e-4);
    std::mt19937 rng(mix_u32((std::uint32_t)seed ^ ((std::uint32_t)(query_begin + i + 1) * 0x9e3779b9u)));
    out[i] = normal(rng);
    out[(std::size_t)n_query + i] = normal(rng);
  }
}

void transform_upload_reference(const double* d_ref_cm, int n_ref, float2* ref, double2* ref_d, cudaStream_t s) {
  const int rb = std::max(1, std::min(ceil_div(n_ref, 256), sm_count() * 8));
  transform_reference_kernel<<<rb, 256, 0, s>>>(d_ref_cm, n_ref, ref, ref_d);
  FE_LAUNCH("transform_reference_kernel");
}

// Iterations per launch: at most ~4e10 pair evaluations, so no launch runs for long.
int transform_chunk(long long n_query, const TransformParams& tp, int k) {
  const double per_iter = (double)n_query * ((tp.exact ? tp.n_ref : tp.n_negatives) + k);
  const double c = 4.0e10 / std::max(per_iter, 1.0);
  return (int)std::max(1.0, std::min((double)tp.iter_total, c));
}

}  // namespace fe

extern "C" int fastembedr_cuda_transform_tsne(const double* reference_layout, int n_reference, const int* indices,
                                              const double* distances, int n_query, int k, const double* y_init,
                                              int init, const char* initialization, double perplexity, int n_iter,
                                              int early_exaggeration_iter, double learning_rate,
                                              double early_exaggeration, double exaggeration, double initial_momentum,
                                              double final_momentum, double max_grad_norm, double max_step_norm,
                                              int n_negatives, int exact_repulsion_threshold, int seed, double* out) {
  return fe::guarded([&] {
    if (!reference_layout || !indices || !distances || !out || (init && !y_init))
      throw fe::Error("null CUDA t-SNE transform pointer");
    if (n_query < 1 || k < 1) throw fe::Error("`knn` must have at least one row and one neighbor column.");
    const std::string ini = initialization ? initialization : "median";
    if (ini != "median" && ini != "weighted" && ini != "random")
      throw fe::Error("`initialization` must be 'median', 'weighted', or 'random'.");
    const int mode = init ? 0 : (ini == "median" ? 1 : (ini == "weighted" ? 2 : 3));
    fe::TransformParams tp = fe::transform_params(
        n_reference, n_negatives, exact_repulsion_threshold, perplexity, n_iter, early_exaggeration_iter,
        learning_rate, early_exaggeration, exaggeration, initial_momentum, final_momentum, max_grad_norm,
        max_step_norm, mode == 3 ? 0 : mode, seed);
    // resolve_reference_index_offset and the range checks of src/tsne_neighbors.cpp:1371-1382, :2175-2185
    const long long items = (long long)n_query * k;
    int lo = INT_MAX, hi = INT_MIN;
    for (long long t = 0; t < items; ++t) {
      lo = std::min(lo, indices[t]);
      hi = std::max(hi, indices[t]);
    }
    const int offset = (lo >= 1 && hi <= n_reference) ? 1 : 0;
    for (long long t = 0; t < items; ++t) {
      const int r = indices[t] - offset;
      if (r < 0 || r >= n_reference) throw fe::Error("KNN indices are out of range for `reference_layout`.");
      if (!std::isfinite(distances[t]) || distances[t] < 0.0)
        throw fe::Error("KNN distances must be finite and non-negative.");
    }
    std::vector<double> random_init;
    if (mode == 3) {
      random_init.resize(2 * (std::size_t)n_query);
      fe::transform_random_init(tp.seed, 0, n_query, random_init.data());
      y_init = random_init.data();
    }
    const bool have_init = mode == 0 || mode == 3;
    fe::Stream st;
    cudaStream_t s = st.s;
    double *d_ref_cm = nullptr, *d_dist = nullptr, *d_init = nullptr, *d_out = nullptr;
    int* d_idx = nullptr;
    float2* d_ref = nullptr;
    double2* d_ref_d = nullptr;
    float2* d_nb = nullptr;
    float* d_p = nullptr;
    float4 *d_state = nullptr, *d_opt = nullptr;
    fe::TransformSegment* d_seg = nullptr;
    fe::XorshiftJump* d_jump = nullptr;
    fe::Arena a;
    a.reserve(&d_ref_cm, 2 * (std::size_t)n_reference);
    a.reserve(&d_ref, n_reference);
    a.reserve(&d_ref_d, n_reference);
    a.reserve(&d_idx, items);
    a.reserve(&d_dist, items);
    if (have_init) a.reserve(&d_init, 2 * (std::size_t)n_query);
    a.reserve(&d_nb, items);
    a.reserve(&d_p, items);
    a.reserve(&d_state, n_query);
    a.reserve(&d_opt, n_query);
    a.reserve(&d_out, 2 * (std::size_t)n_query);
    a.reserve(&d_seg, 1);
    a.reserve(&d_jump, 1);
    a.commit("CUDA t-SNE transform");
    FE_CUDA(cudaMemcpyAsync(d_ref_cm, reference_layout, sizeof(double) * 2 * n_reference, cudaMemcpyHostToDevice, s));
    fe::upload(d_idx, indices, sizeof(int) * items, s);
    fe::upload(d_dist, distances, sizeof(double) * items, s);
    if (have_init)
      FE_CUDA(cudaMemcpyAsync(d_init, y_init, sizeof(double) * 2 * n_query, cudaMemcpyHostToDevice, s));
    fe::TransformSegment seg{d_idx, nullptr, d_dist, have_init ? d_init : nullptr, d_nb, d_p, d_state, d_opt,
                             d_out, 0, n_query, k, offset};
    FE_CUDA(cudaMemcpyAsync(d_seg, &seg, sizeof(seg), cudaMemcpyHostToDevice, s));
    const fe::XorshiftJump jump = fe::xorshift_jump_table(tp.n_negatives);
    FE_CUDA(cudaMemcpyAsync(d_jump, &jump, sizeof(jump), cudaMemcpyHostToDevice, s));
    fe::transform_upload_reference(d_ref_cm, n_reference, d_ref, d_ref_d, s);
    fe::transform_prepare(d_ref, d_ref_d, d_seg, 1, n_query, tp, s);
    const int chunk = fe::transform_chunk(n_query, tp, k);
    for (int it = 0; it < tp.iter_total; it += chunk)
      fe::transform_iterate(d_ref, d_seg, 1, n_query, tp, d_jump, it, std::min(tp.iter_total, it + chunk), s);
    FE_CUDA(cudaMemcpyAsync(out, d_out, sizeof(double) * 2 * n_query, cudaMemcpyDeviceToHost, s));
    FE_CUDA(cudaStreamSynchronize(s));
  });
}
