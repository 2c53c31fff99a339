// Fixed-reference t-SNE transform on the GPU: places query points into an existing layout.
//
// Reference behaviour followed: transform_tsne_cpp (fastEmbedR src/tsne_neighbors.cpp:2124-2373)
// for two-dimensional layouts -
//   - query rows P by the FP64 min-shifted bisection of compute_row_probabilities_flat (:452-530);
//   - initialisation: supplied, median or inverse-distance weighted reference coordinates of the
//     k neighbours (initialize_tsne_transform, :1384-1452);
//   - gradient of compute_tsne_transform_gradient_2d_flat (:1552-1648): exact repulsion against
//     the whole reference (n_ref <= threshold) or n_negatives references drawn from the per-query,
//     per-iteration xorshift32 stream seeded by mix_uint32(seed + 65537 (iter + 1), query), each
//     normalised by its own sum of q; attractive term over the k neighbours;
//   - update of :2316-2347: gradient clip, gains (+0.2 / x0.8 + 0.01, floor 0.01), momentum,
//     step clip, y += update.
// This is the CUDA transform that R's transform_tsne(backend = "cuda") calls
// (R/transform_tsne.R:272-289), which the reference declares but never defines.
// Pair terms are FP32; per-query sums are FP64. Exact mode stages the reference layout through
// shared memory; sampled mode reproduces the reference's sample sequence exactly.
#include <cfloat>
#include <climits>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <random>
#include <string>
#include <vector>

#include "../../include/fastembedr_cuda.h"
#include "tsne.cuh"

namespace fe {

__device__ __forceinline__ unsigned mix_u32(unsigned v) {
  v ^= v >> 16u;
  v *= 0x7feb352du;
  v ^= v >> 15u;
  v *= 0x846ca68bu;
  v ^= v >> 16u;
  return v == 0u ? 0x6d2b79f5u : v;
}
__device__ __forceinline__ unsigned xorshift32(unsigned& s) {
  s ^= s << 13u;
  s ^= s >> 17u;
  s ^= s << 5u;
  return s;
}

// Warp per query row: FP64 bisection of compute_row_probabilities_flat. The row's distances are
// column-major (query-major within a neighbour column), as R stores an n_query x k matrix.
__global__ void transform_row_p_kernel(const double* __restrict__ dist, int nq, int k, double perplexity,
                                       double* __restrict__ p) {
  const int lane = threadIdx.x & 31;
  const int row = (int)(((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  if (row >= nq) return;
  double mn = DBL_MAX, mx = 0.0;
  for (int j = lane; j < k; j += 32) {
    const double d = dist[(long long)j * nq + row];
    mn = fmin(mn, d * d);
    mx = fmax(mx, d * d);
  }
  mn = warp_min(mn);
  mx = warp_max(mx);
  double* prow = p + (long long)row * k;
  if (mx - mn <= DBL_EPSILON * fmax(1.0, mx)) {
    for (int j = lane; j < k; j += 32) prow[j] = 1.0 / (double)k;
    return;
  }
  const double target = log(perplexity);
  double beta = 1.0, bmin = -DBL_MAX, bmax = DBL_MAX;
  double beta_eval = beta, sum_p = DBL_MIN;
  for (int it = 0; it < 200; ++it) {
    double sp = 0.0, ent = 0.0;
    for (int j = lane; j < k; j += 32) {
      const double d = dist[(long long)j * nq + row];
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
    // every term underflowed: uniform over the rows tied at the minimum distance
    const double tol = DBL_EPSILON * fmax(1.0, mn);
    int tied = 0;
    for (int j = lane; j < k; j += 32) {
      const double d = dist[(long long)j * nq + row];
      tied += fabs(d * d - mn) <= tol;
    }
    tied = (int)warp_sum((double)tied);
    for (int j = lane; j < k; j += 32) {
      const double d = dist[(long long)j * nq + row];
      prow[j] = fabs(d * d - mn) <= tol ? 1.0 / (double)max(tied, 1) : 0.0;
    }
    return;
  }
  const double inv = 1.0 / sum_p;
  for (int j = lane; j < k; j += 32) {
    const double d = dist[(long long)j * nq + row];
    prow[j] = exp(-beta_eval * (d * d - mn)) * inv;
  }
}

// Initial query layout: 1 = median, 2 = inverse-distance weighted (per dimension).
__global__ void transform_init_kernel(const double* __restrict__ ref, int nref, const int* __restrict__ idx,
                                      const double* __restrict__ dist, int nq, int k, int offset, int mode,
                                      double2* __restrict__ y) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nq) return;
  double out[2];
  for (int d = 0; d < 2; ++d) {
    if (mode == 2) {
      double num = 0.0, den = DBL_MIN;
      for (int j = 0; j < k; ++j) {
        const int r = idx[(long long)j * nq + i] - offset;
        const double w = 1.0 / (fmax(0.0, dist[(long long)j * nq + i]) + 1e-6);
        num += w * ref[(long long)d * nref + r];
        den += w;
      }
      out[d] = num / den;
    } else {
      // median by counting ranks (k <= 1024): the element whose rank covers k/2 (and k/2 - 1)
      const int mid = k / 2;
      double lo_v = 0.0, hi_v = 0.0;
      for (int j = 0; j < k; ++j) {
        const double v = ref[(long long)d * nref + (idx[(long long)j * nq + i] - offset)];
        int less = 0, equal = 0;
        for (int u = 0; u < k; ++u) {
          const double w = ref[(long long)d * nref + (idx[(long long)u * nq + i] - offset)];
          less += w < v;
          equal += w == v;
        }
        if (less <= mid && mid < less + equal) hi_v = v;
        if (less <= mid - 1 && mid - 1 < less + equal) lo_v = v;
      }
      out[d] = (k & 1) ? hi_v : 0.5 * (hi_v + lo_v);
    }
  }
  y[i] = make_double2(out[0], out[1]);
}

struct TransformParams {
  int nref, nq, k, offset, n_negatives, exact;
  double lr, max_grad, max_step;
};

// One thread per query, one iteration. Exact mode stages the reference layout through shared
// memory in tiles; the attractive term reads the k neighbours from the L2-resident layout.
constexpr int kTransformThreads = 128;
constexpr int kRefTile = 2048;

__global__ void __launch_bounds__(kTransformThreads)
transform_iteration_kernel(const float2* __restrict__ ref, const int* __restrict__ idx, const double* __restrict__ P,
                           double2* __restrict__ y, double2* __restrict__ gains, double2* __restrict__ upd,
                           TransformParams tp, double exag, double mom, int iter_seed) {
  __shared__ float2 tile[kRefTile];
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const bool active = i < tp.nq;
  const double2 yi = active ? y[i] : make_double2(0.0, 0.0);
  const float yx = (float)yi.x, yy = (float)yi.y;
  double sum_q = DBL_MIN, gx = 0.0, gy = 0.0;
  if (tp.exact) {
    double rx = 0.0, ry = 0.0;
    for (int t0 = 0; t0 < tp.nref; t0 += kRefTile) {
      const int cnt = min(kRefTile, tp.nref - t0);
      __syncthreads();
      for (int t = threadIdx.x; t < cnt; t += blockDim.x) tile[t] = ref[t0 + t];
      __syncthreads();
      if (active) {
        float fz = 0.0f, fx = 0.0f, fy = 0.0f;
        for (int t = 0; t < cnt; ++t) {
          const float dx = yx - tile[t].x, dy = yy - tile[t].y;
          const float q = 1.0f / (1.0f + dx * dx + dy * dy);
          fz += q;
          fx += q * q * dx;
          fy += q * q * dy;
        }
        sum_q += fz;
        rx += fx;
        ry += fy;
      }
    }
    gx = -rx / sum_q;
    gy = -ry / sum_q;
  } else if (active) {
    unsigned state = mix_u32((unsigned)iter_seed ^ ((unsigned)(i + 1) * 0x9e3779b9u));
    const unsigned state0 = state;
    for (int m = 0; m < tp.n_negatives; ++m) {
      const int r = (int)(((unsigned long long)xorshift32(state) * (unsigned long long)tp.nref) >> 32);
      const float2 rr = ref[r];
      const float dx = yx - rr.x, dy = yy - rr.y;
      sum_q += (double)(1.0f / (1.0f + dx * dx + dy * dy));
    }
    state = state0;
    double rx = 0.0, ry = 0.0;
    for (int m = 0; m < tp.n_negatives; ++m) {
      const int r = (int)(((unsigned long long)xorshift32(state) * (unsigned long long)tp.nref) >> 32);
      const float2 rr = ref[r];
      const float dx = yx - rr.x, dy = yy - rr.y;
      const float q = 1.0f / (1.0f + dx * dx + dy * dy);
      rx += (double)(q * q * dx);
      ry += (double)(q * q * dy);
    }
    gx = -rx / sum_q;
    gy = -ry / sum_q;
  }
  if (!active) return;
  const double* prow = P + (long long)i * tp.k;
  for (int j = 0; j < tp.k; ++j) {
    const float2 rr = ref[idx[(long long)j * tp.nq + i] - tp.offset];
    const float dx = yx - rr.x, dy = yy - rr.y;
    const double q = (double)(1.0f / (1.0f + dx * dx + dy * dy));
    const double c = exag * prow[j] * q;
    gx += c * (double)dx;
    gy += c * (double)dy;
  }
  const double g2 = gx * gx + gy * gy;
  if (g2 > tp.max_grad * tp.max_grad) {
    const double sc = tp.max_grad / (sqrt(g2) + 1e-12);
    gx *= sc;
    gy *= sc;
  }
  double2 ga = gains[i], up = upd[i];
  auto sgn = [](double v) { return v == 0.0 ? 0.0 : (v < 0.0 ? -1.0 : 1.0); };
  ga.x = sgn(up.x) != sgn(gx) ? ga.x + 0.2 : ga.x * 0.8 + 0.01;
  ga.y = sgn(up.y) != sgn(gy) ? ga.y + 0.2 : ga.y * 0.8 + 0.01;
  if (ga.x < 0.01) ga.x = 0.01;
  if (ga.y < 0.01) ga.y = 0.01;
  up.x = mom * up.x - tp.lr * ga.x * gx;
  up.y = mom * up.y - tp.lr * ga.y * gy;
  const double s2 = up.x * up.x + up.y * up.y;
  if (s2 > tp.max_step * tp.max_step) {
    const double sc = tp.max_step / (sqrt(s2) + 1e-12);
    up.x *= sc;
    up.y *= sc;
  }
  gains[i] = ga;
  upd[i] = up;
  y[i] = make_double2(yi.x + up.x, yi.y + up.y);
}

__global__ void transform_prepare_kernel(const double* __restrict__ ref_cm, int nref, float2* __restrict__ ref) {
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < nref; r += gridDim.x * blockDim.x)
    ref[r] = make_float2((float)ref_cm[r], (float)ref_cm[(long long)nref + r]);
}

__global__ void transform_state_kernel(const double* __restrict__ init_cm, int nq, double2* __restrict__ y,
                                       double2* __restrict__ gains, double2* __restrict__ upd) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nq; i += gridDim.x * blockDim.x) {
    if (init_cm) y[i] = make_double2(init_cm[i], init_cm[(long long)nq + i]);
    gains[i] = make_double2(1.0, 1.0);
    upd[i] = make_double2(0.0, 0.0);
  }
}

__global__ void transform_output_kernel(const double2* __restrict__ y, int nq, double* __restrict__ out_cm) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nq; i += gridDim.x * blockDim.x) {
    out_cm[i] = y[i].x;
    out_cm[(long long)nq + i] = y[i].y;
  }
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
    if (n_reference < 1) throw fe::Error("`reference_layout` must be a non-empty matrix.");
    if (n_query < 1 || k < 1)
      throw fe::Error("KNN input must have at least one query row and one neighbor column.");
    if (!(perplexity > 0.0)) throw fe::Error("`perplexity` must be positive.");
    if (n_iter < 0 || early_exaggeration_iter < 0) throw fe::Error("iteration counts must be non-negative.");
    if (n_iter + early_exaggeration_iter < 1) throw fe::Error("at least one transform iteration is required.");
    if (!(learning_rate > 0.0)) throw fe::Error("`learning_rate` must be positive.");
    if (!(early_exaggeration > 0.0) || !(exaggeration > 0.0)) throw fe::Error("exaggeration values must be positive.");
    if (initial_momentum < 0.0 || final_momentum < 0.0) throw fe::Error("momentum values must be non-negative.");
    if (n_negatives < 1) throw fe::Error("`n_negatives` must be positive.");
    int mode = 0;
    const std::string ini = initialization ? initialization : "median";
    if (ini != "median" && ini != "weighted" && ini != "random")
      throw fe::Error("`initialization` must be 'median', 'weighted', or 'random'.");
    if (!init) mode = ini == "median" ? 1 : (ini == "weighted" ? 2 : 3);
    if (exact_repulsion_threshold < 1) exact_repulsion_threshold = 1;
    if (!(max_grad_norm > 0.0) || !std::isfinite(max_grad_norm)) max_grad_norm = DBL_MAX;
    if (!(max_step_norm > 0.0) || !std::isfinite(max_step_norm)) max_step_norm = DBL_MAX;
    // resolve_reference_index_offset / range checks (src/tsne_neighbors.cpp:1371-1382, :2175-2185)
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
    if (seed == INT_MIN) seed = 5489;  // R's NA_integer_
    // initialization = "random": N(0, 1e-4^2) per coordinate from std::mt19937 seeded per query
    // exactly as initialize_tsne_transform (src/tsne_neighbors.cpp:1398-1413); host work of
    // n_query x 2 draws, uploaded as the initial layout.
    std::vector<double> random_init;
    if (mode == 3) {
      random_init.resize(2 * (std::size_t)n_query);
      for (int i = 0; i < n_query; ++i) {
        std::normal_distribution<double> normal(0.0, 1.0e-4);
        std::uint32_t v = (std::uint32_t)seed ^ ((std::uint32_t)(i + 1) * 0x9e3779b9u);
        v ^= v >> 16u;
        v *= 0x7feb352du;
        v ^= v >> 15u;
        v *= 0x846ca68bu;
        v ^= v >> 16u;
        std::mt19937 rng(v == 0u ? 0x6d2b79f5u : v);
        const double a = normal(rng);
        const double b = normal(rng);
        random_init[i] = a;  // column-major n_query x 2
        random_init[(std::size_t)n_query + i] = b;
      }
      y_init = random_init.data();
      init = 1;
    }
    if (n_negatives > n_reference) n_negatives = n_reference;
    const int exact = (n_reference <= exact_repulsion_threshold || n_negatives >= n_reference) ? 1 : 0;
    fe::Stream st;
    cudaStream_t s = st.s;
    double *d_ref_cm = nullptr, *d_dist = nullptr, *d_P = nullptr, *d_init = nullptr, *d_out = nullptr;
    int* d_idx = nullptr;
    float2* d_ref = nullptr;
    double2 *d_y = nullptr, *d_g = nullptr, *d_u = nullptr;
    fe::Arena a;
    a.reserve(&d_ref_cm, 2 * (std::size_t)n_reference);
    a.reserve(&d_ref, n_reference);
    a.reserve(&d_idx, items);
    a.reserve(&d_dist, items);
    a.reserve(&d_P, items);
    if (init) a.reserve(&d_init, 2 * (std::size_t)n_query);
    a.reserve(&d_out, 2 * (std::size_t)n_query);
    a.reserve(&d_y, n_query);
    a.reserve(&d_g, n_query);
    a.reserve(&d_u, n_query);
    a.commit("CUDA t-SNE transform");
    FE_CUDA(cudaMemcpyAsync(d_ref_cm, reference_layout, sizeof(double) * 2 * n_reference, cudaMemcpyHostToDevice, s));
    FE_CUDA(cudaMemcpyAsync(d_idx, indices, sizeof(int) * items, cudaMemcpyHostToDevice, s));
    FE_CUDA(cudaMemcpyAsync(d_dist, distances, sizeof(double) * items, cudaMemcpyHostToDevice, s));
    if (init) FE_CUDA(cudaMemcpyAsync(d_init, y_init, sizeof(double) * 2 * n_query, cudaMemcpyHostToDevice, s));
    const int pb = std::max(1, std::min(fe::ceil_div(std::max(n_query, n_reference), 256), fe::sm_count() * 8));
    fe::transform_prepare_kernel<<<pb, 256, 0, s>>>(d_ref_cm, n_reference, d_ref);
    FE_LAUNCH("transform_prepare_kernel");
    fe::transform_row_p_kernel<<<fe::ceil_div((long long)n_query * 32, 256), 256, 0, s>>>(d_dist, n_query, k,
                                                                                         perplexity, d_P);
    FE_LAUNCH("transform_row_p_kernel");
    fe::transform_state_kernel<<<pb, 256, 0, s>>>(init ? d_init : nullptr, n_query, d_y, d_g, d_u);
    FE_LAUNCH("transform_state_kernel");
    if (!init) {
      fe::transform_init_kernel<<<fe::ceil_div(n_query, 128), 128, 0, s>>>(d_ref_cm, n_reference, d_idx, d_dist,
                                                                          n_query, k, offset, mode, d_y);
      FE_LAUNCH("transform_init_kernel");
    }
    const fe::TransformParams tp{n_reference, n_query, k, offset, n_negatives, exact,
                                 learning_rate, max_grad_norm, max_step_norm};
    const int total = n_iter + early_exaggeration_iter;
    for (int it = 0; it < total; ++it) {
      const bool early = it < early_exaggeration_iter;
      const int iter_seed = seed + 65537 * (it + 1);
      fe::transform_iteration_kernel<<<fe::ceil_div(n_query, fe::kTransformThreads), fe::kTransformThreads, 0, s>>>(
          d_ref, d_idx, d_P, d_y, d_g, d_u, tp, early ? early_exaggeration : exaggeration,
          early ? initial_momentum : final_momentum, iter_seed);
      FE_LAUNCH("transform_iteration_kernel");
    }
    fe::transform_output_kernel<<<pb, 256, 0, s>>>(d_y, n_query, d_out);
    FE_LAUNCH("transform_output_kernel");
    FE_CUDA(cudaMemcpyAsync(out, d_out, sizeof(double) * 2 * n_query, cudaMemcpyDeviceToHost, s));
    FE_CUDA(cudaStreamSynchronize(s));
  });
}
