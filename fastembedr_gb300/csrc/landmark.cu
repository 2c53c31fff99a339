// Landmark t-SNE transform (project_landmark_model's CUDA route): the C ABI
// fastembedr_cuda_landmark_tsne_from_device_knn of the reference
// (src/embedding_cuda_kernels.cpp:3572-3686, kernels :552-861).
//
// Each query starts at a local affine projection of its nearest landmarks: weights
// w_j = exp(-(d_j - rho) / sigma) over the first m neighbours (rho the nearest distance, sigma the
// median positive excess), a weighted, ridge-regularised least-squares map from the landmarks'
// centred features to their centred layout coordinates, applied to the query's centred features,
// with the displacement bounded by max_extrapolation times the neighbourhood's layout radius;
// a query at distance ~0 from a landmark starts on it, and a singular system falls back to the
// weighted mean. The start is then optimised by the fixed-reference transform engine
// (transform.cu) with the landmark path's hash sampler for the repulsion.
//
// The affine solve runs in FP64 (the reference solves it in FP32), so starts agree to the
// reference's rounding rather than bit for bit.
#include <cfloat>
#include <cmath>
#include <vector>

#include "../../include/fastembedr_cuda.h"
#include "transform.cuh"

namespace fe {

TransformParams transform_params(int n_ref, int n_negatives, int exact_repulsion_threshold, double perplexity,
                                 int n_iter, int early_iter, double learning_rate, double early_exaggeration,
                                 double exaggeration, double initial_momentum, double final_momentum,
                                 double max_grad_norm, double max_step_norm, int init_mode, int seed);
int transform_chunk(long long n_query, const TransformParams& tp, int k);
void transform_upload_reference(const double* d_ref_cm, int n_ref, float2* ref, double2* ref_d, cudaStream_t s);

constexpr int kAffineMax = 12;  // affine neighbours at most (the reference's kCudaAffineMaxNeighbors)
constexpr int kLandmarkMaxK = 128;

// Weighted mean of the valid neighbours' layout positions (the fallback start).
__device__ void weighted_mean_start(const float* __restrict__ layout, int n_ref, const int* __restrict__ idx,
                                    const float* __restrict__ dist, int nq, int k, int offset, int row, double rho,
                                    double sigma, double* out) {
  const double eps = 1.4901161193847656e-8;
  double ws = 0.0, vx = 0.0, vy = 0.0;
  for (int j = 0; j < k; ++j) {
    const int r = idx[(long long)j * nq + row] - offset;
    const float d = dist[(long long)j * nq + row];
    if (r < 0 || r >= n_ref || !isfinite(d) || d < 0.0f) continue;
    const double w = exp(-fmax(0.0, (double)d - rho) / fmax(sigma, eps));
    if (!isfinite(w) || w <= 0.0) continue;
    ws += w;
    vx += w * layout[r];
    vy += w * layout[(long long)n_ref + r];
  }
  if (!isfinite(ws) || ws <= 0.0) ws = 1.0;
  out[0] = vx / ws;
  out[1] = vy / ws;
}

// Thread per query; writes the start as column-major n_query x 2 doubles.
__global__ void landmark_affine_kernel(const float* __restrict__ X, const float* __restrict__ Q,
                                       const float* __restrict__ layout, const int* __restrict__ idx,
                                       const float* __restrict__ dist, int n_ref, int nq, int nf, int k, int offset,
                                       int m, double ridge, double max_extrapolation, double* __restrict__ y0) {
  const int row = blockIdx.x * blockDim.x + threadIdx.x;
  if (row >= nq) return;
  const double eps = 1.4901161193847656e-8;
  double start[2];
  // nearest valid distance, a landmark at (numerically) zero distance
  double rho = INFINITY;
  int zero_ref = -1;
  for (int j = 0; j < k; ++j) {
    const int r = idx[(long long)j * nq + row] - offset;
    const float d = dist[(long long)j * nq + row];
    if (r < 0 || r >= n_ref || !isfinite(d) || d < 0.0f) continue;
    if (d <= eps && zero_ref < 0) zero_ref = r;
    rho = fmin(rho, (double)d);
  }
  if (!isfinite(rho)) rho = 0.0;
  if (zero_ref >= 0) {
    y0[row] = layout[zero_ref];
    y0[(long long)nq + row] = layout[(long long)n_ref + zero_ref];
    return;
  }
  // sigma: median of the positive excess distances (insertion sort of at most k values)
  double exc[kLandmarkMaxK];
  int cnt = 0;
  for (int j = 0; j < k; ++j) {
    const int r = idx[(long long)j * nq + row] - offset;
    const float d = dist[(long long)j * nq + row];
    const bool valid = r >= 0 && r < n_ref && isfinite(d) && d >= 0.0f;
    const double a = valid ? fmax(0.0, (double)d - rho) : INFINITY;
    if (!isfinite(a) || a <= eps) continue;
    int p = cnt++;
    while (p > 0 && exc[p - 1] > a) {
      exc[p] = exc[p - 1];
      --p;
    }
    exc[p] = a;
  }
  double sigma = cnt > 0 ? ((cnt & 1) ? exc[cnt / 2] : 0.5 * (exc[cnt / 2 - 1] + exc[cnt / 2])) : fmax(rho, eps);
  if (!isfinite(sigma) || sigma < eps) sigma = eps;

  int refs[kAffineMax];
  double w[kAffineMax], sw[kAffineMax];
  double wsum = 0.0;
  for (int a = 0; a < m; ++a) {
    const int r = idx[(long long)a * nq + row] - offset;
    const float d = dist[(long long)a * nq + row];
    const bool valid = r >= 0 && r < n_ref && isfinite(d) && d >= 0.0f;
    refs[a] = valid || (r >= 0 && r < n_ref) ? r : -1;
    const double ex = valid ? fmax(0.0, (double)d - rho) : INFINITY;
    w[a] = (r >= 0 && r < n_ref && isfinite(ex)) ? exp(-ex / sigma) : 0.0;
    wsum += w[a];
  }
  if (!isfinite(wsum) || wsum <= 0.0) {
    weighted_mean_start(layout, n_ref, idx, dist, nq, k, offset, row, rho, sigma, start);
    y0[row] = start[0];
    y0[(long long)nq + row] = start[1];
    return;
  }
  double cy[2] = {0.0, 0.0};
  for (int a = 0; a < m; ++a) {
    w[a] /= wsum;
    sw[a] = sqrt(fmax(w[a], 0.0));
    if (refs[a] >= 0) {
      cy[0] += w[a] * layout[refs[a]];
      cy[1] += w[a] * layout[(long long)n_ref + refs[a]];
    }
  }
  // right-hand sides sqrt(w_a) (y_a - centre) and the neighbourhood's layout radius
  double rhs[kAffineMax][2], radius2 = 0.0;
  for (int a = 0; a < m; ++a) {
    const double u = refs[a] >= 0 ? layout[refs[a]] - cy[0] : 0.0;
    const double v = refs[a] >= 0 ? layout[(long long)n_ref + refs[a]] - cy[1] : 0.0;
    rhs[a][0] = sw[a] * u;
    rhs[a][1] = sw[a] * v;
    radius2 = fmax(radius2, u * u + v * v);
  }
  // weighted Gram matrix of the centred landmark features and their products with the query
  double G[kAffineMax][kAffineMax], qv[kAffineMax], norm2[kAffineMax];
  for (int a = 0; a < m; ++a) {
    qv[a] = 0.0;
    norm2[a] = 0.0;
    for (int b = 0; b <= a; ++b) G[a][b] = 0.0;
  }
  for (int f = 0; f < nf; ++f) {
    const float* Xf = X + (long long)f * n_ref;
    double xc = 0.0;
    for (int a = 0; a < m; ++a)
      if (refs[a] >= 0) xc += w[a] * Xf[refs[a]];
    const double qc = (double)Q[(long long)f * nq + row] - xc;
    double c[kAffineMax];
    for (int a = 0; a < m; ++a) {
      c[a] = refs[a] >= 0 ? Xf[refs[a]] - xc : 0.0;
      norm2[a] += c[a] * c[a];
      qv[a] += qc * c[a];
      for (int b = 0; b <= a; ++b) G[a][b] += c[a] * c[b];
    }
  }
  double trace = 0.0;
  for (int a = 0; a < m; ++a) {
    trace += w[a] * norm2[a];
    qv[a] *= sw[a];
    for (int b = 0; b <= a; ++b) G[a][b] *= sw[a] * sw[b];
  }
  const double lambda = ridge * fmax(trace, eps) + eps;
  for (int a = 0; a < m; ++a) G[a][a] += lambda;
  // Cholesky G = L L^T in the lower triangle
  bool ok = true;
  for (int j = 0; j < m && ok; ++j) {
    double dg = G[j][j];
    for (int t = 0; t < j; ++t) dg -= G[j][t] * G[j][t];
    if (!isfinite(dg) || dg <= eps) {
      ok = false;
      break;
    }
    dg = sqrt(dg);
    G[j][j] = dg;
    for (int i = j + 1; i < m; ++i) {
      double v = G[i][j];
      for (int t = 0; t < j; ++t) v -= G[i][t] * G[j][t];
      G[i][j] = v / dg;
    }
  }
  if (ok) {
    double disp[2] = {0.0, 0.0};
    for (int comp = 0; comp < 2; ++comp) {
      double z[kAffineMax];
      for (int i = 0; i < m; ++i) {  // L z = rhs
        double v = rhs[i][comp];
        for (int t = 0; t < i; ++t) v -= G[i][t] * z[t];
        z[i] = v / G[i][i];
      }
      for (int i = m - 1; i >= 0; --i) {  // L^T x = z
        double v = z[i];
        for (int t = i + 1; t < m; ++t) v -= G[t][i] * z[t];
        z[i] = v / G[i][i];
      }
      for (int a = 0; a < m; ++a) disp[comp] += qv[a] * z[a];
    }
    const double cap = max_extrapolation * sqrt(fmax(radius2, eps));
    const double d2 = disp[0] * disp[0] + disp[1] * disp[1];
    if (d2 > cap * cap) {
      const double sc = cap / (sqrt(d2) + eps);
      disp[0] *= sc;
      disp[1] *= sc;
    }
    start[0] = cy[0] + disp[0];
    start[1] = cy[1] + disp[1];
    ok = isfinite(start[0]) && isfinite(start[1]);
  }
  if (!ok) weighted_mean_start(layout, n_ref, idx, dist, nq, k, offset, row, rho, sigma, start);
  y0[row] = start[0];
  y0[(long long)nq + row] = start[1];
}

__global__ void float_to_double_kernel(const float* __restrict__ in, long long n, double* __restrict__ out) {
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x)
    out[t] = in[t];
}

__global__ void layout_interleave_kernel(const double* __restrict__ cm, int n, float* __restrict__ out) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    out[2 * (long long)i] = (float)cm[i];
    out[2 * (long long)i + 1] = (float)cm[(long long)n + i];
  }
}

}  // namespace fe

extern "C" int fastembedr_cuda_landmark_tsne_from_device_knn(
    const int* device_indices, const float* device_distances, int index_offset, const float* reference_data,
    const float* query_data, const float* reference_layout, int n_reference, int n_query, int n_features, int k,
    float perplexity, int n_iter, int early_exaggeration_iter, float learning_rate, float early_exaggeration,
    float exaggeration, float initial_momentum, float final_momentum, float max_grad_norm, float max_step_norm,
    int n_negatives, int exact_repulsion_threshold, unsigned int seed, int affine_neighbors, float affine_ridge,
    float max_extrapolation, float* out) {
  return fe::guarded([&] {
    if (!device_indices || !device_distances || !reference_data || !query_data || !reference_layout || !out)
      throw fe::Error("null CUDA landmark t-SNE pointer");
    if (n_reference < 1 || n_query < 1 || n_features < 1 || k < 1 || k > fe::kLandmarkMaxK || !(perplexity > 0.0f) ||
        n_iter < 0 || early_exaggeration_iter < 0)
      throw fe::Error("invalid CUDA landmark t-SNE dimensions or parameters");
    n_negatives = std::max(1, std::min(n_negatives, n_reference));
    const int m = std::max(3, std::min(affine_neighbors, std::min(k, fe::kAffineMax)));
    fe::Stream st;
    cudaStream_t s = st.s;
    fe::order_after_legacy_stream(s);  // the KNN arrays are the caller's device buffers
    const long long items = (long long)n_query * k;
    float *d_X = nullptr, *d_Q = nullptr, *d_layout = nullptr, *d_out_f = nullptr;
    double *d_layout_d = nullptr, *d_init = nullptr, *d_res = nullptr;
    float2* d_ref = nullptr;
    double2* d_ref_d = nullptr;
    float2* d_nb = nullptr;
    float* d_p = nullptr;
    float4 *d_state = nullptr, *d_opt = nullptr;
    fe::TransformSegment* d_seg = nullptr;
    fe::XorshiftJump* d_jump = nullptr;
    fe::Arena a;
    a.reserve(&d_X, (std::size_t)n_reference * n_features);
    a.reserve(&d_Q, (std::size_t)n_query * n_features);
    a.reserve(&d_layout, 2 * (std::size_t)n_reference);
    a.reserve(&d_layout_d, 2 * (std::size_t)n_reference);
    a.reserve(&d_ref, n_reference);
    a.reserve(&d_ref_d, n_reference);
    a.reserve(&d_init, 2 * (std::size_t)n_query);
    a.reserve(&d_nb, items);
    a.reserve(&d_p, items);
    a.reserve(&d_state, n_query);
    a.reserve(&d_opt, n_query);
    a.reserve(&d_res, 2 * (std::size_t)n_query);
    a.reserve(&d_out_f, 2 * (std::size_t)n_query);
    a.reserve(&d_seg, 1);
    a.reserve(&d_jump, 1);
    a.commit("CUDA landmark t-SNE");
    FE_CUDA(cudaMemcpyAsync(d_X, reference_data, sizeof(float) * n_reference * (std::size_t)n_features,
                            cudaMemcpyHostToDevice, s));
    FE_CUDA(cudaMemcpyAsync(d_Q, query_data, sizeof(float) * n_query * (std::size_t)n_features, cudaMemcpyHostToDevice,
                            s));
    FE_CUDA(cudaMemcpyAsync(d_layout, reference_layout, sizeof(float) * 2 * (std::size_t)n_reference,
                            cudaMemcpyHostToDevice, s));
    const int pb = std::max(1, std::min(fe::ceil_div(2LL * std::max(n_reference, n_query), 256), fe::sm_count() * 8));
    fe::float_to_double_kernel<<<pb, 256, 0, s>>>(d_layout, 2LL * n_reference, d_layout_d);
    FE_LAUNCH("float_to_double_kernel");
    fe::transform_upload_reference(d_layout_d, n_reference, d_ref, d_ref_d, s);
    fe::landmark_affine_kernel<<<fe::ceil_div(n_query, 128), 128, 0, s>>>(
        d_X, d_Q, d_layout, device_indices, device_distances, n_reference, n_query, n_features, k, index_offset, m,
        (double)affine_ridge, (double)max_extrapolation, d_init);
    FE_LAUNCH("landmark_affine_kernel");
    if (n_iter + early_exaggeration_iter == 0) {  // the affine start is the result
      fe::layout_interleave_kernel<<<pb, 256, 0, s>>>(d_init, n_query, d_out_f);
      FE_LAUNCH("layout_interleave_kernel");
      FE_CUDA(cudaMemcpyAsync(out, d_out_f, sizeof(float) * 2 * (std::size_t)n_query, cudaMemcpyDeviceToHost, s));
      FE_CUDA(cudaStreamSynchronize(s));
      return;
    }
    fe::TransformParams tp = fe::transform_params(
        n_reference, n_negatives, exact_repulsion_threshold, perplexity, n_iter, early_exaggeration_iter,
        learning_rate, early_exaggeration, exaggeration, initial_momentum, final_momentum, max_grad_norm,
        max_step_norm, 0, 0);
    tp.seed = (int)seed;
    tp.hash_sampler = 1;
    const fe::TransformSegment seg{device_indices, device_distances, nullptr, d_init, d_nb, d_p, d_state, d_opt,
                                   d_res, 0, n_query, k, index_offset};
    FE_CUDA(cudaMemcpyAsync(d_seg, &seg, sizeof(seg), cudaMemcpyHostToDevice, s));
    const fe::XorshiftJump jump = fe::xorshift_jump_table(tp.n_negatives);
    FE_CUDA(cudaMemcpyAsync(d_jump, &jump, sizeof(jump), cudaMemcpyHostToDevice, s));
    fe::transform_prepare(d_ref, d_ref_d, d_seg, 1, n_query, tp, s);
    const int chunk = fe::transform_chunk(n_query, tp, k);
    for (int it = 0; it < tp.iter_total; it += chunk)
      fe::transform_iterate(d_ref, d_seg, 1, n_query, tp, d_jump, it, std::min(tp.iter_total, it + chunk), s);
    fe::layout_interleave_kernel<<<pb, 256, 0, s>>>(d_res, n_query, d_out_f);
    FE_LAUNCH("layout_interleave_kernel");
    FE_CUDA(cudaMemcpyAsync(out, d_out_f, sizeof(float) * 2 * (std::size_t)n_query, cudaMemcpyDeviceToHost, s));
    FE_CUDA(cudaStreamSynchronize(s));
  });
}
