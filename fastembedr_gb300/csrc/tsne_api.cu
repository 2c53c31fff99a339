// C ABI of the t-SNE optimizer (see include/fastembedr_cuda.h) and the host driver behind it:
// the GB300 counterpart of fastembedr_cuda_opentsne_fft_from_knn_impl
// (fastEmbedR src/embedding_cuda_kernels.cpp:5629-6176) and of the validation in
// knn_tsne_opentsne_cuda_float_impl (src/embedding_cuda_impl.cpp:2239-2370).
#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <tuple>
#include <type_traits>
#include <vector>

#include "../../include/fastembedr_cuda.h"
#include "pca.cuh"
#include "philox.cuh"
#include "tsne_exact.cuh"
#include "tsne_grid.cuh"

namespace fe {

// Seeded N(0, 1e-4^2) layout (Box-Muller on Philox4x32-10 draws) for has_init = 0.
__global__ void random_init_kernel(float2* __restrict__ y, int n, unsigned seed) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const uint4 r = philox4x32_10(make_uint4((unsigned)i, 0u, 0x7a5e11u, 0u), make_uint2(seed, 0x1badb002u));
    const float u1 = fmaxf(u01(r.x), 1.0e-12f), u2 = u01(r.y);
    const float rad = 1.0e-4f * sqrtf(-2.0f * logf(u1));
    float sn, cs;
    sincospif(2.0f * u2, &sn, &cs);
    y[i] = make_float2(rad * cs, rad * sn);
  }
}

__global__ void double_to_float_kernel(const double* __restrict__ in, float* __restrict__ out, long long m) {
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < m; t += (long long)gridDim.x * blockDim.x)
    out[t] = (float)in[t];
}

bool reorder_enabled() {
  const char* env = std::getenv("FASTEMBEDR_TSNE_REORDER");
  return !(env && env[0] == '0');
}

bool autotune_enabled() {
  const char* env = std::getenv("FASTEMBEDR_TSNE_AUTOTUNE");
  return !(env && env[0] == '0');
}

bool graph_capture_enabled() {
  const char* env = std::getenv("FASTEMBEDR_CUDA_GRAPH_CAPTURE");
  if (!env || !env[0]) return true;
  return !(std::strcmp(env, "0") == 0 || std::strcmp(env, "false") == 0 || std::strcmp(env, "FALSE") == 0 ||
           std::strcmp(env, "no") == 0 || std::strcmp(env, "NO") == 0);
}

// Smallest and largest label of a KNN block (knn_index_offset's test on the device).
__global__ void label_range_kernel(const int* __restrict__ idx, long long total, int* __restrict__ range) {
  int lo = INT_MAX, hi = INT_MIN;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
       t += (long long)gridDim.x * blockDim.x) {
    lo = min(lo, idx[t]);
    hi = max(hi, idx[t]);
  }
  for (int o = 16; o > 0; o >>= 1) {
    lo = min(lo, __shfl_xor_sync(0xffffffffu, lo, o));
    hi = max(hi, __shfl_xor_sync(0xffffffffu, hi, o));
  }
  if ((threadIdx.x & 31) == 0) {
    atomicMin(range, lo);
    atomicMax(range + 1, hi);
  }
}

// One instance's nb x k KNN (column-major, or row-major) into the batch's column-major n x k matrix at rows
// [first, first + nb), neighbour labels turned into global 0-based rows.
__global__ void globalize_knn_kernel(const int* __restrict__ idx, const float* __restrict__ dist, int nb, int k,
                                     int offset, int row_major, int first, int n, int* __restrict__ idx_out,
                                     float* __restrict__ dist_out) {
  const long long total = (long long)nb * k;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
       t += (long long)gridDim.x * blockDim.x) {
    long long i, j;
    if (row_major) {
      i = t / k;
      j = t - i * k;
    } else {
      j = t / nb;
      i = t - j * nb;
    }
    const long long o = j * n + first + i;
    idx_out[o] = idx[t] - offset + first;
    dist_out[o] = dist[t];
  }
}

// out[r] = full[inv[rows[r]]] for the two float2 force fields of a diagnostic.
__global__ void gather_rows_kernel(const float2* __restrict__ a, const float2* __restrict__ b,
                                   const int* __restrict__ rows, const int* __restrict__ inv, int n_rows,
                                   float2* __restrict__ a_out, float2* __restrict__ b_out) {
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n_rows; r += gridDim.x * blockDim.x) {
    const int si = inv[rows[r]];
    a_out[r] = a[si];
    b_out[r] = b[si];
  }
}

// Optimizer state of one t-SNE instance (or a batch of instances) resident on the device.
struct TsneJob {
  DeviceCsr P;
  TsneDevice D;
  Stream stream;
  // graph cache keyed by (iterations, exaggeration, lr, momentum, min_gain, max_step)
  using Key = std::tuple<int, float, float, float, float, float>;
  std::map<Key, std::pair<cudaGraph_t, cudaGraphExec_t>> graphs;
  // Adaptive box count: at the start of every chunk each instance gets the smallest power-of-two
  // grid whose node spacing over its current bounding square is at most `spacing` (clamped to
  // [grid_min, grid_max]); grids grow at once and shrink only when four times too fine.
  bool reorder = true;  // periodic spatial reorder (FASTEMBEDR_TSNE_REORDER=0 turns it off), fixed at prepare
  // The 256-node floor keeps small instances on the CUDA size policy's grid (below 20,000 points
  // both give 256 nodes for final spans up to ~180), so adaptivity only coarsens the large
  // instances whose policy grid is finer than their layout needs.
  bool adaptive = false;
  float spacing = 0.7f;
  int grid_min = 256, grid_max = 1024;
  int regrids = 0;
  ~TsneJob() { clear_graphs(); }
  void clear_graphs() {
    for (auto& kv : graphs) {
      if (kv.second.second) cudaGraphExecDestroy(kv.second.second);
      if (kv.second.first) cudaGraphDestroy(kv.second.first);
    }
    graphs.clear();
  }
  // Adaptive grids when asked for, or when FASTEMBEDR_TSNE_FFT_GRID=adaptive; the target spacing
  // comes from FASTEMBEDR_TSNE_GRID_SPACING when set.
  void configure_adaptive(bool on) {
    const char* env = std::getenv("FASTEMBEDR_TSNE_FFT_GRID");
    adaptive = on || (env && std::strcmp(env, "adaptive") == 0);
    const char* sp = std::getenv("FASTEMBEDR_TSNE_GRID_SPACING");
    if (sp && sp[0]) {
      const float v = (float)std::atof(sp);
      if (v > 0.0f && std::isfinite(v)) spacing = v;
    }
  }
  void adapt_grids() {
    cudaStream_t s = stream.s;
    const std::vector<float> ext = tsne_grid_extents(D, s);
    std::vector<int> grids(D.inst.size());
    bool changed = false;
    for (std::size_t b = 0; b < grids.size(); ++b) {
      const float need = (std::isfinite(ext[b]) ? ext[b] : 0.0f) / spacing + 1.0f;
      int g = grid_min;
      while (g < grid_max && (float)g < need) g <<= 1;
      const int cur = D.inst[b].grid;
      grids[b] = (g > cur || 4 * g <= cur) ? g : cur;
      changed |= grids[b] != cur;
    }
    if (!changed) return;
    clear_graphs();
    tsne_regrid(D, grids, s);
    ++regrids;
  }

  // KNN (device, column-major) -> P (CSR) -> optimizer state with the given init.
  void prepare(const int* d_idx, const float* d_dist, const float* init_host, int n, int k, float perplexity,
               int offset, int grid, int mode, unsigned seed) {
    cudaStream_t s = stream.s;
    configure_adaptive(false);
    order_after_legacy_stream(s);  // d_idx / d_dist may be the caller's buffers
    validate_knn(d_idx, d_dist, n, k, offset, s);
    {
      float* d_p = nullptr;
      Arena tmp;
      tmp.reserve(&d_p, (std::size_t)n * k);
      tmp.commit("t-SNE directed probabilities");
      row_probabilities(d_idx, d_dist, n, k, perplexity, d_p, nullptr, s);
      symmetrise(d_idx, d_p, n, k, offset, P, s);
    }
    tsne_device_alloc(D, n, grid, mode);
    reorder = reorder_enabled();
    float2* d_init = nullptr;
    Arena tmp;
    tmp.reserve(&d_init, n);
    tmp.commit("t-SNE init");
    if (init_host) {
      FE_CUDA(cudaMemcpyAsync(d_init, init_host, sizeof(float2) * n, cudaMemcpyHostToDevice, s));
    } else {
      random_init_kernel<<<std::max(1, std::min(ceil_div(n, 256), sm_count() * 8)), 256, 0, s>>>(d_init, n, seed);
      FE_LAUNCH("random_init_kernel");
    }
    tsne_device_init(D, reinterpret_cast<const float*>(d_init), s);
    tsne_bind_rows(D, P, s);
    FE_CUDA(cudaStreamSynchronize(s));
  }

  // Batch: instances in table order (equal grids consecutive); `user` maps table position to
  // the caller's instance index. KNN / init are the caller's host arrays, instance after
  // instance. The instances' KNN are placed in one matrix with global labels and P is built for
  // all of them at once; every instance keeps its own normalisation (symmetrise_batch), so its
  // rows of P equal the P it gets alone.
  std::vector<int> user, user_off;
  void prepare_batch(int ninst, const int* sizes, const int* idx_h, const float* dist_h, const float* init_h, int k,
                     float perplexity, int offset, int grid_size, int mode, unsigned seed) {
    std::vector<const int*> iu(ninst);
    std::vector<const float*> du(ninst), yu(init_h ? ninst : 0);
    std::size_t at = 0;
    for (int u = 0; u < ninst; ++u) {
      iu[u] = idx_h + at * k;
      du[u] = dist_h + at * k;
      if (init_h) yu[u] = init_h + 2 * at;
      at += (std::size_t)std::max(sizes[u], 0);
    }
    prepare_batch(ninst, sizes, iu, du, yu, false, k, perplexity, offset, grid_size, mode, seed);
  }
  // The same from one host pointer per instance (KNN column-major, or row-major n_b x k when
  // row_major; init row-major n_b x 2 or none); offset < 0 detects each instance's 0- or 1-based
  // labels on the device as knn_index_offset does.
  void prepare_batch(int ninst, const int* sizes, const std::vector<const int*>& idx_u,
                     const std::vector<const float*>& dist_u, const std::vector<const float*>& init_u,
                     bool row_major, int k, float perplexity, int offset, int grid_size, int mode, unsigned seed) {
    cudaStream_t s = stream.s;
    std::vector<int> grid_u(ninst);
    user_off.assign(ninst + 1, 0);
    for (int u = 0; u < ninst; ++u) {
      if (sizes[u] < 2) throw Error("t-SNE batch: every instance needs at least two points");
      grid_u[u] = grid_size > 0 ? grid_size
                                : (grid_size == -1 ? cpu_fft_grid_size(sizes[u])
                                                   : (grid_size == -2 ? grid_min : default_grid_size(sizes[u], mode)));
      user_off[u + 1] = user_off[u] + sizes[u];
    }
    user.resize(ninst);
    for (int u = 0; u < ninst; ++u) user[u] = u;
    std::stable_sort(user.begin(), user.end(), [&](int a, int b) { return grid_u[a] > grid_u[b]; });
    std::vector<int> sz(ninst), gr(ninst);
    std::vector<float> lr(ninst);
    int max_n = 0;
    for (int t = 0; t < ninst; ++t) {
      sz[t] = sizes[user[t]];
      gr[t] = grid_u[user[t]];
      lr[t] = (float)sz[t];
      max_n = std::max(max_n, sz[t]);
    }
    tsne_batch_alloc(D, sz, gr, lr, mode);
    const int n = D.n;
    std::vector<int> first(ninst + 1, 0);
    for (int t = 0; t < ninst; ++t) first[t + 1] = first[t] + sz[t];
    {
      // every instance's KNN into one column-major n x k matrix in table order, columns turned
      // into global 0-based slots; then one bisection and one symmetrisation for the whole batch
      const std::size_t items = (std::size_t)n * k;
      int *d_loc_idx = nullptr, *d_idx = nullptr;
      float *d_loc_dist = nullptr, *d_dist = nullptr, *d_p = nullptr;
      Arena tmp;
      tmp.reserve(&d_loc_idx, items);
      tmp.reserve(&d_loc_dist, items);
      tmp.reserve(&d_idx, items);
      tmp.reserve(&d_dist, items);
      tmp.reserve(&d_p, items);
      tmp.commit("t-SNE batch affinities");
      int* d_range = nullptr;
      unsigned* d_flags = nullptr;
      Arena rng;
      rng.reserve(&d_range, 2);
      rng.reserve(&d_flags, 1);
      rng.commit("t-SNE batch label range");
      FE_CUDA(cudaMemsetAsync(d_flags, 0, sizeof(unsigned), s));
      for (int t = 0; t < ninst; ++t) {
        const int u = user[t], nb = sz[t];
        const std::size_t cnt = (std::size_t)nb * k;
        const std::size_t loc = (std::size_t)first[t] * k;
        fe::upload(d_loc_idx + loc, idx_u[u], sizeof(int) * cnt, s);
        fe::upload(d_loc_dist + loc, dist_u[u], sizeof(float) * cnt, s);
        const int blocks = std::max(1, std::min(ceil_div((long long)cnt, 256), sm_count() * 8));
        int off = offset;
        if (off < 0) {
          const int init_range[2] = {INT_MAX, INT_MIN};
          FE_CUDA(cudaMemcpyAsync(d_range, init_range, sizeof(init_range), cudaMemcpyHostToDevice, s));
          label_range_kernel<<<blocks, 256, 0, s>>>(d_loc_idx + loc, (long long)cnt, d_range);
          FE_LAUNCH("label_range_kernel");
          int h_range[2] = {0, 0};
          FE_CUDA(cudaMemcpyAsync(h_range, d_range, sizeof(h_range), cudaMemcpyDeviceToHost, s));
          FE_CUDA(cudaStreamSynchronize(s));
          off = (h_range[0] >= 1 && h_range[1] <= nb) ? 1 : 0;
        }
        validate_knn_async(d_loc_idx + loc, d_loc_dist + loc, nb, k, off, d_flags, s);
        globalize_knn_kernel<<<blocks, 256, 0, s>>>(d_loc_idx + loc, d_loc_dist + loc, nb, k, off, row_major ? 1 : 0,
                                                    first[t], n, d_idx, d_dist);
        FE_LAUNCH("globalize_knn_kernel");
      }
      // every instance's KNN is checked before the global labels are used
      unsigned flags = 0u;
      FE_CUDA(cudaMemcpyAsync(&flags, d_flags, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
      FE_CUDA(cudaStreamSynchronize(s));
      knn_flags_check(flags);
      row_probabilities(d_idx, d_dist, n, k, perplexity, d_p, nullptr, s);
      symmetrise_batch(d_idx, d_p, n, k, 0, first, P, nullptr, s);
    }
    reorder = reorder_enabled();
    float2* d_init = nullptr;
    Arena tmp;
    tmp.reserve(&d_init, n);
    tmp.commit("t-SNE batch init");
    for (int t = 0; t < ninst; ++t) {
      const int u = user[t];
      float2* dst = d_init + D.inst[t].pt_begin;
      if (!init_u.empty()) {
        FE_CUDA(cudaMemcpyAsync(dst, init_u[u], sizeof(float2) * sz[t], cudaMemcpyHostToDevice, s));
      } else {
        random_init_kernel<<<std::max(1, std::min(ceil_div(sz[t], 256), sm_count() * 8)), 256, 0, s>>>(dst, sz[t],
                                                                                                      seed);
        FE_LAUNCH("random_init_kernel");
      }
    }
    tsne_device_init(D, reinterpret_cast<const float*>(d_init), s);
    tsne_bind_rows(D, P, s);
    FE_CUDA(cudaStreamSynchronize(s));
  }

  // Iterations in chunks of 25; each chunk starts with a spatial reorder of the points and
  // is one CUDA graph launch (two streams inside).
  void run(int iters, float exag, float lr, float mom, float min_gain, float max_step, bool use_graph) {
    cudaStream_t s = stream.s;
    if (iters <= 0) return;
    constexpr int kChunk = 25;
    const bool graph = use_graph && graph_capture_enabled();
    // the attractive pass's launch is tuned once, on the first normal-phase run (the compact
    // early-exaggeration layout would time differently)
    if (!D.tuned && exag <= 1.0f && iters >= 25 && autotune_enabled()) {
      if (tsne_tune_attractive(D, P, exag, s)) clear_graphs();
    }
    int left = iters;
    while (left > 0) {
      const int c = std::min(kChunk, left);
      if (adaptive) adapt_grids();
      if (!graph) {
        if (reorder) tsne_reorder(D, P, s);
        for (int r = 0; r < c; ++r) tsne_iteration(D, P, exag, lr, mom, min_gain, max_step, s);
        left -= c;
        continue;
      }
      const Key key{c, exag, lr, mom, min_gain, max_step};
      auto it = graphs.find(key);
      if (it == graphs.end()) {
        cudaGraph_t g = nullptr;
        cudaGraphExec_t ge = nullptr;
        FE_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
        try {
          if (reorder) tsne_reorder(D, P, s);
          for (int r = 0; r < c; ++r) tsne_iteration(D, P, exag, lr, mom, min_gain, max_step, s);
        } catch (...) {
          cudaStreamEndCapture(s, &g);
          if (g) cudaGraphDestroy(g);
          throw;
        }
        FE_CUDA(cudaStreamEndCapture(s, &g));
        FE_CUDA(cudaGraphInstantiate(&ge, g, 0));
        it = graphs.emplace(key, std::make_pair(g, ge)).first;
      }
      FE_CUDA(cudaGraphLaunch(it->second.second, s));
      left -= c;
    }
  }

  void schedule(int early_iter, int n_iter, float early_exag, float exag, float lr, int lr_auto, float m0, float m1,
                float min_gain, float max_step) {
    const int n = D.n;
    const float lr_early = lr_auto ? (float)((double)n / std::max((double)early_exag, 1e-300)) : lr;
    const float lr_normal = lr_auto ? (float)((double)n / std::max((double)exag, 1e-300)) : lr;
    run(early_iter, early_exag, lr_early, m0, min_gain, max_step, true);
    run(n_iter, exag, lr_normal, m1, min_gain, max_step, true);
  }

  // Per-instance learning-rate multipliers (table order), uploaded on the job's stream so that
  // work already queued keeps the values it was queued with.
  void set_lr_mult(const std::vector<float>& mult) {
    for (std::size_t t = 0; t < D.inst.size(); ++t) D.inst[t].lr_mult = mult[t];
    FE_CUDA(cudaMemcpyAsync(D.d_inst, D.inst.data(), sizeof(TsneInstance) * D.inst.size(), cudaMemcpyHostToDevice,
                            stream.s));
    FE_CUDA(cudaStreamSynchronize(stream.s));
  }

  void layout(float* out_host) {
    cudaStream_t s = stream.s;
    float* d_out = nullptr;
    Arena tmp;
    tmp.reserve(&d_out, 2 * (std::size_t)D.n);
    tmp.commit("t-SNE output");
    tsne_finalize(D, d_out, s);
    FE_CUDA(cudaMemcpyAsync(out_host, d_out, sizeof(float) * 2 * D.n, cudaMemcpyDeviceToHost, s));
    FE_CUDA(cudaStreamSynchronize(s));
  }
};

// Argument checks of fastembedr_cuda_opentsne_fft_from_knn_impl (src/embedding_cuda_kernels.cpp:5661-5671).
void check_tsne_args(const void* idx, const void* dist, const float* init, int has_init, int n, int k,
                     int n_components, float perplexity, int early_iter, int n_iter, float early_exag, float exag,
                     float lr, int lr_auto, float m0, float m1, float min_gain, const float* out) {
  if (idx == nullptr || dist == nullptr || out == nullptr || (has_init && init == nullptr))
    throw Error("null CUDA openTSNE input pointer");
  if (n < 2 || k < 1 || k > 1024 || n_components != 2 || !(perplexity > 0.0f) || early_iter < 0 || n_iter < 0 ||
      early_iter + n_iter < 1 || !(early_exag > 0.0f) || !(exag > 0.0f) || (!lr_auto && !(lr > 0.0f)) || m0 < 0.0f ||
      m1 < 0.0f || !(min_gain > 0.0f))
    throw Error("invalid CUDA openTSNE FFT-grid dimensions or parameters");
}

// The PCA start of host data (column-major n x p, float or double) on the GPU, as a host
// row-major n x 2 init.
std::vector<float> pca_start(const void* values, bool is_double, int n, int p, cudaStream_t s) {
  const std::size_t items = (std::size_t)n * p;
  float* X = nullptr;
  double* raw = nullptr;
  float2* init = nullptr;
  Arena a;
  a.reserve(&X, items);
  if (is_double) a.reserve(&raw, items);
  a.reserve(&init, n);
  a.commit("device PCA input");
  if (is_double) {
    fe::upload(raw, values, sizeof(double) * items, s);
    double_to_float_kernel<<<std::max(1, std::min(ceil_div((long long)items, 256), sm_count() * 8)), 256, 0, s>>>(
        raw, X, (long long)items);
    FE_LAUNCH("double_to_float_kernel");
  } else {
    fe::upload(X, values, sizeof(float) * items, s);
  }
  pca_tsne_start(X, n, p, init, s);
  std::vector<float> h(2 * (std::size_t)n);
  FE_CUDA(cudaMemcpyAsync(h.data(), init, sizeof(float) * h.size(), cudaMemcpyDeviceToHost, s));
  FE_CUDA(cudaStreamSynchronize(s));
  return h;
}

template <typename DistT>
int run_tsne_from_knn(const int* indices, const DistT* distances, bool on_device, const float* init, int has_init,
                      int n, int k, int n_components, float perplexity, int early_iter, int n_iter, float early_exag,
                      float exag, float lr, int lr_auto, float m0, float m1, float min_gain, float max_step,
                      unsigned seed, int offset, float* out, const void* pca_values = nullptr,
                      bool pca_double = false, int pca_p = 0) {
  return guarded([&] {
    check_tsne_args(indices, distances, init, has_init, n, k, n_components, perplexity, early_iter, n_iter,
                    early_exag, exag, lr, lr_auto, m0, m1, min_gain, out);
    if (!has_init && pca_values && pca_p < n_components)
      throw Error("invalid CUDA openTSNE FFT-grid dimensions or parameters");
    auto job = std::make_unique<TsneJob>();
    cudaStream_t s = job->stream.s;
    if (on_device) order_after_legacy_stream(s);
    std::vector<float> pca_init;
    if (!has_init && pca_values) {
      pca_init = pca_start(pca_values, pca_double, n, pca_p, s);
      init = pca_init.data();
      has_init = 1;
    }
    const std::size_t items = (std::size_t)n * k;
    int* d_idx = nullptr;
    float* d_dist = nullptr;
    DistT* d_raw = nullptr;
    Arena in;
    if (!on_device) in.reserve(&d_idx, items);
    if (!on_device || !std::is_same<DistT, float>::value) in.reserve(&d_dist, items);
    if (!on_device && !std::is_same<DistT, float>::value) in.reserve(&d_raw, items);
    in.commit("CUDA openTSNE KNN input");
    const int* idx_ptr = on_device ? indices : d_idx;
    if (!on_device) fe::upload(d_idx, indices, sizeof(int) * items, s);
    const float* dist_ptr = nullptr;
    if constexpr (std::is_same<DistT, float>::value) {
      if (on_device) {
        dist_ptr = distances;
      } else {
        fe::upload(d_dist, distances, sizeof(float) * items, s);
        dist_ptr = d_dist;
      }
    } else {
      const DistT* src = distances;
      if (!on_device) {
        fe::upload(d_raw, distances, sizeof(DistT) * items, s);
        src = d_raw;
      }
      double_to_float_kernel<<<std::max(1, std::min(ceil_div((long long)items, 256), sm_count() * 8)), 256, 0, s>>>(
          src, d_dist, (long long)items);
      FE_LAUNCH("double_to_float_kernel");
      dist_ptr = d_dist;
    }
    const int mode = interp_mode_from_env();
    job->prepare(idx_ptr, dist_ptr, has_init ? init : nullptr, n, k, perplexity, offset, default_grid_size(n, mode),
                 mode, seed);
    in.release();
    job->schedule(early_iter, n_iter, early_exag, exag, lr, lr_auto, m0, m1, min_gain, max_step);
    job->layout(out);
  });
}

}  // namespace fe

struct fastembedr_tsne_plan {
  fe::TsneJob job;
};

struct fastembedr_tsne_batch {
  fe::TsneJob job;
};

extern "C" {

bool fastembedr_cuda_available(void) {
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return count > 0;
}

const char* fastembedr_cuda_embedding_last_error(void) { return fe::last_error(); }

int fastembedr_cuda_opentsne_fft_grid_size(int n) { return fe::default_grid_size(n, fe::interp_mode_from_env()); }

int fastembedr_cuda_opentsne_fft_from_knn_float(const int* indices, const float* distances, const float* init,
                                                int has_init, int n, int k, int n_components, float perplexity,
                                                int early_iter, int n_iter, float early_exag, float exag, float lr,
                                                int lr_auto, float m0, float m1, float min_gain, float max_step,
                                                unsigned int seed, int index_offset, float* out) {
  return fe::run_tsne_from_knn<float>(indices, distances, false, init, has_init, n, k, n_components, perplexity,
                                      early_iter, n_iter, early_exag, exag, lr, lr_auto, m0, m1, min_gain, max_step,
                                      seed, index_offset, out);
}

int fastembedr_cuda_opentsne_fft_from_knn(const int* indices, const double* distances, const float* init,
                                          int has_init, int n, int k, int n_components, float perplexity,
                                          int early_iter, int n_iter, float early_exag, float exag, float lr,
                                          int lr_auto, float m0, float m1, float min_gain, float max_step,
                                          unsigned int seed, int index_offset, float* out) {
  return fe::run_tsne_from_knn<double>(indices, distances, false, init, has_init, n, k, n_components, perplexity,
                                       early_iter, n_iter, early_exag, exag, lr, lr_auto, m0, m1, min_gain,
                                       max_step, seed, index_offset, out);
}

int fastembedr_cuda_opentsne_fft_from_device_knn_float(const int* indices, const float* distances,
                                                       const float* init, int has_init, int n, int k,
                                                       int n_components, float perplexity, int early_iter,
                                                       int n_iter, float early_exag, float exag, float lr,
                                                       int lr_auto, float m0, float m1, float min_gain,
                                                       float max_step, unsigned int seed, int index_offset,
                                                       float* out) {
  return fe::run_tsne_from_knn<float>(indices, distances, true, init, has_init, n, k, n_components, perplexity,
                                      early_iter, n_iter, early_exag, exag, lr, lr_auto, m0, m1, min_gain, max_step,
                                      seed, index_offset, out);
}

int fastembedr_cuda_opentsne_fft_from_device_knn_float_pca_double(
    const int* indices, const float* distances, const double* pca_init_values, int pca_init_p, int n, int k,
    int n_components, float perplexity, int early_iter, int n_iter, float early_exag, float exag, float lr,
    int lr_auto, float m0, float m1, float min_gain, float max_step, unsigned int seed, int index_offset, float* out) {
  if (!pca_init_values) return fe::guarded([] { throw fe::Error("null CUDA openTSNE input pointer"); });
  return fe::run_tsne_from_knn<float>(indices, distances, true, nullptr, 0, n, k, n_components, perplexity,
                                      early_iter, n_iter, early_exag, exag, lr, lr_auto, m0, m1, min_gain, max_step,
                                      seed, index_offset, out, pca_init_values, true, pca_init_p);
}

int fastembedr_cuda_opentsne_fft_from_device_knn_float_pca_float(
    const int* indices, const float* distances, const float* pca_init_values, int pca_init_p, int n, int k,
    int n_components, float perplexity, int early_iter, int n_iter, float early_exag, float exag, float lr,
    int lr_auto, float m0, float m1, float min_gain, float max_step, unsigned int seed, int index_offset, float* out) {
  if (!pca_init_values) return fe::guarded([] { throw fe::Error("null CUDA openTSNE input pointer"); });
  return fe::run_tsne_from_knn<float>(indices, distances, true, nullptr, 0, n, k, n_components, perplexity,
                                      early_iter, n_iter, early_exag, exag, lr, lr_auto, m0, m1, min_gain, max_step,
                                      seed, index_offset, out, pca_init_values, false, pca_init_p);
}

int fastembedr_cuda_tsne_pca_init(const void* values, int is_double, int n, int p, float* out) {
  return fe::guarded([&] {
    if (!values || !out) throw fe::Error("null host pointer");
    fe::Stream st;
    const std::vector<float> h = fe::pca_start(values, is_double != 0, n, p, st.s);
    std::copy(h.begin(), h.end(), out);
  });
}

int fastembedr_cuda_tsne_affinities(const int* indices, const float* distances, int n, int k, float perplexity,
                                    int index_offset, int* row_ptr, int* col, float* val, long long capacity,
                                    long long* nnz, float* p_directed, double* entropy, double* total_mass) {
  return fe::guarded([&] {
    if (!indices || !distances || !row_ptr || !nnz) throw fe::Error("null CUDA t-SNE affinity pointer");
    if (n < 2 || k < 1 || k > 1024 || !(perplexity > 0.0f)) throw fe::Error("invalid CUDA t-SNE affinity parameters");
    fe::Stream st;
    const std::size_t items = (std::size_t)n * k;
    int* d_idx = nullptr;
    float* d_dist = nullptr;
    float* d_p = nullptr;
    double* d_h = nullptr;
    fe::Arena a;
    a.reserve(&d_idx, items);
    a.reserve(&d_dist, items);
    a.reserve(&d_p, items);
    a.reserve(&d_h, n);
    a.commit("t-SNE affinity diagnostic");
    fe::upload(d_idx, indices, sizeof(int) * items, st.s);
    fe::upload(d_dist, distances, sizeof(float) * items, st.s);
    fe::validate_knn(d_idx, d_dist, n, k, index_offset, st.s);
    fe::row_probabilities(d_idx, d_dist, n, k, perplexity, d_p, d_h, st.s);
    fe::DeviceCsr P;
    fe::symmetrise(d_idx, d_p, n, k, index_offset, P, st.s);
    *nnz = P.nnz;
    if (total_mass) *total_mass = P.total_mass;
    FE_CUDA(cudaMemcpyAsync(row_ptr, P.row_ptr, sizeof(int) * (n + 1), cudaMemcpyDeviceToHost, st.s));
    if (col && val && P.nnz <= capacity) {
      FE_CUDA(cudaMemcpyAsync(col, P.col, sizeof(int) * P.nnz, cudaMemcpyDeviceToHost, st.s));
      FE_CUDA(cudaMemcpyAsync(val, P.val, sizeof(float) * P.nnz, cudaMemcpyDeviceToHost, st.s));
    }
    if (p_directed) FE_CUDA(cudaMemcpyAsync(p_directed, d_p, sizeof(float) * items, cudaMemcpyDeviceToHost, st.s));
    if (entropy) FE_CUDA(cudaMemcpyAsync(entropy, d_h, sizeof(double) * n, cudaMemcpyDeviceToHost, st.s));
    FE_CUDA(cudaStreamSynchronize(st.s));
  });
}

int fastembedr_cuda_tsne_force_diagnostic(const int* indices, const float* distances, const float* layout, int n,
                                          int k, float perplexity, float exaggeration, int grid_size,
                                          int interpolation, int index_offset, float* attractive, float* repulsive,
                                          double* z_grid, float* repulsive_exact, double* z_exact, double* kl) {
  return fe::guarded([&] {
    if (!indices || !distances || !layout || !attractive || !repulsive)
      throw fe::Error("null CUDA t-SNE diagnostic pointer");
    if (n < 2 || k < 1 || k > 1024 || !(perplexity > 0.0f) || !(exaggeration > 0.0f))
      throw fe::Error("invalid CUDA t-SNE diagnostic parameters");
    for (long long t = 0; t < 2LL * n; ++t)
      if (!std::isfinite(layout[t])) throw fe::Error("`layout` must contain only finite coordinates.");
    const int mode = interpolation == 0 ? fe::kInterpBilinear : fe::kInterpLagrange3;
    const int grid = grid_size > 0 ? grid_size : fe::default_grid_size(n, mode);
    if (grid < 8 || grid > 2048 || (grid & (grid - 1)) != 0)
      throw fe::Error("`grid_size` must be a power of two between 8 and 2048.");
    fe::TsneJob job;
    cudaStream_t s = job.stream.s;
    const std::size_t items = (std::size_t)n * k;
    int* d_idx = nullptr;
    float* d_dist = nullptr;
    float* d_y = nullptr;
    float* d_attr = nullptr;
    float* d_rep = nullptr;
    double* d_rex = nullptr;
    double* d_zrow = nullptr;
    double* d_work = nullptr;
    double* d_sc = nullptr;
    fe::Arena a;
    a.reserve(&d_idx, items);
    a.reserve(&d_dist, items);
    a.reserve(&d_y, 2 * (std::size_t)n);
    a.reserve(&d_attr, 2 * (std::size_t)n);
    a.reserve(&d_rep, 2 * (std::size_t)n);
    a.reserve(&d_rex, 2 * (std::size_t)n);
    a.reserve(&d_zrow, n);
    a.reserve(&d_work, n);
    a.reserve(&d_sc, 4);
    a.commit("t-SNE force diagnostic");
    fe::upload(d_idx, indices, sizeof(int) * items, s);
    fe::upload(d_dist, distances, sizeof(float) * items, s);
    FE_CUDA(cudaMemcpyAsync(d_y, layout, sizeof(float) * 2 * n, cudaMemcpyHostToDevice, s));
    FE_CUDA(cudaStreamSynchronize(s));
    job.prepare(d_idx, d_dist, layout, n, k, perplexity, index_offset, grid, mode, 0u);
    fe::tsne_forces(job.D, job.P, exaggeration, d_attr, d_rep, s);
    FE_CUDA(cudaMemcpyAsync(attractive, d_attr, sizeof(float) * 2 * n, cudaMemcpyDeviceToHost, s));
    FE_CUDA(cudaMemcpyAsync(repulsive, d_rep, sizeof(float) * 2 * n, cudaMemcpyDeviceToHost, s));
    if (z_grid) FE_CUDA(cudaMemcpyAsync(z_grid, &job.D.cur->z, sizeof(double), cudaMemcpyDeviceToHost, s));
    if (repulsive_exact || z_exact) {
      fe::exact_repulsion(d_y, n, d_rex, d_zrow, d_sc, s);
      std::vector<double> rex(2 * (std::size_t)n);
      double zt = 0.0;
      FE_CUDA(cudaMemcpyAsync(rex.data(), d_rex, sizeof(double) * 2 * n, cudaMemcpyDeviceToHost, s));
      FE_CUDA(cudaMemcpyAsync(&zt, d_sc, sizeof(double), cudaMemcpyDeviceToHost, s));
      FE_CUDA(cudaStreamSynchronize(s));
      if (repulsive_exact)
        for (long long t = 0; t < 2LL * n; ++t) repulsive_exact[t] = (float)(rex[t] / zt);
      if (z_exact) *z_exact = zt;
    }
    if (kl) {
      fe::exact_kl(job.P, d_y, nullptr, d_zrow, d_work, d_sc + 2, s);
      FE_CUDA(cudaMemcpyAsync(kl, d_sc + 3, sizeof(double), cudaMemcpyDeviceToHost, s));
    }
    FE_CUDA(cudaStreamSynchronize(s));
  });
}

int fastembedr_tsne_plan_create(const int* indices, const float* distances, const float* init, int n, int k,
                                float perplexity, int index_offset, int grid_size, int interpolation,
                                unsigned int seed, fastembedr_tsne_plan** plan) {
  return fe::guarded([&] {
    if (!indices || !distances || !plan) throw fe::Error("null CUDA t-SNE plan pointer");
    if (n < 2 || k < 1 || k > 1024 || !(perplexity > 0.0f)) throw fe::Error("invalid CUDA t-SNE plan parameters");
    const int mode = interpolation == 0 ? fe::kInterpBilinear : fe::kInterpLagrange3;
    const int grid = grid_size > 0 ? grid_size : fe::default_grid_size(n, mode);
    if (grid < 8 || grid > 2048 || (grid & (grid - 1)) != 0)
      throw fe::Error("`grid_size` must be a power of two between 8 and 2048.");
    auto p = std::make_unique<fastembedr_tsne_plan>();
    p->job.prepare(indices, distances, init, n, k, perplexity, index_offset, grid, mode, seed);
    *plan = p.release();
  });
}

int fastembedr_tsne_plan_run(fastembedr_tsne_plan* plan, int iters, float exag, float lr, float mom, float min_gain,
                             float max_step, int use_graph) {
  return fe::guarded([&] {
    if (!plan) throw fe::Error("null CUDA t-SNE plan");
    plan->job.run(iters, exag, lr, mom, min_gain, max_step, use_graph != 0);
  });
}

int fastembedr_tsne_plan_profile(fastembedr_tsne_plan* plan, int iters, float exag, float lr, float mom,
                                 float min_gain, float max_step, float* ms_total, float* ms_step_kernel,
                                 float* ms_grid_stage) {
  return fe::guarded([&] {
    if (!plan || iters < 1) throw fe::Error("invalid CUDA t-SNE profile request");
    fe::TsneJob& J = plan->job;
    cudaStream_t s = J.stream.s;
    if (J.reorder) fe::tsne_reorder(J.D, J.P, s);
    std::vector<cudaEvent_t> ev(4 * (std::size_t)iters);
    for (auto& e : ev) FE_CUDA(cudaEventCreate(&e));
    for (int it = 0; it < iters; ++it) {
      FE_CUDA(cudaEventRecord(ev[4 * it], s));
      fe::tsne_attractive_stage(J.D, J.P, exag, s);
      FE_CUDA(cudaEventRecord(ev[4 * it + 1], s));
      fe::tsne_grid_stage(J.D, s);
      FE_CUDA(cudaEventRecord(ev[4 * it + 2], s));
      fe::tsne_update_stage(J.D, lr, mom, min_gain, max_step, s);
      FE_CUDA(cudaEventRecord(ev[4 * it + 3], s));
    }
    FE_CUDA(cudaStreamSynchronize(s));
    float tot = 0.0f, stp = 0.0f, grd = 0.0f;
    for (int it = 0; it < iters; ++it) {
      float a = 0.0f, b = 0.0f;
      FE_CUDA(cudaEventElapsedTime(&a, ev[4 * it], ev[4 * it + 1]));
      FE_CUDA(cudaEventElapsedTime(&b, ev[4 * it + 1], ev[4 * it + 2]));
      stp += a;
      grd += b;
    }
    FE_CUDA(cudaEventElapsedTime(&tot, ev[0], ev[4 * (std::size_t)iters - 1]));
    for (auto& e : ev) cudaEventDestroy(e);
    if (ms_total) *ms_total = tot;
    if (ms_step_kernel) *ms_step_kernel = stp;
    if (ms_grid_stage) *ms_grid_stage = grd;
  });
}

int fastembedr_tsne_plan_tuning(fastembedr_tsne_plan* plan, int* chunk, int* blocks, int capacity, int* count,
                                int* cand_chunk, int* cand_blocks, float* cand_ms) {
  return fe::guarded([&] {
    if (!plan) throw fe::Error("null CUDA t-SNE plan");
    const fe::TsneDevice& D = plan->job.D;
    if (chunk) *chunk = D.attr_chunk;
    if (blocks) *blocks = D.attr_blocks;
    if (count) *count = (int)D.tuning.size();
    for (int t = 0; t < (int)D.tuning.size() && t < capacity; ++t) {
      if (cand_chunk) cand_chunk[t] = D.tuning[t].chunk;
      if (cand_blocks) cand_blocks[t] = D.tuning[t].blocks;
      if (cand_ms) cand_ms[t] = D.tuning[t].ms;
    }
  });
}

int fastembedr_tsne_plan_synchronize(fastembedr_tsne_plan* plan) {
  return fe::guarded([&] {
    if (!plan) throw fe::Error("null CUDA t-SNE plan");
    FE_CUDA(cudaStreamSynchronize(plan->job.stream.s));
  });
}

void* fastembedr_tsne_plan_stream(fastembedr_tsne_plan* plan) {
  return plan ? static_cast<void*>(plan->job.stream.s) : nullptr;
}

int fastembedr_tsne_plan_layout(fastembedr_tsne_plan* plan, float* out) {
  return fe::guarded([&] {
    if (!plan || !out) throw fe::Error("null CUDA t-SNE plan or output");
    plan->job.layout(out);
  });
}

int fastembedr_tsne_plan_info(fastembedr_tsne_plan* plan, long long* nnz, int* grid_size, int* interpolation,
                              int* launches, int* launches_per_reorder) {
  return fe::guarded([&] {
    if (!plan) throw fe::Error("null CUDA t-SNE plan");
    if (nnz) *nnz = plan->job.P.nnz;
    if (grid_size) *grid_size = plan->job.D.grid;
    if (interpolation) *interpolation = plan->job.D.mode;
    if (launches) *launches = fe::tsne_launches_per_iteration(plan->job.D);
    if (launches_per_reorder) *launches_per_reorder = fe::tsne_reorder_launches(plan->job.D);
  });
}

int fastembedr_tsne_plan_kl(fastembedr_tsne_plan* plan, double* kl) {
  return fe::guarded([&] {
    if (!plan || !kl) throw fe::Error("null CUDA t-SNE plan or output");
    fe::TsneJob& J = plan->job;
    cudaStream_t s = J.stream.s;
    const int n = J.D.n;
    float* d_y = nullptr;
    double* d_zrow = nullptr;
    double* d_work = nullptr;
    double* d_sc = nullptr;
    fe::Arena a;
    a.reserve(&d_y, 2 * (std::size_t)n);
    a.reserve(&d_zrow, n);
    a.reserve(&d_work, n);
    a.reserve(&d_sc, 2);
    a.commit("t-SNE KL");
    fe::exact_kl(J.P, reinterpret_cast<const float*>(J.D.y), J.D.inv, d_zrow, d_work, d_sc, s);
    FE_CUDA(cudaMemcpyAsync(kl, d_sc + 1, sizeof(double), cudaMemcpyDeviceToHost, s));
    FE_CUDA(cudaStreamSynchronize(s));
  });
}

int fastembedr_tsne_plan_gradient_check(fastembedr_tsne_plan* plan, const int* rows, int n_rows,
                                        float exaggeration, float* attractive, float* repulsive_grid,
                                        double* repulsive_exact, double* z_grid, double* z_exact) {
  return fe::guarded([&] {
    if (!plan || !rows || !attractive || !repulsive_grid || !repulsive_exact)
      throw fe::Error("null CUDA t-SNE gradient check pointer");
    fe::TsneJob& J = plan->job;
    const int n = J.D.n;
    if (n_rows < 1 || n_rows > n || !(exaggeration > 0.0f)) throw fe::Error("invalid CUDA t-SNE gradient check");
    for (int r = 0; r < n_rows; ++r)
      if (rows[r] < 0 || rows[r] >= n) throw fe::Error("gradient check row out of range");
    if (J.D.inst.size() != 1) throw fe::Error("gradient check needs a single-instance plan");
    cudaStream_t s = J.stream.s;
    const int slices = fe::exact_rows_slices(n, n_rows);
    int* d_rows = nullptr;
    float2* d_attr = nullptr;
    float2* d_rep = nullptr;
    float2* d_attr_rows = nullptr;
    float2* d_rep_rows = nullptr;
    double* d_part = nullptr;
    double* d_out = nullptr;
    double* d_zrow = nullptr;
    double* d_sc = nullptr;
    fe::Arena a;
    a.reserve(&d_rows, n_rows);
    a.reserve(&d_attr, n);
    a.reserve(&d_rep, n);
    a.reserve(&d_attr_rows, n_rows);
    a.reserve(&d_rep_rows, n_rows);
    a.reserve(&d_part, (std::size_t)slices * 3 * n_rows);
    a.reserve(&d_out, 3 * (std::size_t)n_rows);
    a.reserve(&d_zrow, n);
    a.reserve(&d_sc, 2);
    a.commit("t-SNE gradient check");
    FE_CUDA(cudaMemcpyAsync(d_rows, rows, sizeof(int) * n_rows, cudaMemcpyHostToDevice, s));
    // the grid forces of the current layout (the optimizer state is left as it was)
    fe::tsne_forces(J.D, J.P, exaggeration, reinterpret_cast<float*>(d_attr), reinterpret_cast<float*>(d_rep), s);
    FE_CUDA(cudaMemcpyAsync(d_sc + 1, &J.D.cur->z, sizeof(double), cudaMemcpyDeviceToDevice, s));
    fe::gather_rows_kernel<<<std::max(1, std::min(fe::ceil_div(n_rows, 256), fe::sm_count() * 4)), 256, 0, s>>>(
        d_attr, d_rep, d_rows, J.D.inv, n_rows, d_attr_rows, d_rep_rows);
    FE_LAUNCH("gather_rows_kernel");
    fe::exact_repulsion_rows(reinterpret_cast<const float*>(J.D.y), n, d_rows, J.D.inv, n_rows, d_part, d_out, d_zrow,
                             d_sc, s);
    std::vector<double> ex(3 * (std::size_t)n_rows);
    double zs[2] = {0.0, 0.0};
    FE_CUDA(cudaMemcpyAsync(attractive, d_attr_rows, sizeof(float2) * n_rows, cudaMemcpyDeviceToHost, s));
    FE_CUDA(cudaMemcpyAsync(repulsive_grid, d_rep_rows, sizeof(float2) * n_rows, cudaMemcpyDeviceToHost, s));
    FE_CUDA(cudaMemcpyAsync(ex.data(), d_out, sizeof(double) * ex.size(), cudaMemcpyDeviceToHost, s));
    FE_CUDA(cudaMemcpyAsync(zs, d_sc, sizeof(zs), cudaMemcpyDeviceToHost, s));
    FE_CUDA(cudaStreamSynchronize(s));
    for (int r = 0; r < n_rows; ++r) {
      repulsive_exact[2 * (std::size_t)r] = ex[r] / zs[0];
      repulsive_exact[2 * (std::size_t)r + 1] = ex[(std::size_t)n_rows + r] / zs[0];
    }
    if (z_exact) *z_exact = zs[0];
    if (z_grid) *z_grid = zs[1];
  });
}

void fastembedr_tsne_plan_destroy(fastembedr_tsne_plan* plan) { delete plan; }

// ---------------------------------------------------------------- batches
int fastembedr_tsne_batch_create(int n_instances, const int* sizes, const int* indices, const float* distances,
                                 const float* init, int k, float perplexity, int index_offset, int grid_size,
                                 int interpolation, unsigned int seed, fastembedr_tsne_batch** batch) {
  return fe::guarded([&] {
    if (!sizes || !indices || !distances || !batch) throw fe::Error("null CUDA t-SNE batch pointer");
    if (n_instances < 1 || k < 1 || k > 1024 || !(perplexity > 0.0f))
      throw fe::Error("invalid CUDA t-SNE batch parameters");
    if (grid_size > 0 && (grid_size < 8 || grid_size > 2048 || (grid_size & (grid_size - 1)) != 0))
      throw fe::Error("`grid_size` must be a power of two between 8 and 2048.");
    if (grid_size < -2)
      throw fe::Error("`grid_size`: 0 (CUDA size policy), -1 (CPU size policy), -2 (adaptive) or a size");
    const int mode = interpolation == 0 ? fe::kInterpBilinear : fe::kInterpLagrange3;
    auto b = std::make_unique<fastembedr_tsne_batch>();
    b->job.configure_adaptive(grid_size == -2);
    b->job.prepare_batch(n_instances, sizes, indices, distances, init, k, perplexity, index_offset, grid_size, mode,
                         seed);
    *batch = b.release();
  });
}

int fastembedr_tsne_batch_create_rows(int n_instances, const int* sizes, const int* const* indices,
                                      const float* const* distances, const float* const* inits, int k,
                                      float perplexity, int index_offset, int grid_size, int interpolation,
                                      unsigned int seed, fastembedr_tsne_batch** batch) {
  return fe::guarded([&] {
    if (!sizes || !indices || !distances || !batch) throw fe::Error("null CUDA t-SNE batch pointer");
    if (n_instances < 1 || k < 1 || k > 1024 || !(perplexity > 0.0f))
      throw fe::Error("invalid CUDA t-SNE batch parameters");
    if (grid_size > 0 && (grid_size < 8 || grid_size > 2048 || (grid_size & (grid_size - 1)) != 0))
      throw fe::Error("`grid_size` must be a power of two between 8 and 2048.");
    if (grid_size < -2)
      throw fe::Error("`grid_size`: 0 (CUDA size policy), -1 (CPU size policy), -2 (adaptive) or a size");
    std::vector<const int*> iu(indices, indices + n_instances);
    std::vector<const float*> du(distances, distances + n_instances);
    std::vector<const float*> yu;
    if (inits) yu.assign(inits, inits + n_instances);
    for (int u = 0; u < n_instances; ++u)
      if (!iu[u] || !du[u] || (inits && !yu[u])) throw fe::Error("null CUDA t-SNE batch pointer");
    const int mode = interpolation == 0 ? fe::kInterpBilinear : fe::kInterpLagrange3;
    auto b = std::make_unique<fastembedr_tsne_batch>();
    b->job.configure_adaptive(grid_size == -2);
    b->job.prepare_batch(n_instances, sizes, iu, du, yu, true, k, perplexity, index_offset, grid_size, mode, seed);
    *batch = b.release();
  });
}

int fastembedr_tsne_batch_iterate(fastembedr_tsne_batch* batch, int iters, float exaggeration, float learning_rate,
                                  float momentum, float min_gain, float max_step_norm) {
  return fe::guarded([&] {
    if (!batch || iters < 0) throw fe::Error("invalid CUDA t-SNE batch run");
    batch->job.run(iters, exaggeration, learning_rate, momentum, min_gain, max_step_norm, true);
  });
}

int fastembedr_tsne_batch_run(fastembedr_tsne_batch* batch, int early_exaggeration_iter, int n_iter,
                              float early_exaggeration, float exaggeration, float learning_rate,
                              float initial_momentum, float final_momentum, float min_gain, float max_step_norm) {
  return fe::guarded([&] {
    if (!batch || early_exaggeration_iter < 0 || n_iter < 0 || !(early_exaggeration > 0.0f) ||
        !(exaggeration > 0.0f) || !(min_gain > 0.0f))
      throw fe::Error("invalid CUDA t-SNE batch schedule");
    fe::TsneJob& J = batch->job;
    if (learning_rate > 0.0f) {
      J.run(early_exaggeration_iter, early_exaggeration, learning_rate, initial_momentum, min_gain, max_step_norm,
            true);
      J.run(n_iter, exaggeration, learning_rate, final_momentum, min_gain, max_step_norm, true);
    } else {
      // opt-SNE rate of the package's auto configuration, n_b / early_exaggeration in both phases,
      // rounded once to float exactly as the one-instance path rounds it (so an instance of the
      // batch takes the same steps as tsne_knn on its own)
      std::vector<float> per(J.D.inst.size()), plain(J.D.inst.size());
      for (std::size_t t = 0; t < per.size(); ++t) {
        plain[t] = (float)J.D.inst[t].n;
        per[t] = (float)((double)J.D.inst[t].n / (double)early_exaggeration);
      }
      J.set_lr_mult(per);
      J.run(early_exaggeration_iter, early_exaggeration, 1.0f, initial_momentum, min_gain, max_step_norm, true);
      J.run(n_iter, exaggeration, 1.0f, final_momentum, min_gain, max_step_norm, true);
      J.set_lr_mult(plain);
    }
    FE_CUDA(cudaStreamSynchronize(J.stream.s));
  });
}

int fastembedr_tsne_batch_synchronize(fastembedr_tsne_batch* batch) {
  return fe::guarded([&] {
    if (!batch) throw fe::Error("null CUDA t-SNE batch");
    FE_CUDA(cudaStreamSynchronize(batch->job.stream.s));
  });
}

void* fastembedr_tsne_batch_stream(fastembedr_tsne_batch* batch) {
  return batch ? static_cast<void*>(batch->job.stream.s) : nullptr;
}

int fastembedr_tsne_batch_layout(fastembedr_tsne_batch* batch, float* out) {
  return fe::guarded([&] {
    if (!batch || !out) throw fe::Error("null CUDA t-SNE batch or output");
    fe::TsneJob& J = batch->job;
    cudaStream_t s = J.stream.s;
    float* d_out = nullptr;
    fe::Arena tmp;
    tmp.reserve(&d_out, 2 * (std::size_t)J.D.n);
    tmp.commit("t-SNE batch output");
    fe::tsne_finalize(J.D, d_out, s);
    for (std::size_t t = 0; t < J.user.size(); ++t) {
      const int u = J.user[t];
      FE_CUDA(cudaMemcpyAsync(out + 2 * (std::size_t)J.user_off[u], d_out + 2 * (std::size_t)J.D.inst[t].pt_begin,
                              sizeof(float) * 2 * J.D.inst[t].n, cudaMemcpyDeviceToHost, s));
    }
    FE_CUDA(cudaStreamSynchronize(s));
  });
}

int fastembedr_tsne_batch_kl(fastembedr_tsne_batch* batch, int instance, double* kl) {
  return fe::guarded([&] {
    if (!batch || !kl) throw fe::Error("null CUDA t-SNE batch or output");
    fe::TsneJob& J = batch->job;
    if (instance < 0 || instance >= (int)J.user.size()) throw fe::Error("t-SNE batch: instance out of range");
    int t = 0;
    while (J.user[t] != instance) ++t;
    const fe::TsneInstance& I = J.D.inst[t];
    cudaStream_t s = J.stream.s;
    double *d_zrow = nullptr, *d_work = nullptr, *d_sc = nullptr;
    fe::Arena a;
    a.reserve(&d_zrow, I.n);
    a.reserve(&d_work, I.n);
    a.reserve(&d_sc, 2);
    a.commit("t-SNE batch KL");
    fe::exact_kl_range(J.P.row_ptr + I.pt_begin, J.P.col, J.P.val, I.n, reinterpret_cast<const float*>(J.D.y),
                       J.D.inv + I.pt_begin, I.pt_begin, d_zrow, d_work, d_sc, s);
    FE_CUDA(cudaMemcpyAsync(kl, d_sc + 1, sizeof(double), cudaMemcpyDeviceToHost, s));
    FE_CUDA(cudaStreamSynchronize(s));
  });
}

int fastembedr_tsne_batch_info(fastembedr_tsne_batch* batch, long long* nnz, long long* points, int* grid_classes,
                               int* launches_per_iteration, int* launches_per_reorder) {
  return fe::guarded([&] {
    if (!batch) throw fe::Error("null CUDA t-SNE batch");
    fe::TsneJob& J = batch->job;
    if (nnz) *nnz = J.P.nnz;
    if (points) *points = J.D.n;
    if (grid_classes) *grid_classes = (int)J.D.classes.size();
    if (launches_per_iteration) *launches_per_iteration = fe::tsne_launches_per_iteration(J.D);
    if (launches_per_reorder) *launches_per_reorder = fe::tsne_reorder_launches(J.D);
  });
}

int fastembedr_tsne_batch_grids(fastembedr_tsne_batch* batch, int* grids, int* regrids) {
  return fe::guarded([&] {
    if (!batch) throw fe::Error("null CUDA t-SNE batch");
    fe::TsneJob& J = batch->job;
    if (grids)
      for (std::size_t t = 0; t < J.user.size(); ++t) grids[J.user[t]] = J.D.inst[t].grid;
    if (regrids) *regrids = J.regrids;
  });
}

void fastembedr_tsne_batch_destroy(fastembedr_tsne_batch* batch) { delete batch; }

int fastembedr_cuda_tsne_batch_from_knn(int n_instances, const int* sizes, const int* indices, const float* distances,
                                        const float* init, int k, float perplexity, int early_exaggeration_iter,
                                        int n_iter, float early_exaggeration, float exaggeration, float learning_rate,
                                        float initial_momentum, float final_momentum, float min_gain,
                                        float max_step_norm, unsigned int seed, int index_offset, float* out) {
  fastembedr_tsne_batch* b = nullptr;
  int st = fastembedr_tsne_batch_create(n_instances, sizes, indices, distances, init, k, perplexity, index_offset, 0,
                                        fe::interp_mode_from_env(), seed, &b);
  if (st == 0)
    st = fastembedr_tsne_batch_run(b, early_exaggeration_iter, n_iter, early_exaggeration, exaggeration,
                                   learning_rate, initial_momentum, final_momentum, min_gain, max_step_norm);
  if (st == 0) st = fastembedr_tsne_batch_layout(b, out);
  fastembedr_tsne_batch_destroy(b);
  return st;
}

}  // extern "C"
