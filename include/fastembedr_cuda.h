/*
 * fastEmbedR GB300 embedding optimizer: C ABI.
 *
 * Drop-in replacement for the extern "C" layer of fastEmbedR
 * src/embedding_cuda_kernels.cpp that src/embedding_cuda_impl.cpp calls. Same names,
 * argument order and meaning; same status convention: every int-returning entry point
 * returns 0 on success and 1 on failure, and the message of the last failure on the calling
 * thread is returned by fastembedr_cuda_embedding_last_error().
 *
 * Layouts (as in the reference):
 *   - KNN indices / distances: column-major n x k (element (i, j) at j * n + i), as R stores
 *     matrices; indices carry `index_offset` (0- or 1-based).
 *   - init / out layouts: row-major interleaved (x, y) floats, n * 2 values.
 * Host pointers unless the name says device. Entry points are synchronous: when they return,
 * outputs are written and all device memory they allocated is released.
 */
#ifndef FASTEMBEDR_CUDA_H
#define FASTEMBEDR_CUDA_H

#include <stdbool.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- runtime */

/* replaces fastembedr_cuda_available, src/embedding_cuda_kernels.cpp:3833-3841 */
bool fastembedr_cuda_available(void);

/* replaces fastembedr_cuda_embedding_last_error, src/embedding_cuda_kernels.cpp:3829-3831 */
const char* fastembedr_cuda_embedding_last_error(void);

/* replaces fastembedr_cuda_opentsne_fft_grid_size, src/embedding_cuda_kernels.cpp:5625-5627:
 * grid nodes per side, 256 (n < 20k) / 512 / 1024 (n >= 100k), FASTEMBEDR_TSNE_FFT_GRID override */
int fastembedr_cuda_opentsne_fft_grid_size(int n);

/* ---------------------------------------------------------------- t-SNE from KNN */

/* replaces fastembedr_cuda_opentsne_fft_from_knn_float, src/embedding_cuda_kernels.cpp:6207-6234.
 * Perplexity affinities, symmetrised CSR P, then early_exaggeration_iter + n_iter iterations of
 * the gains/momentum optimizer with FFT-grid repulsion (grid nodes per side from
 * fastembedr_cuda_opentsne_fft_grid_size). learning_rate_auto: lr = n / exaggeration
 * of each phase. max_step_norm <= 0 or non-finite disables the step clip. has_init = 0 draws a
 * seeded N(0, 1e-4^2) layout. Repulsion interpolation: the reference's bilinear stencil;
 * FASTEMBEDR_TSNE_INTERPOLATION=lagrange selects 3-node Lagrange boxes. */
int fastembedr_cuda_opentsne_fft_from_knn_float(const int* indices, const float* distances, const float* init,
                                                int has_init, int n, int k, int n_components, float perplexity,
                                                int early_exaggeration_iter, int n_iter, float early_exaggeration,
                                                float exaggeration, float learning_rate, int learning_rate_auto,
                                                float initial_momentum, float final_momentum, float min_gain,
                                                float max_step_norm, unsigned int seed, int index_offset,
                                                float* out);

/* replaces fastembedr_cuda_opentsne_fft_from_knn (double distances), src/embedding_cuda_kernels.cpp:6178-6205 */
int fastembedr_cuda_opentsne_fft_from_knn(const int* indices, const double* distances, const float* init,
                                          int has_init, int n, int k, int n_components, float perplexity,
                                          int early_exaggeration_iter, int n_iter, float early_exaggeration,
                                          float exaggeration, float learning_rate, int learning_rate_auto,
                                          float initial_momentum, float final_momentum, float min_gain,
                                          float max_step_norm, unsigned int seed, int index_offset, float* out);

/* replaces fastembedr_cuda_opentsne_fft_from_device_knn_float, src/embedding_cuda_kernels.cpp:6236-6263:
 * indices / distances are device pointers (column-major), init and out are host pointers. */
int fastembedr_cuda_opentsne_fft_from_device_knn_float(const int* indices, const float* distances,
                                                       const float* init, int has_init, int n, int k,
                                                       int n_components, float perplexity,
                                                       int early_exaggeration_iter, int n_iter,
                                                       float early_exaggeration, float exaggeration,
                                                       float learning_rate, int learning_rate_auto,
                                                       float initial_momentum, float final_momentum,
                                                       float min_gain, float max_step_norm, unsigned int seed,
                                                       int index_offset, float* out);

/* replace fastembedr_cuda_opentsne_fft_from_device_knn_float_pca_double / _pca_float
 * (src/embedding_cuda_kernels.cpp:6265-6321, bound by src/embedding_cuda_impl.cpp:2480-2570): the
 * device-KNN entry above with the start computed on the GPU from the data: pca_init_values is a
 * HOST column-major n x pca_init_p matrix (double or float). The two leading principal components
 * (covariance of the centred data, Jacobi eigendecomposition in FP64; the reference calls RAPIDS
 * RAFT's tsvd_fit_transform with the covariance-eigen solver) give the scores; each score column is
 * signed so its largest-magnitude entry is positive, centred, and both are scaled by 1e-4 / the
 * larger standard deviation (src/embedding_cuda_kernels.cpp:1337-1420). pca_init_p <= 1024. */
int fastembedr_cuda_opentsne_fft_from_device_knn_float_pca_double(
    const int* indices, const float* distances, const double* pca_init_values, int pca_init_p, int n, int k,
    int n_components, float perplexity, int early_exaggeration_iter, int n_iter, float early_exaggeration,
    float exaggeration, float learning_rate, int learning_rate_auto, float initial_momentum, float final_momentum,
    float min_gain, float max_step_norm, unsigned int seed, int index_offset, float* out);
int fastembedr_cuda_opentsne_fft_from_device_knn_float_pca_float(
    const int* indices, const float* distances, const float* pca_init_values, int pca_init_p, int n, int k,
    int n_components, float perplexity, int early_exaggeration_iter, int n_iter, float early_exaggeration,
    float exaggeration, float learning_rate, int learning_rate_auto, float initial_momentum, float final_momentum,
    float min_gain, float max_step_norm, unsigned int seed, int index_offset, float* out);
/* The PCA start alone (no reference counterpart as an entry point): host column-major n x p data
 * (is_double: double, else float) -> out, host row-major n x 2 floats. */
int fastembedr_cuda_tsne_pca_init(const void* values, int is_double, int n, int p, float* out);

/* ---------------------------------------------------------------- UMAP */

/* replaces fastembedr_cuda_umap_optimize_coo, src/embedding_cuda_kernels.cpp:5483-5608.
 * COO graph (heads, tails, weights, epochs_per_sample; n_edges_capacity entries, as
 * umap_cuda_optimize_csr_cpp expands the CSR, src/embedding_cuda_bridge.cpp:346-378) and a
 * row-major n x 2 init; n_epochs SGD epochs with the reference schedule (epoch 0 inactive,
 * linear learning-rate decay, gradient clip 4, clamp to +-16 after every epoch). Negative
 * samples come from counter-based Philox streams keyed by (seed, edge, epoch). Only
 * optimizer_mode 0 (the package policy) is provided. */
int fastembedr_cuda_umap_optimize_coo(const int* heads, const int* tails, const float* weights,
                                      const float* epochs_per_sample, const float* init, int n, int n_edges_capacity,
                                      int n_epochs, int negative_sample_rate, float learning_rate, float a, float b,
                                      float repulsion_strength, unsigned int seed, int optimizer_mode, float* out);

/* GPU twin of umap_graph_csr_float_cpp (src/fast_knn_umap.cpp:3996-4052): the default fuzzy
 * graph from column-major KNN (offsets n + 1; neighbors / weights / epochs_per_sample up to
 * `capacity` entries, neighbours ascending per row); *nnz and *max_weight returned. */
int fastembedr_cuda_umap_graph_from_knn(const int* indices, const float* distances, int n, int k, int index_offset,
                                        int* offsets, int* neighbors, float* weights, float* epochs_per_sample,
                                        long long capacity, long long* nnz, float* max_weight);

/* No reference counterpart (the reference computes this start on the CPU even for the CUDA
 * backend: spectral_knn_init(backend = "cpu"), R/fast_knn_umap.R:1343-1365, used by
 * initialize_umap_gpu_host_knn, R/umap_core_helpers.R:205-243). GPU twin of fast_knn_umap_range_cpp
 * with n_epochs = 0 (src/fast_knn_umap.cpp:4461-4501): the fuzzy graph of the column-major n x k
 * KNN, then initialize_layout_csr (:2231-2528) with the reference's std::mt19937(seed) draws and
 * scale_embedding_sdev(init_scale) when init_scale is finite and > 0 (:2681-2703). out: host,
 * column-major n x 2 doubles (an R NumericMatrix). Sums over points are reduced in a fixed block
 * order instead of sequentially, so results equal the CPU start to rounding. */
int fastembedr_cuda_umap_spectral_init_from_knn(const int* indices, const float* distances, int n, int k,
                                                int index_offset, int spectral_n_iter, double init_scale, int seed,
                                                double* out);
/* The same start from a CSR graph (host arrays): the GPU twin of fast_knn_umap_csr_cpp with
 * n_epochs = 0 (src/fast_knn_umap.cpp:5291-5321, as umap_init_from_csr_graph calls it,
 * R/fast_knn_umap.R:665-689). Inputs are checked as validate_csr_inputs does (:747-785; 0- or
 * 1-based neighbours) and must be symmetric (w_ij == w_ji, as every UMAP fuzzy or binary graph
 * is). out: host, column-major n x 2 doubles. */
int fastembedr_cuda_umap_spectral_init_csr(const int* offsets, const int* neighbors, const float* weights, int n,
                                           int spectral_n_iter, double init_scale, int seed, double* out);
/* No reference counterpart: umap_knn(backend = "cuda") with the start above computed on the GPU
 * instead of the CPU (R/umap_core_helpers.R:205-243 then fastembedr_cuda_umap_optimize_coo): KNN ->
 * fuzzy graph -> spectral start -> n_epochs SGD epochs (min_dist through find_ab_params), one
 * seed for both as in the reference. out: row-major n x 2 host floats. */
int fastembedr_cuda_umap_knn_spectral(const int* indices, const float* distances, int n, int k, int index_offset,
                                      int n_epochs, int negative_sample_rate, float learning_rate, float min_dist,
                                      float repulsion_strength, int spectral_n_iter, double init_scale,
                                      unsigned int seed, float* out);

/* find_ab_params (src/fast_knn_umap.cpp:437-497), the curve a, b that the reference's bridges
 * compute on the host before calling the fused UMAP entry points below (host code, no GPU). */
void fastembedr_umap_find_ab_params(double spread, double min_dist, double* a, double* b);

/* No reference counterpart (diagnostic, host code, no GPU): 1 when the multi-threaded normal draws
 * of the spectral start reproduce std::normal_distribution<double> on std::mt19937 bit for bit on
 * this platform (checked once at first use), 0 when the start falls back to drawing through
 * std::normal_distribution itself. Either way the draws equal the reference's. */
int fastembedr_host_normal_stream_check(void);

/* replaces fastembedr_cuda_spectral_init_from_knn, src/embedding_cuda_kernels.cpp:4801-4960
 * (bound by spectral_knn_init_cuda_impl, src/embedding_cuda_impl.cpp:1589-1628): the diffusion
 * start of initialize_layout_csr_cuda_diffusion (src/fast_knn_umap.cpp:2597-2652) over the fuzzy
 * graph of the column-major n x k KNN (the graph of fastembedr_cuda_umap_graph_from_knn, every
 * union entry kept). out: row-major n x 2 floats, whitened (zero mean, unit-norm x, y orthogonal
 * to x with unit norm). Requires 2 <= n, 1 <= k <= 256, spectral_n_iter >= 1. */
int fastembedr_cuda_spectral_init_from_knn(const int* indices, const double* distances, int n, int k,
                                           int spectral_n_iter, unsigned int seed, int index_offset, float* out);

/* replace fastembedr_cuda_umap_from_knn_spectral / _float (src/embedding_cuda_kernels.cpp:5360-5449,
 * bound by knn_umap_cuda_fused_impl / _float_impl / _gpu_impl, src/embedding_cuda_impl.cpp:1716-1900)
 * and fastembedr_cuda_umap_from_device_knn_spectral_float
 * (:5462-5481, device KNN pointers): KNN -> fuzzy graph (unit weights with binary_graph) ->
 * diffusion start (spectral_n_iter rounds, seed) -> n_epochs SGD epochs with curve a, b, all on
 * the GPU. out: row-major n x 2 host floats. Only optimizer_mode 0 (the package policy) is
 * provided. */
int fastembedr_cuda_umap_from_knn_spectral(const int* indices, const double* distances, int n, int k, int n_epochs,
                                           int negative_sample_rate, float learning_rate, float a, float b,
                                           float repulsion_strength, int spectral_n_iter, unsigned int seed,
                                           int index_offset, int optimizer_mode, float* out);
int fastembedr_cuda_umap_from_knn_spectral_float(const int* indices, const float* distances, int n, int k,
                                                 int n_epochs, int negative_sample_rate, float learning_rate, float a,
                                                 float b, float repulsion_strength, int spectral_n_iter,
                                                 unsigned int seed, int index_offset, int optimizer_mode, float* out);
int fastembedr_cuda_umap_from_device_knn_spectral_float(const int* device_indices, const float* device_distances,
                                                        int n, int k, int n_epochs, int negative_sample_rate,
                                                        float learning_rate, float a, float b,
                                                        float repulsion_strength, int spectral_n_iter,
                                                        unsigned int seed, int index_offset, int optimizer_mode,
                                                        int binary_graph, float* out);

/* No reference counterpart (the reference builds the graph on the host): KNN -> fuzzy graph ->
 * SGD entirely on the GPU, with a/b from the package's min_dist policy (spread 1). */
int fastembedr_cuda_umap_from_knn(const int* indices, const float* distances, const float* init, int n, int k,
                                  int index_offset, int n_epochs, int negative_sample_rate, float learning_rate,
                                  float min_dist, float repulsion_strength, unsigned int seed, float* out);
/* No reference counterpart: many UMAP instances in one job. Each instance's fuzzy graph is built
 * on its own and appended (vertices offset by the instance's first point); every epoch is one
 * launch over all edges (negatives drawn inside the edge's own instance, Philox keyed by the
 * instance-local edge, so an instance draws the same negatives alone and in a batch) and one
 * clamp launch. sizes[b] points; indices / distances: each instance's column-major n_b x k KNN
 * one after another (index_offset per instance); init / out: row-major n_b x 2 per instance one
 * after another. sgd_ms (may be NULL): device time of the epochs. */
int fastembedr_cuda_umap_batch_from_knn(int n_instances, const int* sizes, const int* indices, const float* distances,
                                        const float* init, int k, int index_offset, int n_epochs,
                                        int negative_sample_rate, float learning_rate, float min_dist,
                                        float repulsion_strength, unsigned int seed, float* out, float* sgd_ms);
/* No reference counterpart: the same batched UMAP job from one host pointer per instance, so a
 * host whose instances sit in separate arrays makes no concatenated copy: indices[b] /
 * distances[b] row-major (C order) n_b x k, inits[b] and outs[b] row-major n_b x 2. */
int fastembedr_cuda_umap_batch_from_knn_rows(int n_instances, const int* sizes, const int* const* indices,
                                             const float* const* distances, const float* const* inits, int k,
                                             int index_offset, int n_epochs, int negative_sample_rate,
                                             float learning_rate, float min_dist, float repulsion_strength,
                                             unsigned int seed, float* const* outs, float* sgd_ms);
/* The same job, reporting device time (CUDA events on the job's stream) of the graph build and
 * of the n_epochs SGD epochs; either output may be NULL. */
int fastembedr_cuda_umap_from_knn_profile(const int* indices, const float* distances, const float* init, int n,
                                          int k, int index_offset, int n_epochs, int negative_sample_rate,
                                          float learning_rate, float min_dist, float repulsion_strength,
                                          unsigned int seed, float* out, float* graph_ms, float* sgd_ms);

/* ---------------------------------------------------------------- t-SNE diagnostics */

/* GPU twin of the affinity part of opentsne_force_diagnostic_cpp
 * (src/tsne_neighbors.cpp:1698-1817; build_tsne_probabilities_float :616-724).
 * Writes the symmetrised CSR (row_ptr n + 1, col / val up to `capacity`), its size in *nnz and
 * the directed-mass total; p_directed (row-major n x k) and entropy (n) may be NULL. */
int fastembedr_cuda_tsne_affinities(const int* indices, const float* distances, int n, int k, float perplexity,
                                    int index_offset, int* row_ptr, int* col, float* val, long long capacity,
                                    long long* nnz, float* p_directed, double* entropy, double* total_mass);

/* GPU twin of the force part of opentsne_force_diagnostic_cpp (src/tsne_neighbors.cpp:1698-1817):
 * on `layout` (row-major n x 2) computes the attractive force (exaggeration-scaled), the grid
 * repulsion with grid_size nodes per side (interpolation 0 = bilinear, 1 = Lagrange; grid_size
 * <= 0 uses the CUDA policy) and its Z; optionally (repulsive_exact != NULL) the exact
 * repulsion with the all-pairs Z, and the KL (kl != NULL). */
int fastembedr_cuda_tsne_force_diagnostic(const int* indices, const float* distances, const float* layout,
                                          int n, int k, float perplexity, float exaggeration, int grid_size,
                                          int interpolation, int index_offset, float* attractive,
                                          float* repulsive, double* z_grid, float* repulsive_exact,
                                          double* z_exact, double* kl);

/* Exact t-SNE repulsion that allocates no device memory. No counterpart in the reference.
 * For callers that cannot call cudaMalloc where they need the result (the GPU's memory is owned
 * by another framework's pool, or a serving loop forbids allocation on its request path).
 * layout (row-major n x 2 floats), repulsive (n x 2 floats) and sum_q (1 double, may be NULL) are
 * caller-owned DEVICE pointers (layout 8-byte aligned); the working memory is a fixed 1.5 MB array
 * inside the library, so n <= 65536 (larger n is rejected with an error). The first call on a
 * device loads that array onto the device (CUDA loads modules lazily) and resolves its address:
 * make it before a memory pool reserves the device's free memory and before any stream capture.
 * Every call reuses the same array, so calls that overlap on the GPU race and must be serialised
 * by the caller. `stream` is a
 * cudaStream_t (NULL: the legacy default stream); the call returns after the stream has finished.
 * Output equals the repulsive_exact / z_exact of fastembedr_cuda_tsne_force_diagnostic. */
int fastembedr_cuda_tsne_exact_repulsion_noalloc(const float* layout, int n, float* repulsive, double* sum_q,
                                                 void* stream);

/* ---------------------------------------------------------------- fixed-reference transform
 * Replaces transform_tsne_cuda_cpp, which R/transform_tsne.R:272-289 calls for
 * transform_tsne(backend = "cuda") but which the reference never defines; arguments follow
 * transform_tsne_cpp (src/tsne_neighbors.cpp:2124-2144) minus n_threads / batch_size / verbose.
 * Matrices are R layout (column-major doubles): reference_layout n_reference x 2, indices /
 * distances n_query x k (1- or 0-based, detected as resolve_reference_index_offset does),
 * y_init n_query x 2 when init != 0, out n_query x 2. initialization: "median" or "weighted"
 * when init == 0. Repulsion is exact for n_reference <= exact_repulsion_threshold, else
 * n_negatives references per query and iteration from the reference's xorshift32 stream.
 * Host pointers; returns after the result is in `out`. */
int fastembedr_cuda_transform_tsne(const double* reference_layout, int n_reference, const int* indices,
                                   const double* distances, int n_query, int k, const double* y_init, int init,
                                   const char* initialization, double perplexity, int n_iter,
                                   int early_exaggeration_iter, double learning_rate, double early_exaggeration,
                                   double exaggeration, double initial_momentum, double final_momentum,
                                   double max_grad_norm, double max_step_norm, int n_negatives,
                                   int exact_repulsion_threshold, int seed, double* out);

/* replaces fastembedr_cuda_landmark_tsne_from_device_knn, src/embedding_cuda_kernels.cpp:3572-3686
 * (project_landmark_model's CUDA route, landmark_tsne_transform_cuda_gpu_cpp,
 * src/embedding_cuda_bridge.cpp:584-612). device_indices / device_distances: device pointers,
 * column-major n_query x k (k <= 128); reference_data (n_reference x n_features), query_data
 * (n_query x n_features) and reference_layout (n_reference x 2): host, column-major float.
 * Each query starts at the ridge-regularised local affine projection of its first
 * affine_neighbors (3..12) landmarks, displacement bounded by max_extrapolation times their
 * layout radius, then runs the fixed-reference iterations with the landmark hash sampler
 * (n_negatives per query and iteration; exact when n_reference <= exact_repulsion_threshold).
 * out: host, row-major n_query x 2 floats. */
int fastembedr_cuda_landmark_tsne_from_device_knn(const int* device_indices, const float* device_distances,
                                                  int index_offset, const float* reference_data,
                                                  const float* query_data, const float* reference_layout,
                                                  int n_reference, int n_query, int n_features, int k,
                                                  float perplexity, int n_iter, int early_exaggeration_iter,
                                                  float learning_rate, float early_exaggeration, float exaggeration,
                                                  float initial_momentum, float final_momentum, float max_grad_norm,
                                                  float max_step_norm, int n_negatives, int exact_repulsion_threshold,
                                                  unsigned int seed, int affine_neighbors, float affine_ridge,
                                                  float max_extrapolation, float* out);

/* ---------------------------------------------------------------- transform serving loop
 * No counterpart in the reference: fastembedr_cuda_landmark_tsne_from_device_knn
 * (src/embedding_cuda_kernels.cpp:3572-3686) uploads the reference and rebuilds its state on
 * every call. A server keeps the reference layout resident, accepts query batches from any
 * thread, admits them in arrival order while their device memory fits `memory_budget_bytes`
 * (0: 40 GiB, capped by free memory) and one of `max_inflight` streams is free, and runs each
 * admitted group of requests as one merged launch. Options are those of
 * fastembedr_cuda_transform_tsne, fixed per server. Each result equals the one-shot transform
 * of the same request bit for bit, whatever else is in flight. */
typedef struct fastembedr_transform_server fastembedr_transform_server;

int fastembedr_transform_server_create(const double* reference_layout, int n_reference, double perplexity, int n_iter,
                                       int early_exaggeration_iter, double learning_rate, double early_exaggeration,
                                       double exaggeration, double initial_momentum, double final_momentum,
                                       double max_grad_norm, double max_step_norm, int n_negatives,
                                       int exact_repulsion_threshold, int seed, const char* initialization,
                                       unsigned long long memory_budget_bytes, int max_inflight,
                                       fastembedr_transform_server** server);
/* indices (int32) / distances (float32): host, column-major n_query x k KNN into the reference
 * (1- or 0-based). The arrays are copied before the call returns. */
int fastembedr_transform_server_submit(fastembedr_transform_server* server, const int* indices, const float* distances,
                                       int n_query, int k, unsigned long long* request_id);
/* Wait up to timeout_ms (< 0: no limit). Returns 0 when done (out: column-major n_query x 2
 * doubles, latency_ms: submit to result on the host; a non-NULL out consumes the request),
 * 2 while still queued or running, 1 on error. */
int fastembedr_transform_server_wait(fastembedr_transform_server* server, unsigned long long request_id, int timeout_ms,
                                     double* out, double* latency_ms);
/* Counters since creation. device_ms / iterate_ms: summed device time of the groups (CUDA events
 * on each group's stream: prepare + iterations / iterations only; overlapping groups each count
 * their own span). largest_group_*: the iterate time of the group with the most queries. */
int fastembedr_transform_server_stats(fastembedr_transform_server* server, unsigned long long* completed,
                                      unsigned long long* queries, unsigned long long* groups,
                                      unsigned long long* launches, unsigned long long* peak_bytes,
                                      unsigned long long* budget_bytes, double* device_ms, double* iterate_ms,
                                      long long* largest_group_queries, double* largest_group_iterate_ms);
/* Finishes the groups on the device, fails queued requests, frees everything. */
void fastembedr_transform_server_destroy(fastembedr_transform_server* server);

/* ---------------------------------------------------------------- resident t-SNE plan
 * No reference counterpart: the reference rebuilds everything per call. A plan keeps P, the
 * layout and the optimizer state resident in HBM so iterations can be timed and driven in
 * chunks (each chunk is one CUDA graph launch). */
typedef struct fastembedr_tsne_plan fastembedr_tsne_plan;

/* indices / distances: device pointers (column-major n x k); init: host row-major n x 2 or NULL. */
int fastembedr_tsne_plan_create(const int* indices, const float* distances, const float* init, int n, int k,
                                float perplexity, int index_offset, int grid_size, int interpolation,
                                unsigned int seed, fastembedr_tsne_plan** plan);
/* enqueue `iters` iterations on the plan's stream (CUDA graph when use_graph != 0) */
int fastembedr_tsne_plan_run(fastembedr_tsne_plan* plan, int iters, float exaggeration, float learning_rate,
                             float momentum, float min_gain, float max_step_norm, int use_graph);
/* run `iters` iterations eagerly, one stage after the other, and report device time (CUDA
 * events on the plan's stream): total, the attractive CSR kernel alone, and the grid stage
 * (scatter + FFT convolution) */
int fastembedr_tsne_plan_profile(fastembedr_tsne_plan* plan, int iters, float exaggeration, float learning_rate,
                                 float momentum, float min_gain, float max_step_norm, float* ms_total,
                                 float* ms_attractive_kernel, float* ms_grid_stage);
int fastembedr_tsne_plan_synchronize(fastembedr_tsne_plan* plan);
/* the plan's cudaStream_t, for callers that time with their own events */
void* fastembedr_tsne_plan_stream(fastembedr_tsne_plan* plan);
int fastembedr_tsne_plan_layout(fastembedr_tsne_plan* plan, float* out);
/* launches_per_iteration: kernel launches of one iteration; launches_per_reorder: of the spatial
 * reorder that starts every chunk of 25 iterations */
int fastembedr_tsne_plan_info(fastembedr_tsne_plan* plan, long long* nnz, int* grid_size, int* interpolation,
                              int* launches_per_iteration, int* launches_per_reorder);
/* The attractive pass's launch as tuned at run time (on the first normal-phase run of at least 25
 * iterations, unless FASTEMBEDR_TSNE_AUTOTUNE=0): slots per work item and resident blocks, and up
 * to `capacity` timed candidates (count receives how many were timed; 0 before tuning). The
 * launch does not change any result. No counterpart in the reference. */
int fastembedr_tsne_plan_tuning(fastembedr_tsne_plan* plan, int* chunk, int* blocks, int capacity, int* count,
                                int* cand_chunk, int* cand_blocks, float* cand_ms);
/* exact KL of the current layout (all-pairs Z on the GPU) */
int fastembedr_tsne_plan_kl(fastembedr_tsne_plan* plan, double* kl);
/* Gradient check of the plan's current layout at selected points (the force part of
 * opentsne_force_diagnostic_cpp, src/tsne_neighbors.cpp:1698-1817, evaluated in place on a resident
 * run so that an instance too large for the all-pairs diagnostic can still be checked). rows: n_rows
 * 0-based point ids (host). Writes row-major n_rows x 2 arrays: the attractive force
 * (exaggeration-scaled), the grid repulsion divided by the grid Z, and the exact repulsion of each
 * selected point against all n points (FP32 pair terms, FP64 sums) divided by the exact all-pairs
 * Z; z_grid / z_exact (may be NULL) receive both Z. The optimizer state is not changed. */
int fastembedr_tsne_plan_gradient_check(fastembedr_tsne_plan* plan, const int* rows, int n_rows,
                                        float exaggeration, float* attractive, float* repulsive_grid,
                                        double* repulsive_exact, double* z_grid, double* z_exact);
void fastembedr_tsne_plan_destroy(fastembedr_tsne_plan* plan);

/* ---------------------------------------------------------------- batched t-SNE
 * No reference counterpart (the reference runs one instance per call). Many independent
 * instances share every launch: their P matrices are appended into one CSR (rows and columns
 * offset by each instance's first point), instances with the same grid size share the FFT
 * launches, and every iteration of the whole batch is one CUDA graph node sequence
 * (3 + 3 x grid sizes launches). Each instance follows exactly the single-instance algorithm with
 * its own grid (the size policy of fastembedr_cuda_opentsne_fft_grid_size, or grid_size), its
 * own bounding box, Z and recentring, and the opt-SNE learning rate n_b / exaggeration. */
typedef struct fastembedr_tsne_batch fastembedr_tsne_batch;

/* sizes[b] points per instance. indices / distances: host, each instance's column-major
 * n_b x k KNN (its own rows 0..n_b-1, index_offset 0 or 1), instance after instance; init: host,
 * row-major n_b x 2 per instance, instance after instance, or NULL (seeded N(0, 1e-4^2)).
 * grid_size: 0 = the CUDA size policy per instance (256 / 512 / 1024 by n), -1 = the reference
 * CPU policy (tsne_fft_grid_size, src/tsne_neighbors.cpp:403-413: 128 below 50,000 points, else
 * 256), -2 = adaptive (at the start of every 25-iteration chunk each instance gets the smallest
 * power of two in [128, 1024] whose node spacing over its current bounding square is at most 0.7,
 * or FASTEMBEDR_TSNE_GRID_SPACING), > 0 = that many nodes per side for every instance. */
int fastembedr_tsne_batch_create(int n_instances, const int* sizes, const int* indices, const float* distances,
                                 const float* init, int k, float perplexity, int index_offset, int grid_size,
                                 int interpolation, unsigned int seed, fastembedr_tsne_batch** batch);
/* The same batch from one host pointer per instance, without a concatenated copy: indices[b] /
 * distances[b] are ROW-major n_b x k (C order), inits[b] row-major n_b x 2 (inits may be NULL);
 * index_offset < 0 detects each instance's 0- or 1-based labels on the device (min >= 1 and
 * max <= n_b: 1-based, as knn_index_offset). */
int fastembedr_tsne_batch_create_rows(int n_instances, const int* sizes, const int* const* indices,
                                      const float* const* distances, const float* const* inits, int k,
                                      float perplexity, int index_offset, int grid_size, int interpolation,
                                      unsigned int seed, fastembedr_tsne_batch** batch);
/* The two-phase schedule on every instance, returning when done. Instance b uses the learning
 * rate learning_rate x n_b in both phases; learning_rate <= 0 selects the package's opt-SNE
 * rate n_b / early_exaggeration (R/tsne_control.R:191-231). */
int fastembedr_tsne_batch_run(fastembedr_tsne_batch* batch, int early_exaggeration_iter, int n_iter,
                              float early_exaggeration, float exaggeration, float learning_rate,
                              float initial_momentum, float final_momentum, float min_gain, float max_step_norm);
/* Enqueue `iters` iterations on the batch's stream; instance b uses learning_rate x n_b. */
int fastembedr_tsne_batch_iterate(fastembedr_tsne_batch* batch, int iters, float exaggeration, float learning_rate,
                                  float momentum, float min_gain, float max_step_norm);
int fastembedr_tsne_batch_synchronize(fastembedr_tsne_batch* batch);
void* fastembedr_tsne_batch_stream(fastembedr_tsne_batch* batch);
/* Recentred layouts, row-major n_b x 2 per instance, instance after instance. */
int fastembedr_tsne_batch_layout(fastembedr_tsne_batch* batch, float* out);
/* Exact KL of one instance (all-pairs Z of that instance). */
int fastembedr_tsne_batch_kl(fastembedr_tsne_batch* batch, int instance, double* kl);
int fastembedr_tsne_batch_info(fastembedr_tsne_batch* batch, long long* nnz, long long* points, int* grid_classes,
                               int* launches_per_iteration, int* launches_per_reorder);
/* Current grid size of every instance (caller order) and how many times the adaptive policy
 * changed them; either output may be NULL. */
int fastembedr_tsne_batch_grids(fastembedr_tsne_batch* batch, int* grids, int* regrids);
void fastembedr_tsne_batch_destroy(fastembedr_tsne_batch* batch);
/* create + run + layout + destroy with the size-policy grids. */
int fastembedr_cuda_tsne_batch_from_knn(int n_instances, const int* sizes, const int* indices, const float* distances,
                                        const float* init, int k, float perplexity, int early_exaggeration_iter,
                                        int n_iter, float early_exaggeration, float exaggeration, float learning_rate,
                                        float initial_momentum, float final_momentum, float min_gain,
                                        float max_step_norm, unsigned int seed, int index_offset, float* out);

#ifdef __cplusplus
}
#endif
#endif
