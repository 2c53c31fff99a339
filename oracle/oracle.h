/*
 * CPU oracle for the fastEmbedR KNN-input embedding optimizer.
 *
 * TEST INFRASTRUCTURE ONLY. This library is a plain-C restatement of the
 * reference CPU algorithms (fastEmbedR src/tsne_neighbors.cpp,
 * src/fast_knn_umap.cpp, src/embedding_utils.cpp and the FP64 test helper
 * tests/testthat/helper-tsne-reference.R). Only the test suite, the smoke
 * check and the CPU-baseline leg of the benchmark load it, as the checker.
 * The product library never links, loads or calls it.
 *
 * Layout conventions (same as the product C ABI):
 *   - KNN indices / distances: column-major n x k (element (i, j) at j*n + i),
 *     indices carry `offset` (0 or 1).
 *   - Layouts (Y, init, gradients): row-major interleaved n x 2 floats.
 *   - CSR: row_ptr (n + 1), col (nnz), val (nnz); columns ascending per row.
 */
#ifndef FASTEMBEDR_ORACLE_H
#define FASTEMBEDR_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------- shared helpers ---------------- */
int orc_index_offset(const int* idx, int n, int k);
int orc_validate_knn(const int* idx, const float* dist, int n, int k, int offset);
int orc_set_threads(int n_threads);

/* ---------------- t-SNE affinities (T3/T4) ---------------- */
void orc_row_p_f32(const float* dist, int n, int k, double perplexity, float* p_rowmajor);
void orc_row_p_f64(const float* dist, int n, int k, double perplexity,
                   double* p_rowmajor, double* beta_out);
int64_t orc_csr_build(const int* idx, const float* p_rowmajor, int n, int k, int offset,
                      int* row_ptr, int* col, float* val, int64_t cap, double* total_mass);

/* ---------------- t-SNE forces (T5-T11, T14, T15) ---------------- */
int orc_fft_grid_size_cpu(int n);
void orc_attractive(const int* row_ptr, const int* col, const float* val, const float* y,
                    int n, float exaggeration, float* attr_out);
void orc_exact_rep_f32(const float* y, int n, float* rep_out, double* sum_q_out);
void orc_exact_rep_f64(const float* y, int n, double* rep_out, double* sum_q_out);
void orc_fft_grid_rep_f32(const float* y, int n, int grid_size, float* rep_out, double* z_out);
void orc_interp_rep_f64(const float* y, int n, int grid_size, int lagrange,
                        double* rep_out, double* z_out);
void orc_update(float* y, float* update, float* gains, const float* grad, int n,
                float learning_rate, float momentum, float min_gain, float max_step_norm);
void orc_zero_mean(float* y, int n);
double orc_sum_q(const float* y, int n);
double orc_kl(const int* row_ptr, const int* col, const float* val, const float* y, int n);

/* full optimizer (E2 of the reference); repulsion: 0 = fft_grid, 1 = exact pairs */
int orc_tsne_run(const int* idx, const float* dist, int n, int k, const float* init,
                 double perplexity, int early_iter, int n_iter, double early_exag,
                 double exag, double learning_rate, int lr_auto, double m0, double m1,
                 double min_gain, double max_step_norm, int repulsion, int grid_size,
                 float* y_out, double* kl_trace, int* kl_iters, int kl_cap);

/* step-wise driver used by the CPU baseline: build once, time iterations */
typedef struct orc_tsne_state orc_tsne_state;
orc_tsne_state* orc_tsne_prepare(const int* idx, const float* dist, int n, int k,
                                 const float* init, double perplexity, int grid_size);
void orc_tsne_iterate(orc_tsne_state* s, int iters, float exaggeration, float learning_rate,
                      float momentum, float min_gain, float max_step_norm);
void orc_tsne_get_y(const orc_tsne_state* s, float* y_out);
int64_t orc_tsne_nnz(const orc_tsne_state* s);
void orc_tsne_free(orc_tsne_state* s);

/* ---------------- UMAP (U1-U5) ---------------- */
void orc_umap_smooth_knn(const float* dist, int n, int k, float* sigmas, float* rhos);
int64_t orc_umap_graph(const int* idx, const float* dist, int n, int k, int offset,
                       int* offsets, int* neighbors, float* weights, float* epochs_per_sample,
                       int64_t cap, float* max_weight);
void orc_umap_ab(double spread, double min_dist, double* a, double* b);
void orc_umap_ab_cuda_host(double spread, double min_dist, double* a, double* b);
float orc_umap_powf_fast(float x, float b);
double orc_umap_pow(double x, double b);
void orc_umap_sgd_serial(int n, const int* offsets, const int* neighbors, const float* weights,
                         double* emb_colmajor, int n_epochs, double a, double b,
                         int negative_sample_rate, double learning_rate,
                         double repulsion_strength, int seed);
void orc_umap_sgd_threaded(int n, const int* offsets, const int* neighbors, const float* weights,
                           double* emb_colmajor, int n_epochs, double a, double b,
                           int negative_sample_rate, double learning_rate,
                           double repulsion_strength, int seed, int threads);
void orc_umap_diffusion_init(const int* offsets, const int* neighbors, const float* weights, int n,
                             int index_offset, int n_iter, int seed, float* out);
void orc_umap_spectral_init(const int* offsets, const int* neighbors, const float* weights, int n,
                            int n_iter, double init_scale, int seed, double* out);
void orc_umap_sgd_coo_schedule(int n, int n_edges, const int* heads, const int* tails,
                               const float* epochs_per_sample, float* y, int n_epochs,
                               float a, float b, int negative_sample_rate, float learning_rate,
                               float repulsion_strength, unsigned seed);

/* ---------------- fixed-reference transform (X1) ---------------- */
int orc_transform_tsne(const double* ref_y, int n_ref, const int* idx, const double* dist,
                       int n_query, int k, const double* y_init, int init_mode,
                       double perplexity, int n_iter, int early_iter, double learning_rate,
                       double early_exag, double exag, double m0, double m1,
                       double max_grad_norm, double max_step_norm, int n_negatives,
                       int exact_threshold, int seed, double* y_out);

/* ---------------- quality metric (M1) ---------------- */
double orc_knn_preservation(const float* y, int n, const int* idx_hi, int k_hi, int offset,
                            const int* keep, int n_keep, int preserve_k);

#ifdef __cplusplus
}
#endif
#endif
