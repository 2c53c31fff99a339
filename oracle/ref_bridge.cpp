// C entry points over the reference's own exported CPU functions (fastEmbedR
// src/tsne_neighbors.cpp, src/fast_knn_umap.cpp and src/embedding_utils.cpp, compiled
// unchanged against the test-only Rcpp shim). TEST INFRASTRUCTURE ONLY: used to generate golden vectors and
// to pin the plain-C oracle; never part of the product library.
#include <Rcpp.h>

#include <algorithm>
#include <cstring>
#include <limits>
#include <string>

using Rcpp::IntegerMatrix;
using Rcpp::IntegerVector;
using Rcpp::List;
using Rcpp::NumericMatrix;
using Rcpp::NumericVector;

// prototypes of the reference exports (src/tsne_neighbors.cpp:1656, :1698, :1871, :2124;
// src/fast_knn_umap.cpp:3996, :4461, :4525, :4547, :5291)
double opentsne_kl_diagnostic_cpp(IntegerMatrix, SEXP, SEXP, double, int);
List opentsne_force_diagnostic_cpp(IntegerMatrix, SEXP, SEXP, double, double, int, int);
List knn_tsne_opentsne_float_cpp(IntegerMatrix, SEXP, NumericMatrix, bool, int, double, double, int,
                                 int, double, double, double, bool, double, double, double, double,
                                 std::string, int, int, bool, bool, bool, double);
List transform_tsne_cpp(NumericMatrix, IntegerMatrix, NumericMatrix, NumericMatrix, bool, std::string,
                        double, int, int, double, double, double, double, double, double, double, int,
                        int, int, int, bool);
Rcpp::List umap_graph_csr_float_cpp(IntegerMatrix, SEXP, int, int, int, int);
NumericMatrix fast_knn_umap_csr_init_cpp(IntegerVector, IntegerVector, SEXP, NumericMatrix, int, double,
                                         int, double, double, int, int, bool);
NumericMatrix umap_cuda_diffusion_init_csr_cpp(IntegerVector, IntegerVector, SEXP, int, int, int);
NumericMatrix fast_knn_umap_csr_cpp(IntegerVector, IntegerVector, SEXP, int, int, double, int, double, double, int,
                                    int, double, int, bool);
NumericMatrix fast_knn_umap_range_cpp(IntegerMatrix, NumericMatrix, int, int, int, int, double, int, double, double,
                                      int, int, double, int, bool);
// src/embedding_utils.cpp:1386, :2120
NumericVector knn_structure_score_cpp(NumericMatrix, IntegerMatrix, IntegerVector, int, IntegerVector, int);
List project_embedding_affine_cpp(NumericMatrix, NumericMatrix, NumericMatrix, IntegerMatrix, NumericMatrix, int,
                                  double, double);

namespace {
thread_local std::string last_error;

IntegerMatrix int_matrix(const int* v, int n, int k) {
  IntegerMatrix m(n, k);
  std::copy(v, v + static_cast<std::size_t>(n) * k, m.begin());
  return m;
}
NumericMatrix num_matrix(const double* v, int n, int k) {
  NumericMatrix m(n, k);
  std::copy(v, v + static_cast<std::size_t>(n) * k, m.begin());
  return m;
}
template <typename T>
T get(const List& l, const char* name) {
  return std::any_cast<T>(l.get(name));
}
double get_num(const List& l, const char* name) {
  const std::any& a = l.get(name);
  if (a.type() == typeid(double)) return std::any_cast<double>(a);
  if (a.type() == typeid(float)) return std::any_cast<float>(a);
  if (a.type() == typeid(int)) return std::any_cast<int>(a);
  if (a.type() == typeid(bool)) return std::any_cast<bool>(a) ? 1.0 : 0.0;
  throw std::runtime_error(std::string("not a number: ") + name);
}
void copy_out(const NumericMatrix& m, double* out) { std::copy(m.begin(), m.end(), out); }
}  // namespace

extern "C" {

const char* ref_last_error() { return last_error.c_str(); }

// opentsne_force_diagnostic_cpp. All matrices column-major; col_out is 0-based.
int ref_force_diagnostic(const int* idx, const double* dist, const double* layout, int n, int k,
                         double perplexity, double exaggeration, int grid, int threads,
                         double* attractive, double* rep_exact, double* rep_fft, int* row_ptr,
                         int* col_out, double* weight_out, long long cap, long long* nnz,
                         double* sum_q, double* kl) {
  try {
    List d = opentsne_force_diagnostic_cpp(int_matrix(idx, n, k), num_matrix(dist, n, k),
                                           num_matrix(layout, n, 2), perplexity, exaggeration, grid, threads);
    copy_out(get<NumericMatrix>(d, "attractive_force"), attractive);
    copy_out(get<NumericMatrix>(d, "repulsive_force_exact"), rep_exact);
    copy_out(get<NumericMatrix>(d, "repulsive_force_fft"), rep_fft);
    IntegerVector rp = get<IntegerVector>(d, "affinity_row_ptr0");
    IntegerVector c1 = get<IntegerVector>(d, "affinity_col1");
    NumericVector w = get<NumericVector>(d, "affinity_weight");
    std::copy(rp.begin(), rp.end(), row_ptr);
    *nnz = c1.size();
    if (c1.size() > cap) throw std::runtime_error("capacity too small");
    for (R_xlen_t t = 0; t < c1.size(); ++t) {
      col_out[t] = c1[t] - 1;
      weight_out[t] = w[t];
    }
    *sum_q = get_num(d, "sum_q");
    *kl = get_num(d, "kl");
    return 0;
  } catch (const std::exception& e) {
    last_error = e.what();
    return 1;
  }
}

double ref_kl_diagnostic(const int* idx, const double* dist, const double* layout, int n, int k,
                         double perplexity, int threads) {
  try {
    return opentsne_kl_diagnostic_cpp(int_matrix(idx, n, k), num_matrix(dist, n, k), num_matrix(layout, n, 2),
                                      perplexity, threads);
  } catch (const std::exception& e) {
    last_error = e.what();
    return -1.0;
  }
}

// knn_tsne_opentsne_float_cpp with an explicit Y_init (column-major n x 2).
int ref_tsne_run(const int* idx, const double* dist, const double* y_init, int n, int k, double perplexity,
                 int early_iter, int n_iter, double early_exag, double exag, double learning_rate,
                 int lr_auto, double m0, double m1, double min_gain, double max_step_norm,
                 const char* method, int threads, int seed, int record_costs, double* y_out,
                 double* itercosts, int* n_costs, int* fft_grid) {
  try {
    List r = knn_tsne_opentsne_float_cpp(int_matrix(idx, n, k), num_matrix(dist, n, k), num_matrix(y_init, n, 2),
                                         true, 2, perplexity, 0.5, early_iter, n_iter, early_exag, exag,
                                         learning_rate, lr_auto != 0, m0, m1, min_gain, max_step_norm,
                                         std::string(method), threads, seed, false, record_costs != 0, false,
                                         5000.0);
    copy_out(get<NumericMatrix>(r, "Y"), y_out);
    NumericVector c = get<NumericVector>(r, "itercosts");
    if (n_costs) *n_costs = static_cast<int>(c.size());
    if (itercosts) std::copy(c.begin(), c.end(), itercosts);
    if (fft_grid) fft_grid[0] = static_cast<int>(get_num(r, "fft_grid_size"));
    return 0;
  } catch (const std::exception& e) {
    last_error = e.what();
    return 1;
  }
}

// transform_tsne_cpp; init: 0 = y_init, else "median"/"weighted" by name.
int ref_transform(const double* ref_layout, int n_ref, const int* idx, const double* dist, int n_query, int k,
                  const double* y_init, int use_init, const char* initialization, double perplexity,
                  int n_iter, int early_iter, double learning_rate, double early_exag, double exag, double m0,
                  double m1, double max_grad_norm, double max_step_norm, int n_negatives, int exact_threshold,
                  int threads, int seed, double* y_out) {
  try {
    NumericMatrix init = use_init ? num_matrix(y_init, n_query, 2) : NumericMatrix(0, 0);
    List r = transform_tsne_cpp(num_matrix(ref_layout, n_ref, 2), int_matrix(idx, n_query, k),
                                num_matrix(dist, n_query, k), init, use_init != 0, std::string(initialization),
                                perplexity, n_iter, early_iter, learning_rate, early_exag, exag, m0, m1,
                                max_grad_norm, max_step_norm, n_negatives, exact_threshold, threads, seed, false);
    copy_out(get<NumericMatrix>(r, "Y"), y_out);
    return 0;
  } catch (const std::exception& e) {
    last_error = e.what();
    return 1;
  }
}

// umap_graph_csr_float_cpp over all k columns (default fuzzy graph, edge_budget = k).
int ref_umap_graph(const int* idx, const double* dist, int n, int k, int threads, int* offsets,
                   int* neighbors, double* weights, double* eps, long long cap, long long* nnz,
                   double* max_weight) {
  try {
    List g = umap_graph_csr_float_cpp(int_matrix(idx, n, k), num_matrix(dist, n, k), 0, k, k, threads);
    IntegerVector o = get<IntegerVector>(g, "offsets");
    IntegerVector nb = get<IntegerVector>(g, "neighbors");
    NumericVector w = get<NumericVector>(g, "weights");
    NumericVector e = get<NumericVector>(g, "epochs_per_sample");
    std::copy(o.begin(), o.end(), offsets);
    *nnz = nb.size();
    if (nb.size() > cap) throw std::runtime_error("capacity too small");
    std::copy(nb.begin(), nb.end(), neighbors);
    std::copy(w.begin(), w.end(), weights);
    std::copy(e.begin(), e.end(), eps);
    *max_weight = get_num(g, "max_weight");
    return 0;
  } catch (const std::exception& e) {
    last_error = e.what();
    return 1;
  }
}

// fast_knn_umap_csr_init_cpp (CSR + init -> SGD layout), init/out column-major n x 2.
int ref_umap_sgd(const int* offsets, const int* neighbors, const double* weights, const double* init, int n,
                 long long nnz, int n_epochs, double min_dist, int nsr, double learning_rate, double gamma,
                 int threads, int seed, double* out) {
  try {
    IntegerVector o(offsets, offsets + n + 1);
    IntegerVector nb(neighbors, neighbors + nnz);
    NumericVector w(weights, weights + nnz);
    NumericMatrix r = fast_knn_umap_csr_init_cpp(o, nb, w, num_matrix(init, n, 2), n_epochs, min_dist, nsr,
                                                 learning_rate, gamma, threads, seed, false);
    copy_out(r, out);
    return 0;
  } catch (const std::exception& e) {
    last_error = e.what();
    return 1;
  }
}

// umap_cuda_diffusion_init_csr_cpp (the CPU statement of the GPU diffusion start) with one
// worker; out row-major n x 2.
int ref_umap_diffusion_init(const int* offsets, const int* neighbors, const double* weights, int n, long long nnz,
                            int n_iter, int seed, double* out) {
  try {
    IntegerVector o(offsets, offsets + n + 1);
    IntegerVector nb(neighbors, neighbors + nnz);
    NumericVector w(weights, weights + nnz);
    NumericMatrix r = umap_cuda_diffusion_init_csr_cpp(o, nb, w, n_iter, 1, seed);
    for (int i = 0; i < n; ++i) {
      out[2 * i] = r(i, 0);
      out[2 * i + 1] = r(i, 1);
    }
    return 0;
  } catch (const std::exception& e) {
    last_error = e.what();
    return 1;
  }
}

// fast_knn_umap_csr_cpp with n_epochs = 0 (the CPU spectral start, as umap_init_from_csr_graph
// calls it) with one worker; out row-major n x 2.
int ref_umap_spectral_init(const int* offsets, const int* neighbors, const double* weights, int n, long long nnz,
                           int n_iter, double init_scale, int seed, double* out) {
  try {
    IntegerVector o(offsets, offsets + n + 1);
    IntegerVector nb(neighbors, neighbors + nnz);
    NumericVector w(weights, weights + nnz);
    NumericMatrix r = fast_knn_umap_csr_cpp(o, nb, w, 2, 0, 0.01, 0, 1.0, 1.0, n_iter, 1, init_scale, seed, false);
    for (int i = 0; i < n; ++i) {
      out[2 * i] = r(i, 0);
      out[2 * i + 1] = r(i, 1);
    }
    return 0;
  } catch (const std::exception& e) {
    last_error = e.what();
    return 1;
  }
}

// spectral_knn_init(backend = "cpu") (R/fast_knn_umap.R:1343-1365): fast_knn_umap_range_cpp over
// all k columns with n_epochs = 0, one worker; idx / dist column-major n x k, out row-major n x 2.
int ref_umap_spectral_knn(const int* idx, const double* dist, int n, int k, int n_iter, int seed, double* out) {
  try {
    NumericMatrix r = fast_knn_umap_range_cpp(int_matrix(idx, n, k), num_matrix(dist, n, k), 0, k, 2, 0, 0.01, 0,
                                              1.0, 1.0, n_iter, 1, std::numeric_limits<double>::quiet_NaN(), seed,
                                              false);
    for (int i = 0; i < n; ++i) {
      out[2 * i] = r(i, 0);
      out[2 * i + 1] = r(i, 1);
    }
    return 0;
  } catch (const std::exception& e) {
    last_error = e.what();
    return 1;
  }
}

// knn_structure_score_cpp: layout n x 2, high-dimensional KNN n x k (1-based), keep (1-based rows),
// no labels. out: preservation, trustworthiness, continuity, structure score (4 values).
int ref_knn_structure_score(const double* layout, int n, const int* idx, int k, const int* keep, int n_keep,
                            int preserve_k, double* out) {
  try {
    IntegerVector kv(n_keep);
    std::copy(keep, keep + n_keep, kv.begin());
    NumericVector r = knn_structure_score_cpp(num_matrix(layout, n, 2), int_matrix(idx, n, k), kv, preserve_k,
                                              IntegerVector(0), 0);
    for (int i = 0; i < 4; ++i) out[i] = r[i];
    return 0;
  } catch (const std::exception& e) {
    last_error = e.what();
    return 1;
  }
}

// project_embedding_affine_cpp: reference data n_ref x f, query data n_query x f, reference
// layout n_ref x 2, projection KNN n_query x k (1-based) with distances. out_layout n_query x 2;
// fallback per query (1 where the weighted mean was used).
int ref_project_affine(const double* ref_data, int n_ref, const double* query_data, int n_query, int n_features,
                       const double* ref_layout, const int* idx, const double* dist, int k, int max_neighbors,
                       double ridge, double max_extrapolation, double* out_layout, double* confidence,
                       int* fallback) {
  try {
    List r = project_embedding_affine_cpp(num_matrix(ref_data, n_ref, n_features),
                                          num_matrix(query_data, n_query, n_features), num_matrix(ref_layout, n_ref, 2),
                                          int_matrix(idx, n_query, k), num_matrix(dist, n_query, k), max_neighbors,
                                          ridge, max_extrapolation);
    copy_out(get<NumericMatrix>(r, "layout"), out_layout);
    const NumericVector c = get<NumericVector>(r, "confidence");
    std::copy(c.begin(), c.end(), confidence);
    const IntegerVector f = get<IntegerVector>(r, "fallback");
    std::copy(f.begin(), f.end(), fallback);
    return 0;
  } catch (const std::exception& e) {
    last_error = e.what();
    return 1;
  }
}

}  // extern "C"
