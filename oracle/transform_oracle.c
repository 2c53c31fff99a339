/*
 * CPU oracle, fixed-reference transform and quality metric. TEST INFRASTRUCTURE ONLY.
 *
 * Restates transform_tsne_cpp (fastEmbedR src/tsne_neighbors.cpp:2124-2373) for
 * two-dimensional layouts and the knn_preservation part of knn_structure_score_cpp
 * (src/embedding_utils.cpp:1386-1579).
 */
#include "oracle.h"

#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

/* mix_uint32 / xorshift32 / uniform_index, src/tsne_neighbors.cpp:67-88 */
static uint32_t mix_u32(uint32_t v) {
  v ^= v >> 16u;
  v *= 0x7feb352du;
  v ^= v >> 15u;
  v *= 0x846ca68bu;
  v ^= v >> 16u;
  return v == 0u ? 0x6d2b79f5u : v;
}
static uint32_t xorshift32(uint32_t* s) {
  *s ^= *s << 13u;
  *s ^= *s >> 17u;
  *s ^= *s << 5u;
  return *s;
}
static int uniform_index(uint32_t* s, int n) {
  return (int)(((uint64_t)xorshift32(s) * (uint64_t)n) >> 32u);
}

/* compute_row_probabilities_flat, src/tsne_neighbors.cpp:452-530 */
static void row_p_flat(const double* dist, int n_query, int k, int row, double perplexity, double* p) {
  for (int j = 0; j < k; ++j) p[j] = 0.0;
  double min_d2 = DBL_MAX, max_d2 = 0.0;
  for (int j = 0; j < k; ++j) {
    const double d = dist[(int64_t)j * n_query + row];
    const double d2 = d * d;
    if (d2 < min_d2) min_d2 = d2;
    if (d2 > max_d2) max_d2 = d2;
  }
  if (max_d2 - min_d2 <= DBL_EPSILON * (max_d2 > 1.0 ? max_d2 : 1.0)) {
    for (int j = 0; j < k; ++j) p[j] = 1.0 / (double)k;
    return;
  }
  int found = 0;
  double beta = 1.0, min_beta = -DBL_MAX, max_beta = DBL_MAX, sum_p = DBL_MIN;
  for (int it = 0; !found && it < 200; ++it) {
    sum_p = DBL_MIN;
    for (int j = 0; j < k; ++j) {
      const double d = dist[(int64_t)j * n_query + row];
      p[j] = exp(-beta * (d * d - min_d2));
      sum_p += p[j];
    }
    double entropy = 0.0;
    for (int j = 0; j < k; ++j) {
      const double d = dist[(int64_t)j * n_query + row];
      entropy += beta * ((d * d - min_d2) * p[j]);
    }
    entropy = entropy / sum_p + log(sum_p);
    const double diff = entropy - log(perplexity);
    if (fabs(diff) < 1e-5) {
      found = 1;
    } else if (diff > 0.0) {
      min_beta = beta;
      beta = (max_beta == DBL_MAX || max_beta == -DBL_MAX) ? beta * 2.0 : (beta + max_beta) / 2.0;
    } else {
      max_beta = beta;
      beta = (min_beta == -DBL_MAX || min_beta == DBL_MAX) ? beta / 2.0 : (beta + min_beta) / 2.0;
    }
    if (!isfinite(beta)) break;
  }
  if (!isfinite(sum_p) || sum_p <= DBL_MIN) {
    int tied = 0;
    for (int j = 0; j < k; ++j) {
      const double d = dist[(int64_t)j * n_query + row];
      if (fabs(d * d - min_d2) <= DBL_EPSILON * (min_d2 > 1.0 ? min_d2 : 1.0)) ++tied;
    }
    for (int j = 0; j < k; ++j) {
      const double d = dist[(int64_t)j * n_query + row];
      p[j] = fabs(d * d - min_d2) <= DBL_EPSILON * (min_d2 > 1.0 ? min_d2 : 1.0) ? 1.0 / (tied > 1 ? tied : 1) : 0.0;
    }
    return;
  }
  const double inv = 1.0 / sum_p;
  for (int j = 0; j < k; ++j) p[j] *= inv;
}

static int cmp_double(const void* a, const void* b) {
  const double x = *(const double*)a, y = *(const double*)b;
  return x < y ? -1 : (x > y ? 1 : 0);
}

static double sign_d(double x) { return x == 0.0 ? 0.0 : (x < 0.0 ? -1.0 : 1.0); }

/* transform_tsne_cpp, src/tsne_neighbors.cpp:2124-2373 (dims = 2, one batch; the
 * reference's batching does not change results). init_mode: 0 = y_init, 1 = median,
 * 2 = weighted. ref_y row-major interleaved; idx/dist column-major n_query x k. */
int orc_transform_tsne(const double* ref_y, int n_ref, const int* idx, const double* dist,
                       int n_query, int k, const double* y_init, int init_mode,
                       double perplexity, int n_iter, int early_iter, double learning_rate,
                       double early_exag, double exag, double m0, double m1,
                       double max_grad_norm, double max_step_norm, int n_negatives,
                       int exact_threshold, int seed, double* y) {
  if (exact_threshold < 1) exact_threshold = 1;
  if (max_grad_norm <= 0.0 || !isfinite(max_grad_norm)) max_grad_norm = DBL_MAX;
  if (max_step_norm <= 0.0 || !isfinite(max_step_norm)) max_step_norm = DBL_MAX;
  int lo = 2147483647, hi = -2147483647 - 1;
  for (int64_t t = 0; t < (int64_t)n_query * k; ++t) {
    if (idx[t] < lo) lo = idx[t];
    if (idx[t] > hi) hi = idx[t];
  }
  const int offset = (lo >= 1 && hi <= n_ref) ? 1 : 0;
  for (int64_t t = 0; t < (int64_t)n_query * k; ++t) {
    const int r = idx[t] - offset;
    if (r < 0 || r >= n_ref) return 1;
    if (!isfinite(dist[t]) || dist[t] < 0.0) return 2;
  }
  if (n_negatives > n_ref) n_negatives = n_ref;
  const int exact = n_ref <= exact_threshold || n_negatives >= n_ref;
  double* P = (double*)malloc(sizeof(double) * (size_t)n_query * k);
  for (int i = 0; i < n_query; ++i) row_p_flat(dist, n_query, k, i, perplexity, P + (int64_t)i * k);
  double* vals = (double*)malloc(sizeof(double) * (size_t)k);
  for (int i = 0; i < n_query; ++i) {
    for (int d = 0; d < 2; ++d) {
      if (init_mode == 0) {
        y[2 * (int64_t)i + d] = y_init[2 * (int64_t)i + d];
      } else if (init_mode == 2) {
        double num = 0.0, den = DBL_MIN;
        for (int j = 0; j < k; ++j) {
          const int r = idx[(int64_t)j * n_query + i] - offset;
          const double dd = dist[(int64_t)j * n_query + i] > 0.0 ? dist[(int64_t)j * n_query + i] : 0.0;
          const double w = 1.0 / (dd + 1e-6);
          num += w * ref_y[2 * (int64_t)r + d];
          den += w;
        }
        y[2 * (int64_t)i + d] = num / den;
      } else {
        for (int j = 0; j < k; ++j) vals[j] = ref_y[2 * (int64_t)(idx[(int64_t)j * n_query + i] - offset) + d];
        qsort(vals, (size_t)k, sizeof(double), cmp_double);
        const int mid = k / 2;
        y[2 * (int64_t)i + d] = (k & 1) ? vals[mid] : 0.5 * (vals[mid] + vals[mid - 1]);
      }
    }
  }
  free(vals);
  double* upd = (double*)calloc(2 * (size_t)n_query, sizeof(double));
  double* gains = (double*)malloc(sizeof(double) * 2 * (size_t)n_query);
  for (int64_t t = 0; t < 2 * (int64_t)n_query; ++t) gains[t] = 1.0;
  const int total = early_iter + n_iter;
  const int qsz = exact ? n_ref : (n_negatives > 1 ? n_negatives : 1);
  for (int it = 0; it < total; ++it) {
    const int in_early = it < early_iter;
    const double ex = in_early ? early_exag : exag;
    const double mom = in_early ? m0 : m1;
    const int iter_seed = seed + 65537 * (it + 1);
#pragma omp parallel
    {
      double* qv = (double*)malloc(sizeof(double) * (size_t)qsz);
      int* smp = (int*)malloc(sizeof(int) * (size_t)qsz);
#pragma omp for schedule(static)
      for (int i = 0; i < n_query; ++i) {
        const double yi0 = y[2 * (int64_t)i], yi1 = y[2 * (int64_t)i + 1];
        double g0 = 0.0, g1 = 0.0, sum_q = DBL_MIN;
        uint32_t rs = mix_u32((uint32_t)iter_seed ^ ((uint32_t)(i + 1) * 0x9e3779b9u));
        if (exact) {
          for (int r = 0; r < n_ref; ++r) {
            const double dx = yi0 - ref_y[2 * (int64_t)r], dy = yi1 - ref_y[2 * (int64_t)r + 1];
            qv[r] = 1.0 / (1.0 + dx * dx + dy * dy);
            sum_q += qv[r];
          }
          const double inv = 1.0 / sum_q;
          for (int r = 0; r < n_ref; ++r) {
            const double c = -(qv[r] * qv[r]) * inv;
            g0 += c * (yi0 - ref_y[2 * (int64_t)r]);
            g1 += c * (yi1 - ref_y[2 * (int64_t)r + 1]);
          }
        } else {
          for (int m = 0; m < n_negatives; ++m) {
            const int r = uniform_index(&rs, n_ref);
            smp[m] = r;
            const double dx = yi0 - ref_y[2 * (int64_t)r], dy = yi1 - ref_y[2 * (int64_t)r + 1];
            qv[m] = 1.0 / (1.0 + dx * dx + dy * dy);
            sum_q += qv[m];
          }
          const double inv = 1.0 / sum_q;
          for (int m = 0; m < n_negatives; ++m) {
            const int r = smp[m];
            const double c = -(qv[m] * qv[m]) * inv;
            g0 += c * (yi0 - ref_y[2 * (int64_t)r]);
            g1 += c * (yi1 - ref_y[2 * (int64_t)r + 1]);
          }
        }
        for (int j = 0; j < k; ++j) {
          const int r = idx[(int64_t)j * n_query + i] - offset;
          const double dx = yi0 - ref_y[2 * (int64_t)r], dy = yi1 - ref_y[2 * (int64_t)r + 1];
          const double q = 1.0 / (1.0 + dx * dx + dy * dy);
          const double c = ex * P[(int64_t)i * k + j] * q;
          g0 += c * dx;
          g1 += c * dy;
        }
        double g[2] = {g0, g1};
        const double gn2 = g[0] * g[0] + g[1] * g[1];
        if (gn2 > max_grad_norm * max_grad_norm) {
          const double sc = max_grad_norm / (sqrt(gn2) + 1e-12);
          g[0] *= sc;
          g[1] *= sc;
        }
        for (int d = 0; d < 2; ++d) {
          const int64_t t = 2 * (int64_t)i + d;
          if (sign_d(upd[t]) != sign_d(g[d])) gains[t] += 0.2;
          else gains[t] = gains[t] * 0.8 + 0.01;
          if (gains[t] < 0.01) gains[t] = 0.01;
          upd[t] = mom * upd[t] - learning_rate * gains[t] * g[d];
        }
        const double s2 = upd[2 * (int64_t)i] * upd[2 * (int64_t)i] + upd[2 * (int64_t)i + 1] * upd[2 * (int64_t)i + 1];
        if (s2 > max_step_norm * max_step_norm) {
          const double sc = max_step_norm / (sqrt(s2) + 1e-12);
          upd[2 * (int64_t)i] *= sc;
          upd[2 * (int64_t)i + 1] *= sc;
        }
        y[2 * (int64_t)i] += upd[2 * (int64_t)i];
        y[2 * (int64_t)i + 1] += upd[2 * (int64_t)i + 1];
      }
      free(qv);
      free(smp);
    }
  }
  free(P);
  free(upd);
  free(gains);
  return 0;
}

typedef struct { double d; int j; } dj_pair;

static int pair_less(dj_pair a, dj_pair b) { return a.d < b.d || (a.d == b.d && a.j < b.j); }

/* knn_preservation of knn_structure_score_cpp, src/embedding_utils.cpp:1386-1579:
 * mean over kept rows of |low-dim exact preserve_k-NN  n  first preserve_k high-dim columns| / k.
 * keep holds 0-based row ids; idx_hi column-major n x k_hi with index offset. */
double orc_knn_preservation(const float* y, int n, const int* idx_hi, int k_hi, int offset,
                            const int* keep, int n_keep, int preserve_k) {
  double total = 0.0;
  int scored = 0;
#pragma omp parallel for schedule(dynamic, 4) reduction(+ : total, scored)
  for (int kk = 0; kk < n_keep; ++kk) {
    const int q = keep[kk];
    dj_pair* best = (dj_pair*)malloc(sizeof(dj_pair) * (size_t)(preserve_k + 1));
    int cnt = 0;
    const double qx = y[2 * (int64_t)q], qy = y[2 * (int64_t)q + 1];
    for (int c = 0; c < n; ++c) {
      if (c == q) continue;
      const double dx = qx - y[2 * (int64_t)c], dy = qy - y[2 * (int64_t)c + 1];
      dj_pair cand = {dx * dx + dy * dy, c};
      if (cnt < preserve_k) {
        int p = cnt++;
        while (p > 0 && pair_less(cand, best[p - 1])) {
          best[p] = best[p - 1];
          --p;
        }
        best[p] = cand;
      } else if (pair_less(cand, best[preserve_k - 1])) {
        int p = preserve_k - 1;
        while (p > 0 && pair_less(cand, best[p - 1])) {
          best[p] = best[p - 1];
          --p;
        }
        best[p] = cand;
      }
    }
    if (cnt >= preserve_k) {
      int shared = 0;
      for (int r = 0; r < preserve_k; ++r) {
        int rank = k_hi + 1;
        for (int h = 0; h < k_hi; ++h)
          if (idx_hi[(int64_t)h * n + q] - offset == best[r].j) {
            rank = h + 1;
            break;
          }
        if (rank <= preserve_k) ++shared;
      }
      total += (double)shared / (double)preserve_k;
      ++scored;
    }
    free(best);
  }
  return scored > 0 ? total / scored : 0.0;
}
