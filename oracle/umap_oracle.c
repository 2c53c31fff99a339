/*
 * CPU oracle, UMAP part. TEST INFRASTRUCTURE ONLY (see oracle.h).
 *
 * Restates the reference CPU UMAP pieces in fastEmbedR src/fast_knn_umap.cpp
 * (smooth-KNN, fuzzy-union CSR, a/b fit, serial SGD, and the asynchronous
 * multi-threaded SGD branch, which only serves as a timing baseline) and the COO
 * epoch schedule of src/embedding_cuda_kernels.cpp, each cited per function.
 */
#include "oracle.h"

#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* smooth_knn_dist, src/fast_knn_umap.cpp:876-1003 (distances column-major) */
void orc_umap_smooth_knn(const float* dist, int n, int k, float* sigmas, float* rhos) {
  const double target = log2((double)k);
  const double tol = 1.0e-5, min_k_dist_scale = 1.0e-3;
  long double gsum = 0.0L;
  size_t gcount = 0u;
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < k; ++j) {
      const float d = dist[(int64_t)j * n + i];
      if (isfinite(d) && d >= 0.0f) {
        gsum += (long double)d;
        ++gcount;
      }
    }
  const double global_mean = gcount > 0u ? (double)(gsum / (long double)gcount) : 1.0;
#pragma omp parallel for schedule(static)
  for (int i = 0; i < n; ++i) {
    double rho = INFINITY, row_sum = 0.0;
    int row_count = 0;
    for (int j = 0; j < k; ++j) {
      const float d = dist[(int64_t)j * n + i];
      if (!isfinite(d)) continue;
      if (d >= 0.0f) {
        row_sum += (double)d;
        ++row_count;
      }
      if (d > 0.0f && (double)d < rho) rho = (double)d;
    }
    if (!isfinite(rho)) rho = 0.0;
    rhos[i] = (float)rho;
    const double sigma_max = DBL_MAX;
    double sigma = 1.0, sigma_best = sigma, best_diff = sigma_max, lo = 0.0, hi = sigma_max;
    for (int it = 0; it < 64; ++it) {
      double psum = 0.0;
      const double safe_sigma = sigma > 1.0e-12 ? sigma : 1.0e-12;
      for (int j = 0; j < k; ++j) {
        const float raw = dist[(int64_t)j * n + i];
        if (!isfinite(raw)) continue;
        const double d = (double)raw - rho;
        psum += d <= 0.0 ? 1.0 : exp(-d / safe_sigma);
      }
      const double diff = fabs(psum - target);
      if (diff < best_diff) {
        best_diff = diff;
        sigma_best = sigma;
      }
      if (psum > target) {
        hi = sigma;
        sigma = 0.5 * (lo + hi);
      } else {
        lo = sigma;
        if (hi == sigma_max) sigma *= 2.0;
        else sigma = 0.5 * (lo + hi);
      }
      if (diff < tol) break;
    }
    const double row_mean = row_count > 0 ? row_sum / (double)row_count : global_mean;
    const double floor_s = min_k_dist_scale * (rho > 0.0 ? row_mean : global_mean);
    if (sigma_best < floor_s) sigma_best = floor_s;
    sigmas[i] = (float)(sigma_best > 1.0e-12 ? sigma_best : 1.0e-12);
  }
}

/* build_graph_csr_native_direct_values, src/fast_knn_umap.cpp:1562-1780, with
 * compact_directed_rows_inplace (:1284-1365) and attach_csr_epoch_schedule (:1264-1282).
 * Returns nnz; with neighbors == NULL (or cap too small) only offsets are filled. */
int64_t orc_umap_graph(const int* idx, const float* dist, int n, int k, int offset,
                       int* offsets, int* neighbors, float* weights, float* eps,
                       int64_t cap, float* max_weight_out) {
  float* sig = (float*)malloc(sizeof(float) * (size_t)n);
  float* rho = (float*)malloc(sizeof(float) * (size_t)n);
  orc_umap_smooth_knn(dist, n, k, sig, rho);
  int* doff = (int*)calloc((size_t)n + 1, sizeof(int));
  int* dnb = (int*)malloc(sizeof(int) * (size_t)n * k);
  float* dw = (float*)malloc(sizeof(float) * (size_t)n * k);
  int64_t w = 0;
  for (int i = 0; i < n; ++i) {
    const int64_t begin = w;
    for (int j = 0; j < k; ++j) {
      const int nb = idx[(int64_t)j * n + i] - offset;
      const float d = dist[(int64_t)j * n + i];
      if (nb < 0 || nb >= n || nb == i || !isfinite(d)) continue;
      const float weight = d <= rho[i] ? 1.0f : expf(-(d - rho[i]) / sig[i]);
      if (!isfinite(weight) || weight <= 0.0f) continue;
      dnb[w] = nb;
      dw[w] = weight;
      ++w;
    }
    /* stable insertion sort by neighbour, then dedupe keeping the max weight */
    for (int64_t pos = begin + 1; pos < w; ++pos) {
      const int nb = dnb[pos];
      const float wt = dw[pos];
      int64_t c = pos;
      while (c > begin && dnb[c - 1] > nb) {
        dnb[c] = dnb[c - 1];
        dw[c] = dw[c - 1];
        --c;
      }
      dnb[c] = nb;
      dw[c] = wt;
    }
    int64_t out = begin;
    for (int64_t r = begin; r < w;) {
      const int nb = dnb[r];
      float wt = dw[r];
      ++r;
      while (r < w && dnb[r] == nb) {
        if (dw[r] > wt) wt = dw[r];
        ++r;
      }
      dnb[out] = nb;
      dw[out] = wt;
      ++out;
    }
    w = out;
    doff[i + 1] = (int)w;
  }
  /* transpose: incoming lists in increasing source order */
  int* ioff = (int*)calloc((size_t)n + 1, sizeof(int));
  for (int64_t t = 0; t < w; ++t) ioff[dnb[t] + 1]++;
  for (int i = 0; i < n; ++i) ioff[i + 1] += ioff[i];
  int* cur = (int*)malloc(sizeof(int) * (size_t)n);
  memcpy(cur, ioff, sizeof(int) * (size_t)n);
  int* inb = (int*)malloc(sizeof(int) * (size_t)(w > 0 ? w : 1));
  float* iw = (float*)malloc(sizeof(float) * (size_t)(w > 0 ? w : 1));
  for (int i = 0; i < n; ++i)
    for (int pos = doff[i]; pos < doff[i + 1]; ++pos) {
      const int o = cur[dnb[pos]]++;
      inb[o] = i;
      iw[o] = dw[pos];
    }
  /* merge-union rows: w = f + r - f*r, drop <= 1e-6 */
  offsets[0] = 0;
  int64_t nnz = 0;
  for (int pass = 0; pass < 2; ++pass) {
    nnz = 0;
    for (int i = 0; i < n; ++i) {
      int op = doff[i], oe = doff[i + 1], ip = ioff[i], ie = ioff[i + 1];
      while (op < oe || ip < ie) {
        const int onb = op < oe ? dnb[op] : 2147483647;
        const int inn = ip < ie ? inb[ip] : 2147483647;
        int nb;
        float f = 0.0f, r = 0.0f;
        if (onb == inn) {
          nb = onb; f = dw[op]; r = iw[ip]; ++op; ++ip;
        } else if (onb < inn) {
          nb = onb; f = dw[op]; ++op;
        } else {
          nb = inn; r = iw[ip]; ++ip;
        }
        if (nb == i) continue;
        const float wt = f + r - f * r;
        if (!isfinite(wt) || wt <= 1.0e-6f) continue;
        if (pass == 1) {
          neighbors[nnz] = nb;
          weights[nnz] = wt;
        }
        ++nnz;
      }
      if (pass == 0) offsets[i + 1] = (int)nnz;
    }
    if (pass == 0 && (neighbors == NULL || nnz > cap)) break;
  }
  if (neighbors != NULL && nnz <= cap) {
    float mw = 0.0f;
    for (int64_t t = 0; t < nnz; ++t)
      if (isfinite(weights[t]) && weights[t] > mw) mw = weights[t];
    for (int64_t t = 0; t < nnz; ++t) {
      const float wt = weights[t] > 1.0e-6f ? weights[t] : 1.0e-6f;
      eps[t] = mw > 0.0f ? mw / wt : INFINITY;
    }
    if (max_weight_out) *max_weight_out = mw;
  }
  free(sig); free(rho); free(doff); free(dnb); free(dw); free(ioff); free(cur); free(inb); free(iw);
  return nnz;
}

static void ab_fit(double spread, double min_dist, double* a_out, double* b_out) {
  double xs[300], ys[300];
  for (int i = 0; i < 300; ++i) {
    const double x = (spread * 3.0) * (double)i / 299.0;
    xs[i] = x;
    ys[i] = x < min_dist ? 1.0 : exp(-(x - min_dist) / spread);
  }
  double best_a = 1.5769434601962196, best_b = 0.8950608781227859, best_loss = INFINITY;
  for (double loga = -4.0; loga <= 4.0001; loga += 0.2) {
    for (double b = 0.25; b <= 2.0001; b += 0.05) {
      const double a = exp(loga);
      double loss = 0.0;
      for (int i = 0; i < 300; ++i) {
        const double x2b = pow(xs[i], 2.0 * b);
        const double e = 1.0 / (1.0 + a * x2b) - ys[i];
        loss += e * e;
      }
      if (loss < best_loss) {
        best_loss = loss;
        best_a = a;
        best_b = b;
      }
    }
  }
  for (int it = 0; it < 80; ++it) {
    double ga = 0.0, gb = 0.0;
    for (int i = 0; i < 300; ++i) {
      const double x = xs[i] > 1e-6 ? xs[i] : 1e-6;
      const double x2b = pow(x, 2.0 * best_b);
      const double den = 1.0 + best_a * x2b;
      const double e = 1.0 / den - ys[i];
      ga += e * (-x2b / (den * den));
      gb += e * (-(best_a * x2b * 2.0 * log(x)) / (den * den));
    }
    best_a = best_a - 0.01 * ga > 1e-4 ? best_a - 0.01 * ga : 1e-4;
    best_b = best_b - 0.01 * gb > 0.1 ? best_b - 0.01 * gb : 0.1;
  }
  *a_out = best_a;
  *b_out = best_b;
}

/* find_ab_params (CPU policy), src/fast_knn_umap.cpp:437-497 */
void orc_umap_ab(double spread, double min_dist, double* a, double* b) {
  if (fabs(spread - 1.0) < 1e-12 && fabs(min_dist - 0.01) < 1e-12) {
    *a = 1.895605865596314; *b = 0.8006377738365004; return;
  }
  if (fabs(spread - 1.0) < 1e-12 && fabs(min_dist - 0.1) < 1e-12) {
    *a = 1.5769434601962196; *b = 0.8950608781227859; return;
  }
  if (fabs(spread - 1.0) < 1e-12 && fabs(min_dist - 0.5) < 1e-12) {
    *a = 0.5830300199018228; *b = 1.3341669931033755; return;
  }
  ab_fit(spread, min_dist, a, b);
}

/* find_ab_params (CUDA host policy), src/embedding_cuda_impl.cpp:491-545 */
void orc_umap_ab_cuda_host(double spread, double min_dist, double* a, double* b) {
  if (fabs(spread - 1.0) < 1e-12 && fabs(min_dist - 0.1) < 1e-12) {
    *a = 1.5769434601962196; *b = 0.8950608781227859; return;
  }
  ab_fit(spread, min_dist, a, b);
}

/* umap_powf_fast / umap_pow, src/fast_knn_umap.cpp:156-215 (Schraudolph-style power) */
float orc_umap_powf_fast(float x, float b) {
  if (x <= 0.0f) return 0.0f;
  uint32_t xb;
  memcpy(&xb, &x, sizeof(float));
  const float bias = 1064866805.0f;
  const int whole = (int)b;
  const float frac = b - (float)whole;
  const uint32_t ib = (uint32_t)(frac * ((float)xb - bias) + bias);
  float fp;
  memcpy(&fp, &ib, sizeof(float));
  float ip = 1.0f, base = x;
  for (int e = whole; e > 0; e >>= 1) {
    if (e & 1) ip *= base;
    base *= base;
  }
  return ip * fp;
}

double orc_umap_pow(double x, double b) {
  if (x <= 0.0) return 0.0;
  uint64_t xb;
  memcpy(&xb, &x, sizeof(double));
  const double bias = 1072632447.0;
  const int whole = (int)b;
  const double frac = b - (double)whole;
  const double high = (double)(uint32_t)(xb >> 32);
  const uint64_t ih = (uint64_t)(frac * (high - bias) + bias);
  const uint64_t ibits = (ih & 0xffffffffull) << 32;
  double fp;
  memcpy(&fp, &ibits, sizeof(double));
  double ip = 1.0, base = x;
  for (int e = whole; e > 0; e >>= 1) {
    if (e & 1) ip *= base;
    base *= base;
  }
  return ip * fp;
}

static uint32_t mix_seed(uint32_t x) {
  x ^= x >> 16;
  x *= 0x7feb352du;
  x ^= x >> 15;
  x *= 0x846ca68bu;
  x ^= x >> 16;
  return x;
}

/* deterministic_vertex, src/fast_knn_umap.cpp:532-542 */
static int det_vertex(int n, int seed, int epoch, size_t edge, int sample) {
  uint32_t x = (uint32_t)seed;
  x ^= (uint32_t)((uint32_t)epoch * 0x9e3779b9u);
  x ^= (uint32_t)((edge + 1u) * 0x85ebca6bu);
  x ^= (uint32_t)((uint32_t)(sample + 1) * 0xc2b2ae35u);
  return (int)(mix_seed(x) % (uint32_t)n);
}

static double clip4d(double v) { return v < -4.0 ? -4.0 : (v > 4.0 ? 4.0 : v); }

/* serial branch of optimize_layout_csr, src/fast_knn_umap.cpp:3088-3165 (edge selection and
 * schedule) and :3458-3555 (SGD), n_components = 2; emb is column-major n x 2 doubles. */
void orc_umap_sgd_serial(int n, const int* offsets, const int* neighbors, const float* weights,
                         double* emb, int n_epochs, double a, double b, int nsr,
                         double learning_rate, double gamma, int seed) {
  double max_weight = 0.0;
  for (int row = 0; row < n; ++row)
    for (int pos = offsets[row]; pos < offsets[row + 1]; ++pos) {
      const int nb = neighbors[pos];
      if (nb >= 0 && nb < n && nb != row && (double)weights[pos] > max_weight) max_weight = weights[pos];
    }
  if (max_weight <= 0.0) return;
  const double min_sample_weight = n_epochs > 0 ? max_weight / (double)n_epochs : 0.0;
  const int64_t nnz = offsets[n];
  int* arow = (int*)malloc(sizeof(int) * (size_t)(nnz > 0 ? nnz : 1));
  int* atail = (int*)malloc(sizeof(int) * (size_t)(nnz > 0 ? nnz : 1));
  float* eps = (float*)malloc(sizeof(float) * (size_t)(nnz > 0 ? nnz : 1));
  float* next = (float*)malloc(sizeof(float) * (size_t)(nnz > 0 ? nnz : 1));
  float* epsn = (float*)malloc(sizeof(float) * (size_t)(nnz > 0 ? nnz : 1));
  float* nextn = (float*)malloc(sizeof(float) * (size_t)(nnz > 0 ? nnz : 1));
  size_t na = 0;
  for (int row = 0; row < n; ++row)
    for (int pos = offsets[row]; pos < offsets[row + 1]; ++pos) {
      const int nb = neighbors[pos];
      if (nb >= 0 && nb < n && nb != row && (double)weights[pos] >= min_sample_weight) {
        arow[na] = row;
        atail[na] = nb;
        const double wd = (double)weights[pos] > 1e-6 ? (double)weights[pos] : 1e-6;
        eps[na] = (float)(max_weight / wd);
        next[na] = eps[na];
        if (nsr > 0) {
          epsn[na] = eps[na] / (float)nsr;
          nextn[na] = epsn[na];
        } else {
          epsn[na] = INFINITY;
          nextn[na] = INFINITY;
        }
        ++na;
      }
    }
  double* ex = emb;
  double* ey = emb + n;
  for (int epoch = 0; epoch < n_epochs; ++epoch) {
    const double alpha = learning_rate * (1.0 - (double)epoch / n_epochs);
    for (size_t i = 0; i < na; ++i) {
      if (next[i] > (float)epoch) continue;
      const int j = arow[i], kk = atail[i];
      const double dx = ex[j] - ex[kk], dy = ey[j] - ey[kk];
      const double d2 = dx * dx + dy * dy;
      double gc = 0.0;
      if (d2 > 0.0) {
        const double dp = orc_umap_pow(d2, b);
        gc = -2.0 * a * b * (dp / d2) / (a * dp + 1.0);
      }
      const double gx = clip4d(gc * dx), gy = clip4d(gc * dy);
      ex[j] += gx * alpha;
      ey[j] += gy * alpha;
      ex[kk] -= gx * alpha;
      ey[kk] -= gy * alpha;
      next[i] += eps[i];
      int nneg = 0;
      if (nsr > 0 && (float)epoch >= nextn[i]) {
        nneg = (int)floorf(((float)epoch - nextn[i]) / epsn[i]);
        if (nneg < 0) nneg = 0;
      }
      for (int p = 0; p < nneg; ++p) {
        const int neg = det_vertex(n, seed, epoch, i, p);
        if (neg == j) continue;
        const double ndx = ex[j] - ex[neg], ndy = ey[j] - ey[neg];
        const double nd2 = ndx * ndx + ndy * ndy;
        double rep = 0.0;
        if (nd2 > 0.0) rep = 2.0 * gamma * b / ((0.001 + nd2) * (a * orc_umap_pow(nd2, b) + 1.0));
        ex[j] += clip4d(rep * ndx) * alpha;
        ey[j] += clip4d(rep * ndy) * alpha;
      }
      if (nneg > 0) nextn[i] += (float)nneg * epsn[i];
    }
  }
  free(arow); free(atail); free(eps); free(next); free(epsn); free(nextn);
}

static float clip4f(float x);

/* TauPrng and make_tau_prng, src/fast_knn_umap.cpp:659-701: a per-(worker, epoch) xorshift32
 * stream whose seed mixes the seed, the epoch, the worker and the end of its edge range. */
static uint32_t tau_seed(uint32_t s0, uint32_t s1, uint32_t s2) {
  const uint32_t st = mix_seed(s0 ^ (s1 << 7) ^ (s2 << 17));
  return st == 0u ? 0x9e3779b9u : st;
}

static uint32_t tau_make(int seed, int epoch, size_t window_end, int worker) {
  const uint32_t base = mix_seed((uint32_t)seed ^ (uint32_t)((uint32_t)(epoch + 1) * 0x9e3779b9u) ^
                                 (uint32_t)((uint32_t)(worker + 1) * 0x85ebca6bu) ^
                                 (uint32_t)((window_end + 1u) * 0xc2b2ae35u));
  return tau_seed(mix_seed(base ^ 0xa341316cu), mix_seed(base ^ 0xc8013ea4u), mix_seed(base ^ 0xad90777du));
}

static int tau_vertex(uint32_t* st, int n) {
  uint32_t x = *st;
  x ^= x << 13;
  x ^= x >> 17;
  x ^= x << 5;
  *st = x == 0u ? 0x9e3779b9u : x;
  return (int)(*st % (uint32_t)n);
}

/* The multi-threaded branch of optimize_layout_csr (n_components = 2, more than one worker,
 * n >= 10000), src/fast_knn_umap.cpp:3224-3350, which the package's default thread policy
 * (umap_default_threads, R/fast_knn_umap.R:966-981: up to 4 workers at n >= 500, k >= 15) selects
 * at these sizes. The edges are selected and scheduled as in the serial branch (:3116-3190);
 * each worker runs every epoch over its own range of them (ranges end at row boundaries), moves
 * float positions with atomic adds while the others do the same, draws negatives from its own
 * stream, and the workers meet every 50 epochs and at the last. Asynchronous by construction,
 * so results vary from run to run: a timing baseline for the reference's CPU path, not a parity
 * pin (the serial branch above is). */
void orc_umap_sgd_threaded(int n, const int* offsets, const int* neighbors, const float* weights,
                           double* emb, int n_epochs, double a, double b, int nsr, double learning_rate,
                           double gamma, int seed, int threads) {
  double max_weight = 0.0;
  for (int row = 0; row < n; ++row)
    for (int pos = offsets[row]; pos < offsets[row + 1]; ++pos) {
      const int nb = neighbors[pos];
      if (nb >= 0 && nb < n && nb != row && (double)weights[pos] > max_weight) max_weight = weights[pos];
    }
  if (max_weight <= 0.0 || n_epochs < 1) return;
  const double min_sample_weight = max_weight / (double)n_epochs;
  const int64_t nnz = offsets[n];
  const size_t cap = (size_t)(nnz > 0 ? nnz : 1);
  int* arow = (int*)malloc(sizeof(int) * cap);
  int* atail = (int*)malloc(sizeof(int) * cap);
  float* eps = (float*)malloc(sizeof(float) * cap);
  float* next = (float*)malloc(sizeof(float) * cap);
  float* epsn = (float*)malloc(sizeof(float) * cap);
  float* nextn = (float*)malloc(sizeof(float) * cap);
  float* x = (float*)malloc(sizeof(float) * (size_t)n);
  float* y = (float*)malloc(sizeof(float) * (size_t)n);
  size_t na = 0;
  for (int row = 0; row < n; ++row)
    for (int pos = offsets[row]; pos < offsets[row + 1]; ++pos) {
      const int nb = neighbors[pos];
      if (nb >= 0 && nb < n && nb != row && (double)weights[pos] >= min_sample_weight) {
        arow[na] = row;
        atail[na] = nb;
        const double wd = (double)weights[pos] > 1e-6 ? (double)weights[pos] : 1e-6;
        eps[na] = (float)(max_weight / wd);
        next[na] = eps[na];
        if (nsr > 0) {
          epsn[na] = eps[na] / (float)nsr;
          nextn[na] = epsn[na];
        } else {
          epsn[na] = INFINITY;
          nextn[na] = INFINITY;
        }
        ++na;
      }
    }
  for (int i = 0; i < n; ++i) {
    x[i] = (float)emb[i];
    y[i] = (float)emb[(int64_t)n + i];
  }
  const float af = (float)a, bf = (float)b;
  const float attraction = (float)(-2.0 * a * b), repulsion = (float)(2.0 * gamma * b);
  const float alpha0 = (float)learning_rate, alpha_step = alpha0 / (float)n_epochs;
  const float fe = FLT_EPSILON;
  if (threads < 1) threads = 1;
  size_t* begin = (size_t*)malloc(sizeof(size_t) * (size_t)(threads + 1));
#pragma omp parallel num_threads(threads)
  {
#ifdef _OPENMP
    const int t = omp_get_thread_num(), nt = omp_get_num_threads();
#else
    const int t = 0, nt = 1;
#endif
#pragma omp single
    {
      begin[0] = 0;
      begin[nt] = na;
      for (int w = 1; w < nt; ++w) {
        size_t bd = na * (size_t)w / (size_t)nt;
        while (bd < na && bd > 0 && arow[bd] == arow[bd - 1]) ++bd;
        begin[w] = bd;
      }
    }
    const size_t lo = begin[t], hi = begin[t + 1];
    float alpha = alpha0;
    for (int epoch = 0; epoch < n_epochs; ++epoch) {
      uint32_t st = tau_make(seed, epoch, hi, t);
      for (size_t i = lo; i < hi; ++i) {
        if (next[i] > (float)epoch) continue;
        const int j = arow[i], k = atail[i];
        float hx, hy, tx, ty;
#pragma omp atomic read
        hx = x[j];
#pragma omp atomic read
        hy = y[j];
#pragma omp atomic read
        tx = x[k];
#pragma omp atomic read
        ty = y[k];
        const float dx = hx - tx, dy = hy - ty;
        const float d2 = fmaxf(fe, dx * dx + dy * dy);
        const float dp = orc_umap_powf_fast(d2, bf);
        const float gc = attraction * dp / (d2 * (af * dp + 1.0f));
        const float gx = clip4f(gc * dx) * alpha, gy = clip4f(gc * dy) * alpha;
#pragma omp atomic
        x[j] += gx;
#pragma omp atomic
        y[j] += gy;
#pragma omp atomic
        x[k] += -gx;
#pragma omp atomic
        y[k] += -gy;
        next[i] += eps[i];
        int nneg = 0;
        if (nsr > 0 && (float)epoch >= nextn[i]) {
          nneg = (int)floorf(((float)epoch - nextn[i]) / epsn[i]);
          if (nneg < 0) nneg = 0;
        }
        for (int p = 0; p < nneg; ++p) {
          const int neg = tau_vertex(&st, n);
          if (neg == j) continue;
          float cx, cy, nx, ny;
#pragma omp atomic read
          cx = x[j];
#pragma omp atomic read
          cy = y[j];
#pragma omp atomic read
          nx = x[neg];
#pragma omp atomic read
          ny = y[neg];
          const float ndx = cx - nx, ndy = cy - ny;
          const float nd2 = fmaxf(fe, ndx * ndx + ndy * ndy);
          const float np = orc_umap_powf_fast(nd2, bf);
          const float rep = repulsion / ((0.001f + nd2) * (af * np + 1.0f));
          const float rx = clip4f(rep * ndx) * alpha, ry = clip4f(rep * ndy) * alpha;
#pragma omp atomic
          x[j] += rx;
#pragma omp atomic
          y[j] += ry;
        }
        if (nneg > 0) nextn[i] += (float)nneg * epsn[i];
      }
      if ((epoch + 1) % 50 == 0 || epoch == n_epochs - 1) {
#pragma omp barrier
      }
      alpha -= alpha_step;
    }
  }
  for (int i = 0; i < n; ++i) {
    emb[i] = (double)x[i];
    emb[(int64_t)n + i] = (double)y[i];
  }
  free(begin); free(arow); free(atail); free(eps); free(next); free(epsn); free(nextn); free(x); free(y);
}

/* ---- COO epoch schedule of the reference CUDA optimizer, src/embedding_cuda_kernels.cpp ---- */
static int pos_samples(float period, unsigned epoch) { /* :3044-3052 */
  if (period <= 0.0f || !isfinite(period) || epoch == 0u) return 0;
  const float now = (float)epoch, prev = (float)(epoch - 1u);
  const int s = (int)floorf(now / period) - (int)floorf(prev / period);
  return s > 0 ? s : 0;
}

static int neg_samples(float period, int nsr, unsigned epoch) { /* :3054-3084 */
  if (nsr <= 0 || period <= 0.0f || !isfinite(period) || epoch == 0u) return 0;
  const float now = (float)epoch, prev = (float)(epoch - 1u);
  const int cur = (int)floorf(now / period), pre = (int)floorf(prev / period);
  if (cur <= pre) return 0;
  const float np = period / (float)nsr;
  if (np <= 0.0f || !isfinite(np)) return 0;
  const int ct = (int)floorf((now - np) / np);
  int pt = 0;
  if (cur > 1) {
    const float pa = ceilf((float)(cur - 1) * period);
    pt = (int)floorf((pa - np) / np);
  }
  const int s = ct - pt;
  return s > 0 ? s : 0;
}

static uint32_t det_vertex_cuda(uint32_t n, uint32_t seed, uint32_t epoch, uint32_t i,
                                uint32_t edge, uint32_t sample) { /* :262-274 */
  uint32_t x = seed;
  x ^= epoch * 0x9e3779b9u;
  x ^= (i + 1u) * 0x85ebca6bu;
  x ^= (edge + 1u) * 0xc2b2ae35u;
  x ^= (sample + 1u) * 0x27d4eb2du;
  return mix_seed(x) % n;
}

static float clip4f(float x) { return x < -4.0f ? -4.0f : (x > 4.0f ? 4.0f : x); }

/* embed_epoch_coo_atomic_kernel + umap_sanitize_layout_kernel, :3086-3154 and :3244-3258,
 * executed edge by edge in order (the device version runs them concurrently). */
void orc_umap_sgd_coo_schedule(int n, int n_edges, const int* heads, const int* tails,
                               const float* eps, float* y, int n_epochs, float a, float b,
                               int nsr, float lr, float gamma, unsigned seed) {
  const float fe = 1.1920928955078125e-7f;
  for (int epoch = 0; epoch < n_epochs; ++epoch) {
    const float alpha = lr * (1.0f - (float)epoch / fmaxf(1.0f, (float)n_epochs));
    for (int e = 0; e < n_edges; ++e) {
      const int h = heads[e], t = tails[e];
      if (h < 0 || h >= n || t < 0 || t >= n || h == t) continue;
      const int ps = pos_samples(eps[e], (unsigned)epoch);
      if (ps <= 0) continue;
      for (int s = 0; s < ps; ++s) {
        const float dx = y[2 * h] - y[2 * t], dy = y[2 * h + 1] - y[2 * t + 1];
        const float d2 = fmaxf(fe, dx * dx + dy * dy);
        const float d2b = orc_umap_powf_fast(d2, b);
        const float c = -2.0f * a * b * (d2b / d2) / (a * d2b + 1.0f);
        const float gx = clip4f(c * dx) * alpha, gy = clip4f(c * dy) * alpha;
        y[2 * h] += gx; y[2 * h + 1] += gy;
        y[2 * t] -= gx; y[2 * t + 1] -= gy;
      }
      const int ns = neg_samples(eps[e], nsr, (unsigned)epoch);
      for (int s = 0; s < ns; ++s) {
        const int neg = (int)det_vertex_cuda((uint32_t)n, seed, (uint32_t)epoch, (uint32_t)h, (uint32_t)t, (uint32_t)s);
        if (neg == h || neg == t) continue;
        const float ndx = y[2 * h] - y[2 * neg], ndy = y[2 * h + 1] - y[2 * neg + 1];
        const float nd2 = fmaxf(fe, ndx * ndx + ndy * ndy);
        const float d2b = orc_umap_powf_fast(nd2, b);
        const float rc = gamma * 2.0f * b / ((0.001f + nd2) * (a * d2b + 1.0f));
        y[2 * h] += clip4f(rc * ndx) * alpha;
        y[2 * h + 1] += clip4f(rc * ndy) * alpha;
      }
    }
    for (int i = 0; i < n; ++i)
      for (int d = 0; d < 2; ++d) {
        float v = y[2 * i + d];
        if (!isfinite(v)) v = 0.0f;
        y[2 * i + d] = fminf(16.0f, fmaxf(-16.0f, v));
      }
  }
}

/* deterministic_unit, src/fast_knn_umap.cpp:522-530: a value in [-1, 1] from (seed, row, col) */
static float det_unit(int seed, int row, int col) {
  uint32_t x = (uint32_t)seed;
  x ^= (uint32_t)(row + 1) * 0x9e3779b9u;
  x ^= (uint32_t)(col + 1) * 0x85ebca6bu;
  return (float)(mix_seed(x) & 0x00ffffffu) / 8388607.5f - 1.0f;
}

/* normalize_cuda_like_init, src/fast_knn_umap.cpp:2541-2595 with one worker (sequential sums):
 * centre both columns, scale x to unit norm, remove x's projection from y and scale it to unit
 * norm (row-major n x 2 floats in place). */
static void whiten_pair(float* v, int n) {
  double sx = 0.0, sy = 0.0, sx2 = 0.0, sxy = 0.0, sy2 = 0.0;
  for (int i = 0; i < n; ++i) {
    const double x = v[2 * i], y = v[2 * i + 1];
    sx += x;
    sy += y;
    sx2 += x * x;
    sxy += x * y;
    sy2 += y * y;
  }
  const double dn = (double)n;
  const double mx = sx / dn, my = sy / dn;
  const double xss = fmax(sx2 - sx * sx / dn, 1.0e-24), yss = fmax(sy2 - sy * sy / dn, 1.0e-24);
  const double xy = sxy - sx * sy / dn;
  const double nx = sqrt(xss), inx = 1.0 / nx, proj = xy / nx;
  const double iny = 1.0 / sqrt(fmax(yss - proj * proj, 1.0e-24));
  for (int i = 0; i < n; ++i) {
    const double x = ((double)v[2 * i] - mx) * inx;
    const double y = (((double)v[2 * i + 1] - my) - proj * x) * iny;
    v[2 * i] = (float)x;
    v[2 * i + 1] = (float)y;
  }
}

/* initialize_layout_csr_cuda_diffusion, src/fast_knn_umap.cpp:2597-2652 (the CPU statement of
 * the reference's GPU spectral start): hashed start, whitened, then n_iter rounds of weighted
 * neighbour averaging over the CSR graph, whitened after each. out: row-major n x 2. */
void orc_umap_diffusion_init(const int* offsets, const int* neighbors, const float* weights, int n,
                             int index_offset, int n_iter, int seed, float* out) {
  float* cur = out;
  float* nxt = (float*)malloc(sizeof(float) * 2 * (size_t)n);
  for (int i = 0; i < n; ++i) {
    cur[2 * i] = det_unit(seed, i, 0);
    cur[2 * i + 1] = det_unit(seed, i, 1);
  }
  whiten_pair(cur, n);
  for (int it = 0; it < n_iter; ++it) {
    for (int i = 0; i < n; ++i) {
      float sx = 0.0f, sy = 0.0f, sw = 0.0f;
      for (int p = offsets[i]; p < offsets[i + 1]; ++p) {
        const int nb = neighbors[p] - index_offset;
        const float w = weights[p];
        if (nb < 0 || nb >= n || nb == i || w <= 0.0f || !isfinite(w)) continue;
        sx += w * cur[2 * nb];
        sy += w * cur[2 * nb + 1];
        sw += w;
      }
      if (sw <= 0.0f) {
        nxt[2 * i] = cur[2 * i];
        nxt[2 * i + 1] = cur[2 * i + 1];
      } else {
        nxt[2 * i] = sx / sw;
        nxt[2 * i + 1] = sy / sw;
      }
    }
    whiten_pair(nxt, n);
    memcpy(cur, nxt, sizeof(float) * 2 * (size_t)n);
  }
  free(nxt);
}
