/*
 * CPU oracle, t-SNE part. TEST INFRASTRUCTURE ONLY (see oracle.h).
 *
 * Restates the reference CPU optimizer in fastEmbedR src/tsne_neighbors.cpp
 * (cited per function) and the FP64 dense test oracle in
 * tests/testthat/helper-tsne-reference.R. Float code paths keep the reference's
 * operation order so that, compiled with -ffp-contract=off, they reproduce the
 * reference arithmetic; the FP64 paths are the accuracy yardsticks.
 */
#include "oracle.h"

#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

int orc_set_threads(int n_threads) {
#ifdef _OPENMP
  if (n_threads > 0) omp_set_num_threads(n_threads);
  return omp_get_max_threads();
#else
  (void)n_threads;
  return 1;
#endif
}

static float fminf_(float a, float b) { return b < a ? b : a; }
static float fmaxf_(float a, float b) { return a < b ? b : a; }

/* resolve_index_offset, src/tsne_neighbors.cpp:90-101 */
int orc_index_offset(const int* idx, int n, int k) {
  int lo = 2147483647, hi = -2147483647 - 1;
  for (int64_t t = 0; t < (int64_t)n * k; ++t) {
    if (idx[t] < lo) lo = idx[t];
    if (idx[t] > hi) hi = idx[t];
  }
  return (lo >= 1 && hi <= n) ? 1 : 0;
}

/* range / finiteness validation, src/tsne_neighbors.cpp:630-640.
 * Returns 0 = ok, 1 = index out of range, 2 = distance not finite/negative. */
int orc_validate_knn(const int* idx, const float* dist, int n, int k, int offset) {
  for (int i = 0; i < n; ++i) {
    for (int j = 0; j < k; ++j) {
      const int nb = idx[(int64_t)j * n + i] - offset;
      if (nb < 0 || nb >= n) return 1;
      const float d = dist[(int64_t)j * n + i];
      if (!isfinite(d) || d < 0.0f) return 2;
    }
  }
  return 0;
}

/* compute_row_probabilities_float, src/tsne_neighbors.cpp:532-614 (FP32, min-shifted) */
static void row_p_f32(const float* dist, int n, int k, int row, double perplexity, float* row_p) {
  for (int j = 0; j < k; ++j) row_p[j] = 0.0f;
  float min_d2 = FLT_MAX, max_d2 = 0.0f;
  for (int j = 0; j < k; ++j) {
    const float d = dist[(int64_t)j * n + row];
    const float d2 = d * d;
    min_d2 = fminf_(min_d2, d2);
    max_d2 = fmaxf_(max_d2, d2);
  }
  const float spread = max_d2 - min_d2;
  if (spread <= FLT_EPSILON * fmaxf_(1.0f, max_d2)) {
    const float uniform = 1.0f / (float)k;
    for (int j = 0; j < k; ++j) row_p[j] = uniform;
    return;
  }
  int found = 0;
  float beta = 1.0f, min_beta = -FLT_MAX, max_beta = FLT_MAX;
  const float tol = 1e-5f;
  float sum_p = FLT_MIN;
  const float target = (float)log(perplexity);
  for (int iter = 0; !found && iter < 200; ++iter) {
    sum_p = FLT_MIN;
    for (int j = 0; j < k; ++j) {
      const float d = dist[(int64_t)j * n + row];
      const float d2 = d * d - min_d2;
      const float p = expf(-beta * d2);
      row_p[j] = p;
      sum_p += p;
    }
    float entropy = 0.0f;
    for (int j = 0; j < k; ++j) {
      const float d = dist[(int64_t)j * n + row];
      entropy += beta * ((d * d - min_d2) * row_p[j]);
    }
    entropy = entropy / sum_p + logf(sum_p);
    const float diff = entropy - target;
    if (fabsf(diff) < tol) {
      found = 1;
    } else if (diff > 0.0f) {
      min_beta = beta;
      beta = (max_beta == FLT_MAX || max_beta == -FLT_MAX) ? beta * 2.0f : (beta + max_beta) * 0.5f;
    } else {
      max_beta = beta;
      beta = (min_beta == -FLT_MAX || min_beta == FLT_MAX) ? beta * 0.5f : (beta + min_beta) * 0.5f;
    }
    if (!isfinite(beta)) break;
  }
  if (!isfinite(sum_p) || sum_p <= FLT_MIN) {
    int tied = 0;
    for (int j = 0; j < k; ++j) {
      const float d = dist[(int64_t)j * n + row];
      const float d2 = d * d;
      if (fabsf(d2 - min_d2) <= FLT_EPSILON * fmaxf_(1.0f, min_d2)) ++tied;
    }
    const float tied_mass = 1.0f / (float)(tied > 1 ? tied : 1);
    for (int j = 0; j < k; ++j) {
      const float d = dist[(int64_t)j * n + row];
      const float d2 = d * d;
      row_p[j] = fabsf(d2 - min_d2) <= FLT_EPSILON * fmaxf_(1.0f, min_d2) ? tied_mass : 0.0f;
    }
    return;
  }
  const float inv_sum_p = 1.0f / sum_p;
  for (int j = 0; j < k; ++j) row_p[j] *= inv_sum_p;
}

void orc_row_p_f32(const float* dist, int n, int k, double perplexity, float* p) {
#pragma omp parallel for schedule(static)
  for (int i = 0; i < n; ++i) row_p_f32(dist, n, k, i, perplexity, p + (int64_t)i * k);
}

/* FP64 bisection of tests/testthat/helper-tsne-reference.R:1-54 (min-shifted d^2,
 * same update rule and tolerance as the reference CPU path). */
void orc_row_p_f64(const float* dist, int n, int k, double perplexity, double* p, double* beta_out) {
  const double target = log(perplexity);
#pragma omp parallel for schedule(static)
  for (int i = 0; i < n; ++i) {
    double* row = p + (int64_t)i * k;
    double min_d2 = DBL_MAX, max_d2 = 0.0, max_shift = 0.0;
    for (int j = 0; j < k; ++j) {
      const double d = dist[(int64_t)j * n + i];
      const double d2 = d * d;
      if (d2 < min_d2) min_d2 = d2;
      if (d2 > max_d2) max_d2 = d2;
    }
    for (int j = 0; j < k; ++j) {
      const double d = dist[(int64_t)j * n + i];
      const double s = d * d - min_d2;
      if (s > max_shift) max_shift = s;
    }
    if (max_shift <= DBL_EPSILON * (max_d2 > 1.0 ? max_d2 : 1.0)) {
      for (int j = 0; j < k; ++j) row[j] = 1.0 / k;
      if (beta_out) beta_out[i] = 1.0;
      continue;
    }
    double beta = 1.0, beta_min = -INFINITY, beta_max = INFINITY, mass = 0.0;
    for (int it = 0; it < 200; ++it) {
      mass = 0.0;
      double wsum = 0.0;
      for (int j = 0; j < k; ++j) {
        const double d = dist[(int64_t)j * n + i];
        const double s = d * d - min_d2;
        row[j] = exp(-beta * s);
        mass += row[j];
        wsum += s * row[j];
      }
      const double entropy = beta * wsum / mass + log(mass);
      const double diff = entropy - target;
      if (fabs(diff) < 1e-5) break;
      if (diff > 0) {
        beta_min = beta;
        beta = isinf(beta_max) ? 2.0 * beta : 0.5 * (beta + beta_max);
      } else {
        beta_max = beta;
        beta = isinf(beta_min) ? 0.5 * beta : 0.5 * (beta + beta_min);
      }
    }
    for (int j = 0; j < k; ++j) row[j] /= mass;
    if (beta_out) beta_out[i] = beta;
  }
}

/* ---- stable LSD radix sort of (key, value) pairs on the bits that vary ---- */
typedef struct { uint64_t key; float value; } orc_edge;

static void radix_sort_edges(orc_edge* a, int64_t m, int key_bits) {
  orc_edge* tmp = (orc_edge*)malloc((size_t)(m > 0 ? m : 1) * sizeof(orc_edge));
  static const int kShiftsMax = 8;
  int shifts[16];
  int ns = 0;
  const int half_passes = (key_bits + 7) / 8;
  for (int p = 0; p < half_passes && p < kShiftsMax; ++p) shifts[ns++] = 8 * p;
  for (int p = 0; p < half_passes && p < kShiftsMax; ++p) shifts[ns++] = 32 + 8 * p;
  orc_edge* src = a;
  orc_edge* dst = tmp;
  for (int s = 0; s < ns; ++s) {
    int64_t count[257];
    memset(count, 0, sizeof(count));
    const int sh = shifts[s];
    for (int64_t t = 0; t < m; ++t) count[((src[t].key >> sh) & 255u) + 1]++;
    for (int d = 0; d < 256; ++d) count[d + 1] += count[d];
    for (int64_t t = 0; t < m; ++t) dst[count[(src[t].key >> sh) & 255u]++] = src[t];
    orc_edge* sw = src; src = dst; dst = sw;
  }
  if (src != a) memcpy(a, src, (size_t)m * sizeof(orc_edge));
  free(tmp);
}

/* build_tsne_probabilities_float, src/tsne_neighbors.cpp:616-724: (min,max) pair keys,
 * sort, double sums of duplicates, both-direction CSR fill, value = float(sum) * float(0.5/total). */
int64_t orc_csr_build(const int* idx, const float* p, int n, int k, int offset,
                      int* row_ptr, int* col, float* val, int64_t cap, double* total_mass) {
  orc_edge* edges = (orc_edge*)malloc((size_t)n * k * sizeof(orc_edge));
  int64_t m = 0;
  for (int i = 0; i < n; ++i) {
    for (int j = 0; j < k; ++j) {
      const int nb = idx[(int64_t)j * n + i] - offset;
      if (nb == i) continue;
      const uint32_t a = (uint32_t)(i < nb ? i : nb);
      const uint32_t b = (uint32_t)(i < nb ? nb : i);
      edges[m].key = ((uint64_t)a << 32) | b;
      edges[m].value = p[(int64_t)i * k + j];
      ++m;
    }
  }
  int bits = 1;
  while ((1LL << bits) < n) ++bits;
  radix_sort_edges(edges, m, bits);
  for (int i = 0; i <= n; ++i) row_ptr[i] = 0;
  int64_t write = 0;
  double total = 0.0;
  for (int64_t r = 0; r < m;) {
    const uint64_t key = edges[r].key;
    double sum = 0.0;
    while (r < m && edges[r].key == key) {
      sum += (double)edges[r].value;
      ++r;
    }
    edges[write].key = key;
    edges[write].value = (float)sum;
    ++write;
    total += sum;
    row_ptr[(key >> 32) + 1]++;
    row_ptr[(key & 0xffffffffu) + 1]++;
  }
  for (int i = 0; i < n; ++i) row_ptr[i + 1] += row_ptr[i];
  if (total_mass) *total_mass = total;
  const int64_t nnz = row_ptr[n];
  if (col == NULL || nnz > cap) {
    free(edges);
    return nnz;
  }
  int* fill = (int*)malloc(sizeof(int) * (size_t)(n + 1));
  memcpy(fill, row_ptr, sizeof(int) * (size_t)(n + 1));
  const float norm = (float)(0.5 / total);
  for (int64_t t = 0; t < write; ++t) {
    const int a = (int)(edges[t].key >> 32);
    const int b = (int)(edges[t].key & 0xffffffffu);
    const float value = edges[t].value * norm;
    int pos = fill[a]++;
    col[pos] = b;
    val[pos] = value;
    pos = fill[b]++;
    col[pos] = a;
    val[pos] = value;
  }
  free(fill);
  free(edges);
  return nnz;
}

/* tsne_fft_grid_size, src/tsne_neighbors.cpp:403-413 (without the env override) */
int orc_fft_grid_size_cpu(int n) {
  const int requested = n >= 50000 ? 256 : 128;
  int grid = 32;
  while (grid < requested && grid < 512) grid <<= 1;
  return grid < 32 ? 32 : (grid > 512 ? 512 : grid);
}

/* add_sparse_attractive_gradient_f, src/tsne_neighbors.cpp:1061-1088 */
void orc_attractive(const int* row_ptr, const int* col, const float* val, const float* y,
                    int n, float exaggeration, float* out) {
#pragma omp parallel for schedule(static)
  for (int i = 0; i < n; ++i) {
    float gx = 0.0f, gy = 0.0f;
    for (int pos = row_ptr[i]; pos < row_ptr[i + 1]; ++pos) {
      const int j = col[pos];
      const float dx = y[2 * (int64_t)i] - y[2 * (int64_t)j];
      const float dy = y[2 * (int64_t)i + 1] - y[2 * (int64_t)j + 1];
      float d2 = 0.0f;
      d2 += dx * dx;
      d2 += dy * dy;
      const float q = 1.0f / (1.0f + d2);
      const float coeff = exaggeration * val[pos] * q;
      gx += coeff * dx;
      gy += coeff * dy;
    }
    out[2 * (int64_t)i] = gx;
    out[2 * (int64_t)i + 1] = gy;
  }
}

/* repulsive half of compute_gradient_pair_symmetric_f, src/tsne_neighbors.cpp:1090-1150
 * (single worker: the reference's per-thread sums collapse to one) */
void orc_exact_rep_f32(const float* y, int n, float* rep, double* sum_q_out) {
  for (int64_t t = 0; t < 2 * (int64_t)n; ++t) rep[t] = 0.0f;
  double sum_q = 0.0;
  for (int i = 0; i < n - 1; ++i) {
    for (int j = i + 1; j < n; ++j) {
      float d2 = 0.0f;
      for (int d = 0; d < 2; ++d) {
        const float diff = y[2 * (int64_t)i + d] - y[2 * (int64_t)j + d];
        d2 += diff * diff;
      }
      const float q = 1.0f / (1.0f + d2);
      sum_q += 2.0 * (double)q;
      const float coeff = -(q * q);
      for (int d = 0; d < 2; ++d) {
        const float step = coeff * (y[2 * (int64_t)i + d] - y[2 * (int64_t)j + d]);
        rep[2 * (int64_t)i + d] += step;
        rep[2 * (int64_t)j + d] -= step;
      }
    }
  }
  const double s = sum_q > (double)FLT_MIN ? sum_q : (double)FLT_MIN;
  const float inv = (float)(1.0 / s);
  for (int64_t t = 0; t < 2 * (int64_t)n; ++t) rep[t] = (0.0f + rep[t]) * inv;
  if (sum_q_out) *sum_q_out = sum_q;
}

/* FP64 exact repulsion (the dense oracle of tests/testthat/helper-tsne-reference.R:56-98) */
void orc_exact_rep_f64(const float* y, int n, double* rep, double* sum_q_out) {
  double sum_q = 0.0;
#pragma omp parallel for schedule(dynamic, 64) reduction(+ : sum_q)
  for (int i = 0; i < n; ++i) {
    const double xi = y[2 * (int64_t)i], yi = y[2 * (int64_t)i + 1];
    double gx = 0.0, gy = 0.0, zs = 0.0;
    for (int j = 0; j < n; ++j) {
      if (j == i) continue;
      const double dx = xi - y[2 * (int64_t)j], dy = yi - y[2 * (int64_t)j + 1];
      const double q = 1.0 / (1.0 + dx * dx + dy * dy);
      zs += q;
      gx += q * q * dx;
      gy += q * q * dy;
    }
    rep[2 * (int64_t)i] = gx;
    rep[2 * (int64_t)i + 1] = gy;
    sum_q += zs;
  }
  for (int64_t t = 0; t < 2 * (int64_t)n; ++t) rep[t] = -rep[t] / sum_q;
  if (sum_q_out) *sum_q_out = sum_q;
}

/* ---------------- radix-2 FFT, FftPlanT / fft_1d_t, src/tsne_neighbors.cpp:726-805 ---------------- */
typedef struct {
  int size;
  int* bitrev;
  float* fwd; /* per stage (re, im) */
  float* inv;
} fplan;

static void fplan_init(fplan* p, int size) {
  p->size = size;
  int bits = 0;
  for (int v = size; v > 1; v >>= 1) ++bits;
  p->bitrev = (int*)malloc(sizeof(int) * (size_t)size);
  for (int i = 0; i < size; ++i) {
    unsigned v = (unsigned)i, r = 0u;
    for (int b = 0; b < bits; ++b) {
      r = (r << 1u) | (v & 1u);
      v >>= 1u;
    }
    p->bitrev[i] = (int)r;
  }
  p->fwd = (float*)malloc(sizeof(float) * 2 * (size_t)(bits + 1));
  p->inv = (float*)malloc(sizeof(float) * 2 * (size_t)(bits + 1));
  int s = 0;
  for (int len = 2; len <= size; len <<= 1, ++s) {
    const float angle = 6.283185307179586476925286766559f / (float)len;
    p->fwd[2 * s] = cosf(angle);
    p->fwd[2 * s + 1] = sinf(angle);
    p->inv[2 * s] = cosf(-angle);
    p->inv[2 * s + 1] = sinf(-angle);
  }
}

static void fplan_free(fplan* p) {
  free(p->bitrev);
  free(p->fwd);
  free(p->inv);
}

/* complex float multiply as std::complex<float> does it for finite values */
static inline void cmulf(float ar, float ai, float br, float bi, float* cr, float* ci) {
  *cr = ar * br - ai * bi;
  *ci = ar * bi + ai * br;
}

static void fft1_f(float* a, int n, int inverse, const fplan* p) {
  for (int i = 1; i < n; ++i) {
    const int j = p->bitrev[i];
    if (i < j) {
      float t0 = a[2 * i], t1 = a[2 * i + 1];
      a[2 * i] = a[2 * j];
      a[2 * i + 1] = a[2 * j + 1];
      a[2 * j] = t0;
      a[2 * j + 1] = t1;
    }
  }
  const float* roots = inverse ? p->inv : p->fwd;
  int stage = 0;
  for (int len = 2; len <= n; len <<= 1, ++stage) {
    const float rr = roots[2 * stage], ri = roots[2 * stage + 1];
    const int half = len >> 1;
    for (int i = 0; i < n; i += len) {
      float wr = 1.0f, wi = 0.0f;
      for (int j = 0; j < half; ++j) {
        const float ur = a[2 * (i + j)], ui = a[2 * (i + j) + 1];
        float vr, vi;
        cmulf(a[2 * (i + j + half)], a[2 * (i + j + half) + 1], wr, wi, &vr, &vi);
        a[2 * (i + j)] = ur + vr;
        a[2 * (i + j) + 1] = ui + vi;
        a[2 * (i + j + half)] = ur - vr;
        a[2 * (i + j + half) + 1] = ui - vi;
        float nr, ni;
        cmulf(wr, wi, rr, ri, &nr, &ni);
        wr = nr;
        wi = ni;
      }
    }
  }
  if (inverse) {
    const float scale = 1.0f / (float)n;
    for (int i = 0; i < 2 * n; ++i) a[i] *= scale;
  }
}

/* fft_2d_t, src/tsne_neighbors.cpp:807-834 */
static void fft2_f(float* v, int size, int inverse, const fplan* p) {
#pragma omp parallel for schedule(static)
  for (int r = 0; r < size; ++r) fft1_f(v + 2 * (int64_t)r * size, size, inverse, p);
#pragma omp parallel
  {
    float* colbuf = (float*)malloc(sizeof(float) * 2 * (size_t)size);
#pragma omp for schedule(static)
    for (int c = 0; c < size; ++c) {
      for (int r = 0; r < size; ++r) {
        colbuf[2 * r] = v[2 * ((int64_t)r * size + c)];
        colbuf[2 * r + 1] = v[2 * ((int64_t)r * size + c) + 1];
      }
      fft1_f(colbuf, size, inverse, p);
      for (int r = 0; r < size; ++r) {
        v[2 * ((int64_t)r * size + c)] = colbuf[2 * r];
        v[2 * ((int64_t)r * size + c) + 1] = colbuf[2 * r + 1];
      }
    }
    free(colbuf);
  }
}

/* bilinear_grid_value_t, src/tsne_neighbors.cpp:836-857 */
static float bilinear_value(const float* grid, int g, float gx, float gy) {
  const float cx = fmaxf_(0.0f, fminf_((float)(g - 1), gx));
  const float cy = fmaxf_(0.0f, fminf_((float)(g - 1), gy));
  int x0 = (int)floorf(cx), y0 = (int)floorf(cy);
  if (x0 > g - 2) x0 = g - 2;
  if (x0 < 0) x0 = 0;
  if (y0 > g - 2) y0 = g - 2;
  if (y0 < 0) y0 = 0;
  const float tx = cx - (float)x0, ty = cy - (float)y0;
  const int x1 = x0 + 1, y1 = y0 + 1;
  const float v00 = grid[(int64_t)y0 * g + x0], v10 = grid[(int64_t)y0 * g + x1];
  const float v01 = grid[(int64_t)y1 * g + x0], v11 = grid[(int64_t)y1 * g + x1];
  return (1.0f - tx) * (1.0f - ty) * v00 + tx * (1.0f - ty) * v10 + (1.0f - tx) * ty * v01 + tx * ty * v11;
}

/* compute_gradient_fft_grid_f (repulsive part), src/tsne_neighbors.cpp:1152-1258, with the
 * convolution of compute_fft_grid_convolution_workspace_t, :956-1018. rep_out receives the
 * gradient before the attractive term is added; z_out = sum_i q_grid(y_i) - n. */
void orc_fft_grid_rep_f32(const float* y, int n, int grid_size, float* rep, double* z_out) {
  const int g = grid_size;
  float min_x = y[0], max_x = y[0], min_y = y[1], max_y = y[1];
  for (int i = 1; i < n; ++i) {
    min_x = fminf_(min_x, y[2 * (int64_t)i]);
    max_x = fmaxf_(max_x, y[2 * (int64_t)i]);
    min_y = fminf_(min_y, y[2 * (int64_t)i + 1]);
    max_y = fmaxf_(max_y, y[2 * (int64_t)i + 1]);
  }
  const float cx = 0.5f * (min_x + max_x), cy = 0.5f * (min_y + max_y);
  float span = fmaxf_(max_x - min_x, max_y - min_y);
  if (!isfinite(span) || span <= 0.0f) span = 1.0f;
  const float half = 0.55f * span + 1.0e-3f;
  const float lower_x = cx - half, lower_y = cy - half;
  const float spacing = (2.0f * half) / (float)(g - 1);
  const float inv_spacing = 1.0f / spacing;
  const int64_t gt = (int64_t)g * g;
  float* mass = (float*)calloc((size_t)gt, sizeof(float));
  float* mx = (float*)calloc((size_t)gt, sizeof(float));
  float* my = (float*)calloc((size_t)gt, sizeof(float));
  float* gxs = (float*)malloc(sizeof(float) * (size_t)n);
  float* gys = (float*)malloc(sizeof(float) * (size_t)n);
  for (int i = 0; i < n; ++i) {
    const float xc = y[2 * (int64_t)i], yc = y[2 * (int64_t)i + 1];
    const float raw_x = (xc - lower_x) * inv_spacing, raw_y = (yc - lower_y) * inv_spacing;
    const float clx = fmaxf_(0.0f, fminf_((float)(g - 1), raw_x));
    const float cly = fmaxf_(0.0f, fminf_((float)(g - 1), raw_y));
    int x0 = (int)floorf(clx), y0 = (int)floorf(cly);
    if (x0 > g - 2) x0 = g - 2;
    if (x0 < 0) x0 = 0;
    if (y0 > g - 2) y0 = g - 2;
    if (y0 < 0) y0 = 0;
    const int x1 = x0 + 1, y1 = y0 + 1;
    const float tx = clx - (float)x0, ty = cly - (float)y0;
    gxs[i] = clx;
    gys[i] = cly;
    const float w00 = (1.0f - tx) * (1.0f - ty), w10 = tx * (1.0f - ty);
    const float w01 = (1.0f - tx) * ty, w11 = tx * ty;
    const int64_t p00 = (int64_t)y0 * g + x0, p10 = (int64_t)y0 * g + x1;
    const int64_t p01 = (int64_t)y1 * g + x0, p11 = (int64_t)y1 * g + x1;
    mass[p00] += w00; mass[p10] += w10; mass[p01] += w01; mass[p11] += w11;
    mx[p00] += w00 * xc; mx[p10] += w10 * xc; mx[p01] += w01 * xc; mx[p11] += w11 * xc;
    my[p00] += w00 * yc; my[p10] += w10 * yc; my[p01] += w01 * yc; my[p11] += w11 * yc;
  }
  const int m = 2 * g;
  const int64_t mt = (int64_t)m * m;
  float* fmass = (float*)calloc((size_t)(2 * mt), sizeof(float));
  float* fmx = (float*)calloc((size_t)(2 * mt), sizeof(float));
  float* fmy = (float*)calloc((size_t)(2 * mt), sizeof(float));
  float* kq = (float*)calloc((size_t)(2 * mt), sizeof(float));
  float* kq2 = (float*)calloc((size_t)(2 * mt), sizeof(float));
  float* work = (float*)malloc(sizeof(float) * 2 * (size_t)mt);
  for (int r = 0; r < g; ++r) {
    for (int c = 0; c < g; ++c) {
      fmass[2 * ((int64_t)r * m + c)] = mass[(int64_t)r * g + c];
      fmx[2 * ((int64_t)r * m + c)] = mx[(int64_t)r * g + c];
      fmy[2 * ((int64_t)r * m + c)] = my[(int64_t)r * g + c];
    }
  }
  for (int row = 0; row < 2 * g - 1; ++row) {
    const int dy = row - (g - 1);
    const int yy = dy < 0 ? dy + m : dy;
    const float yo = (float)dy * spacing;
    for (int dx = -(g - 1); dx <= g - 1; ++dx) {
      const int xx = dx < 0 ? dx + m : dx;
      const float xo = (float)dx * spacing;
      const float d2 = xo * xo + yo * yo;
      const float q = 1.0f / (1.0f + d2);
      kq[2 * ((int64_t)yy * m + xx)] = q;
      kq2[2 * ((int64_t)yy * m + xx)] = q * q;
    }
  }
  fplan plan;
  fplan_init(&plan, m);
  fft2_f(fmass, m, 0, &plan);
  fft2_f(fmx, m, 0, &plan);
  fft2_f(fmy, m, 0, &plan);
  fft2_f(kq, m, 0, &plan);
  fft2_f(kq2, m, 0, &plan);
  float* qg = (float*)malloc(sizeof(float) * (size_t)gt);
  float* q2g = (float*)malloc(sizeof(float) * (size_t)gt);
  float* xq2g = (float*)malloc(sizeof(float) * (size_t)gt);
  float* yq2g = (float*)malloc(sizeof(float) * (size_t)gt);
  const float* srcs[4] = {fmass, fmass, fmx, fmy};
  const float* kers[4] = {kq, kq2, kq2, kq2};
  float* outs[4] = {qg, q2g, xq2g, yq2g};
  for (int o = 0; o < 4; ++o) {
    for (int64_t t = 0; t < mt; ++t) {
      cmulf(srcs[o][2 * t], srcs[o][2 * t + 1], kers[o][2 * t], kers[o][2 * t + 1], &work[2 * t], &work[2 * t + 1]);
    }
    fft2_f(work, m, 1, &plan);
    for (int r = 0; r < g; ++r)
      for (int c = 0; c < g; ++c) outs[o][(int64_t)r * g + c] = work[2 * ((int64_t)r * m + c)];
  }
  double sum_q = 0.0;
  for (int i = 0; i < n; ++i) sum_q += (double)bilinear_value(qg, g, gxs[i], gys[i]);
  const double zz = sum_q - (double)n;
  const float inv_sum_q = (float)(1.0 / (zz > (double)FLT_MIN ? zz : (double)FLT_MIN));
#pragma omp parallel for schedule(static)
  for (int i = 0; i < n; ++i) {
    const float px = gxs[i], py = gys[i];
    const float q2v = bilinear_value(q2g, g, px, py);
    const float xq2v = bilinear_value(xq2g, g, px, py);
    const float yq2v = bilinear_value(yq2g, g, px, py);
    rep[2 * (int64_t)i] = -(y[2 * (int64_t)i] * q2v - xq2v) * inv_sum_q;
    rep[2 * (int64_t)i + 1] = -(y[2 * (int64_t)i + 1] * q2v - yq2v) * inv_sum_q;
  }
  if (z_out) *z_out = zz;
  fplan_free(&plan);
  free(mass); free(mx); free(my); free(gxs); free(gys);
  free(fmass); free(fmx); free(fmy); free(kq); free(kq2); free(work);
  free(qg); free(q2g); free(xq2g); free(yq2g);
}

/* ---------------- FP64 oracle of the product's interpolation scheme ----------------
 * Same algebra as the reference grid gradient, evaluated in double with an FP64 FFT:
 *   lagrange = 0: bilinear splat on G shared nodes (the reference stencil);
 *   lagrange = 1: 3 equispaced Lagrange nodes per box, floor(G/3) boxes per side.
 * Charges are taken relative to the grid centre; Z = sum_i phi_q(y_i) - n. */
static void fft1_d(double* a, int n, int inverse) {
  for (int i = 1, j = 0; i < n; ++i) {
    int bit = n >> 1;
    for (; j & bit; bit >>= 1) j ^= bit;
    j ^= bit;
    if (i < j) {
      double t0 = a[2 * i], t1 = a[2 * i + 1];
      a[2 * i] = a[2 * j]; a[2 * i + 1] = a[2 * j + 1];
      a[2 * j] = t0; a[2 * j + 1] = t1;
    }
  }
  for (int len = 2; len <= n; len <<= 1) {
    const int half = len >> 1;
    for (int j = 0; j < half; ++j) {
      const double ang = (inverse ? 2.0 : -2.0) * M_PI * (double)j / (double)len;
      const double wr = cos(ang), wi = sin(ang);
      for (int i = 0; i < n; i += len) {
        const double ur = a[2 * (i + j)], ui = a[2 * (i + j) + 1];
        const double xr = a[2 * (i + j + half)], xi = a[2 * (i + j + half) + 1];
        const double vr = xr * wr - xi * wi, vi = xr * wi + xi * wr;
        a[2 * (i + j)] = ur + vr; a[2 * (i + j) + 1] = ui + vi;
        a[2 * (i + j + half)] = ur - vr; a[2 * (i + j + half) + 1] = ui - vi;
      }
    }
  }
  if (inverse)
    for (int i = 0; i < 2 * n; ++i) a[i] /= (double)n;
}

static void fft2_d(double* v, int size, int inverse) {
#pragma omp parallel for schedule(static)
  for (int r = 0; r < size; ++r) fft1_d(v + 2 * (int64_t)r * size, size, inverse);
#pragma omp parallel
  {
    double* cb = (double*)malloc(sizeof(double) * 2 * (size_t)size);
#pragma omp for schedule(static)
    for (int c = 0; c < size; ++c) {
      for (int r = 0; r < size; ++r) {
        cb[2 * r] = v[2 * ((int64_t)r * size + c)];
        cb[2 * r + 1] = v[2 * ((int64_t)r * size + c) + 1];
      }
      fft1_d(cb, size, inverse);
      for (int r = 0; r < size; ++r) {
        v[2 * ((int64_t)r * size + c)] = cb[2 * r];
        v[2 * ((int64_t)r * size + c) + 1] = cb[2 * r + 1];
      }
    }
    free(cb);
  }
}

typedef struct { int base; double w[3]; } stencil1d;

static stencil1d make_stencil(double x, double x0, double h, int nodes, int lagrange) {
  stencil1d s;
  if (!lagrange) {
    double t = (x - x0) / h;
    if (t < 0.0) t = 0.0;
    if (t > (double)(nodes - 1)) t = (double)(nodes - 1);
    int u0 = (int)floor(t);
    if (u0 > nodes - 2) u0 = nodes - 2;
    if (u0 < 0) u0 = 0;
    const double f = t - (double)u0;
    s.base = u0;
    s.w[0] = 1.0 - f;
    s.w[1] = f;
    s.w[2] = 0.0;
  } else {
    const int nbox = nodes / 3;
    const double box = 3.0 * h;
    int b = (int)floor((x - x0) / box);
    if (b < 0) b = 0;
    if (b > nbox - 1) b = nbox - 1;
    const double t = (x - x0) / h - 3.0 * b - 0.5;
    s.base = 3 * b;
    s.w[0] = 0.5 * (t - 1.0) * (t - 2.0);
    s.w[1] = t * (2.0 - t);
    s.w[2] = 0.5 * t * (t - 1.0);
  }
  return s;
}

void orc_interp_rep_f64(const float* y, int n, int grid_size, int lagrange, double* rep, double* z_out) {
  double min_x = y[0], max_x = y[0], min_y = y[1], max_y = y[1];
  for (int i = 1; i < n; ++i) {
    if (y[2 * (int64_t)i] < min_x) min_x = y[2 * (int64_t)i];
    if (y[2 * (int64_t)i] > max_x) max_x = y[2 * (int64_t)i];
    if (y[2 * (int64_t)i + 1] < min_y) min_y = y[2 * (int64_t)i + 1];
    if (y[2 * (int64_t)i + 1] > max_y) max_y = y[2 * (int64_t)i + 1];
  }
  const double cx = 0.5 * (min_x + max_x), cy = 0.5 * (min_y + max_y);
  double span = (max_x - min_x) > (max_y - min_y) ? (max_x - min_x) : (max_y - min_y);
  if (!(span > 0.0) || !isfinite(span)) span = 1.0;
  const double half = 0.55 * span + 1.0e-3;
  const int g = grid_size;
  const int nodes = lagrange ? 3 * (g / 3) : g;
  const double h = lagrange ? (2.0 * half) / (double)(g / 3) / 3.0 : (2.0 * half) / (double)(g - 1);
  const double x0 = cx - half, y0 = cy - half;
  const int m = 2 * g;
  const int64_t mt = (int64_t)m * m;
  double* cm = (double*)calloc((size_t)(2 * mt), sizeof(double));  /* mass */
  double* cxg = (double*)calloc((size_t)(2 * mt), sizeof(double)); /* mx */
  double* cyg = (double*)calloc((size_t)(2 * mt), sizeof(double)); /* my */
  double* kq = (double*)calloc((size_t)(2 * mt), sizeof(double));
  double* kq2 = (double*)calloc((size_t)(2 * mt), sizeof(double));
  const int taps = lagrange ? 3 : 2;
  for (int i = 0; i < n; ++i) {
    const double px = y[2 * (int64_t)i], py = y[2 * (int64_t)i + 1];
    const stencil1d sx = make_stencil(px, x0, h, nodes, lagrange);
    const stencil1d sy = make_stencil(py, y0, h, nodes, lagrange);
    for (int a = 0; a < taps; ++a)
      for (int b = 0; b < taps; ++b) {
        const double w = sy.w[a] * sx.w[b];
        const int64_t pos = 2 * ((int64_t)(sy.base + a) * m + (sx.base + b));
        cm[pos] += w;
        cxg[pos] += w * (px - cx);
        cyg[pos] += w * (py - cy);
      }
  }
  for (int r = 0; r < m; ++r) {
    const int dy = r < g ? r : r - m;
    if (r == g) continue;
    for (int c = 0; c < m; ++c) {
      const int dx = c < g ? c : c - m;
      if (c == g) continue;
      const double d2 = h * h * ((double)dx * dx + (double)dy * dy);
      const double q = 1.0 / (1.0 + d2);
      kq[2 * ((int64_t)r * m + c)] = q;
      kq2[2 * ((int64_t)r * m + c)] = q * q;
    }
  }
  fft2_d(cm, m, 0); fft2_d(cxg, m, 0); fft2_d(cyg, m, 0); fft2_d(kq, m, 0); fft2_d(kq2, m, 0);
  double* phi[4];
  const double* srcs[4] = {cm, cm, cxg, cyg};
  const double* kers[4] = {kq, kq2, kq2, kq2};
  for (int o = 0; o < 4; ++o) {
    phi[o] = (double*)malloc(sizeof(double) * 2 * (size_t)mt);
    for (int64_t t = 0; t < mt; ++t) {
      const double ar = srcs[o][2 * t], ai = srcs[o][2 * t + 1];
      const double br = kers[o][2 * t], bi = kers[o][2 * t + 1];
      phi[o][2 * t] = ar * br - ai * bi;
      phi[o][2 * t + 1] = ar * bi + ai * br;
    }
    fft2_d(phi[o], m, 1);
  }
  double* pv = (double*)malloc(sizeof(double) * 4 * (size_t)n);
#pragma omp parallel for schedule(static)
  for (int i = 0; i < n; ++i) {
    const double px = y[2 * (int64_t)i], py = y[2 * (int64_t)i + 1];
    const stencil1d sx = make_stencil(px, x0, h, nodes, lagrange);
    const stencil1d sy = make_stencil(py, y0, h, nodes, lagrange);
    double acc[4] = {0, 0, 0, 0};
    for (int a = 0; a < taps; ++a)
      for (int b = 0; b < taps; ++b) {
        const double w = sy.w[a] * sx.w[b];
        const int64_t pos = 2 * ((int64_t)(sy.base + a) * m + (sx.base + b));
        for (int o = 0; o < 4; ++o) acc[o] += w * phi[o][pos];
      }
    for (int o = 0; o < 4; ++o) pv[4 * (int64_t)i + o] = acc[o];
  }
  double zs = 0.0;
  for (int i = 0; i < n; ++i) zs += pv[4 * (int64_t)i];
  const double z = zs - (double)n;
  for (int i = 0; i < n; ++i) {
    const double px = (double)y[2 * (int64_t)i] - cx, py = (double)y[2 * (int64_t)i + 1] - cy;
    rep[2 * (int64_t)i] = -(px * pv[4 * (int64_t)i + 1] - pv[4 * (int64_t)i + 2]) / z;
    rep[2 * (int64_t)i + 1] = -(py * pv[4 * (int64_t)i + 1] - pv[4 * (int64_t)i + 3]) / z;
  }
  if (z_out) *z_out = z;
  for (int o = 0; o < 4; ++o) free(phi[o]);
  free(pv); free(cm); free(cxg); free(cyg); free(kq); free(kq2);
}

/* apply_open_tsne_update_f, src/tsne_neighbors.cpp:1293-1336 */
static float sign_f(float x) { return x == 0.0f ? 0.0f : (x < 0.0f ? -1.0f : 1.0f); }

void orc_update(float* y, float* update, float* gains, const float* grad, int n,
                float learning_rate, float momentum, float min_gain, float max_step_norm) {
  const int clip = isfinite(max_step_norm) && max_step_norm > 0.0f;
  const float max2 = max_step_norm * max_step_norm;
#pragma omp parallel for schedule(static)
  for (int i = 0; i < n; ++i) {
    float step2 = 0.0f;
    for (int d = 0; d < 2; ++d) {
      const int64_t t = 2 * (int64_t)i + d;
      if (sign_f(update[t]) != sign_f(grad[t])) gains[t] += 0.2f;
      else gains[t] = gains[t] * 0.8f + min_gain;
      if (gains[t] < min_gain) gains[t] = min_gain;
      update[t] = momentum * update[t] - learning_rate * gains[t] * grad[t];
      step2 += update[t] * update[t];
    }
    float scale = 1.0f;
    if (clip && step2 > max2) scale = max_step_norm / sqrtf(fmaxf_(step2, FLT_MIN));
    for (int d = 0; d < 2; ++d) {
      const int64_t t = 2 * (int64_t)i + d;
      update[t] *= scale;
      y[t] += update[t];
    }
  }
}

/* zero_mean_f, src/tsne_neighbors.cpp:1280-1291 */
void orc_zero_mean(float* y, int n) {
  double mean[2] = {0.0, 0.0};
  for (int i = 0; i < n; ++i)
    for (int d = 0; d < 2; ++d) mean[d] += y[2 * (int64_t)i + d];
  for (int d = 0; d < 2; ++d) mean[d] /= (double)n;
  for (int i = 0; i < n; ++i)
    for (int d = 0; d < 2; ++d) y[2 * (int64_t)i + d] -= (float)mean[d];
}

static float sqdist_f(const float* y, int i, int j) {
  float out = 0.0f;
  for (int d = 0; d < 2; ++d) {
    const float diff = y[2 * (int64_t)i + d] - y[2 * (int64_t)j + d];
    out += diff * diff;
  }
  return out;
}

/* compute_sum_q_f, src/tsne_neighbors.cpp:1034-1059 (returned as the float the reference keeps) */
double orc_sum_q(const float* y, int n) {
  double local = 0.0;
#pragma omp parallel for schedule(dynamic, 64) reduction(+ : local)
  for (int i = 0; i < n - 1; ++i) {
    double row = 0.0;
    for (int j = i + 1; j < n; ++j) row += 2.0 / (1.0 + (double)sqdist_f(y, i, j));
    local += row;
  }
  const double s = local > (double)FLT_MIN ? local : (double)FLT_MIN;
  return (double)(float)s;
}

/* evaluate_kl_f, src/tsne_neighbors.cpp:1338-1365 */
double orc_kl(const int* row_ptr, const int* col, const float* val, const float* y, int n) {
  const double sum_q = orc_sum_q(y, n);
  double total = 0.0;
  for (int i = 0; i < n; ++i) {
    double row_total = 0.0;
    for (int pos = row_ptr[i]; pos < row_ptr[i + 1]; ++pos) {
      const int j = col[pos];
      const double p = (double)val[pos];
      const double q = (1.0 / (1.0 + (double)sqdist_f(y, i, j))) / sum_q;
      row_total += p * log((p + 1e-9) / (q + 1e-9));
    }
    total += row_total;
  }
  return total;
}

/* ---------------- optimizer state (knn_tsne_opentsne_float_cpp, :1871-2121) ---------------- */
struct orc_tsne_state {
  int n, grid;
  int* row_ptr;
  int* col;
  float* val;
  float *y, *grad, *update, *gains, *rep, *attr;
};

orc_tsne_state* orc_tsne_prepare(const int* idx, const float* dist, int n, int k,
                                 const float* init, double perplexity, int grid_size) {
  orc_tsne_state* s = (orc_tsne_state*)calloc(1, sizeof(orc_tsne_state));
  s->n = n;
  s->grid = grid_size > 0 ? grid_size : orc_fft_grid_size_cpu(n);
  const int offset = orc_index_offset(idx, n, k);
  float* p = (float*)malloc(sizeof(float) * (size_t)n * k);
  orc_row_p_f32(dist, n, k, perplexity, p);
  s->row_ptr = (int*)malloc(sizeof(int) * (size_t)(n + 1));
  const int64_t cap = 2 * (int64_t)n * k;
  s->col = (int*)malloc(sizeof(int) * (size_t)cap);
  s->val = (float*)malloc(sizeof(float) * (size_t)cap);
  orc_csr_build(idx, p, n, k, offset, s->row_ptr, s->col, s->val, cap, NULL);
  free(p);
  s->y = (float*)malloc(sizeof(float) * 2 * (size_t)n);
  memcpy(s->y, init, sizeof(float) * 2 * (size_t)n);
  orc_zero_mean(s->y, n);
  s->grad = (float*)calloc(2 * (size_t)n, sizeof(float));
  s->update = (float*)calloc(2 * (size_t)n, sizeof(float));
  s->gains = (float*)malloc(sizeof(float) * 2 * (size_t)n);
  for (int64_t t = 0; t < 2 * (int64_t)n; ++t) s->gains[t] = 1.0f;
  s->rep = (float*)malloc(sizeof(float) * 2 * (size_t)n);
  s->attr = (float*)malloc(sizeof(float) * 2 * (size_t)n);
  return s;
}

static void tsne_gradient(orc_tsne_state* s, float exaggeration, int exact) {
  const int n = s->n;
  if (exact) orc_exact_rep_f32(s->y, n, s->rep, NULL);
  else orc_fft_grid_rep_f32(s->y, n, s->grid, s->rep, NULL);
  /* the reference accumulates attractive terms onto grad row by row */
#pragma omp parallel for schedule(static)
  for (int i = 0; i < n; ++i) {
    float gx = s->rep[2 * (int64_t)i], gy = s->rep[2 * (int64_t)i + 1];
    for (int pos = s->row_ptr[i]; pos < s->row_ptr[i + 1]; ++pos) {
      const int j = s->col[pos];
      const float dx = s->y[2 * (int64_t)i] - s->y[2 * (int64_t)j];
      const float dy = s->y[2 * (int64_t)i + 1] - s->y[2 * (int64_t)j + 1];
      float d2 = 0.0f;
      d2 += dx * dx;
      d2 += dy * dy;
      const float q = 1.0f / (1.0f + d2);
      const float coeff = exaggeration * s->val[pos] * q;
      gx += coeff * dx;
      gy += coeff * dy;
    }
    s->grad[2 * (int64_t)i] = gx;
    s->grad[2 * (int64_t)i + 1] = gy;
  }
}

void orc_tsne_iterate(orc_tsne_state* s, int iters, float exaggeration, float learning_rate,
                      float momentum, float min_gain, float max_step_norm) {
  for (int it = 0; it < iters; ++it) {
    tsne_gradient(s, exaggeration, 0);
    orc_update(s->y, s->update, s->gains, s->grad, s->n, learning_rate, momentum, min_gain, max_step_norm);
    orc_zero_mean(s->y, s->n);
  }
}

void orc_tsne_get_y(const orc_tsne_state* s, float* y_out) {
  memcpy(y_out, s->y, sizeof(float) * 2 * (size_t)s->n);
}

int64_t orc_tsne_nnz(const orc_tsne_state* s) { return s->row_ptr[s->n]; }

void orc_tsne_free(orc_tsne_state* s) {
  if (!s) return;
  free(s->row_ptr); free(s->col); free(s->val); free(s->y); free(s->grad);
  free(s->update); free(s->gains); free(s->rep); free(s->attr);
  free(s);
}

/* knn_tsne_opentsne_float_cpp run_phase schedule, src/tsne_neighbors.cpp:1976-2067
 * (auto KLD stop disabled, as for n > 5000 or auto_config = FALSE). */
int orc_tsne_run(const int* idx, const float* dist, int n, int k, const float* init,
                 double perplexity, int early_iter, int n_iter, double early_exag,
                 double exag, double learning_rate, int lr_auto, double m0, double m1,
                 double min_gain, double max_step_norm, int repulsion, int grid_size,
                 float* y_out, double* kl_trace, int* kl_iters, int kl_cap) {
  if (orc_validate_knn(idx, dist, n, k, orc_index_offset(idx, n, k)) != 0) return 1;
  orc_tsne_state* s = orc_tsne_prepare(idx, dist, n, k, init, perplexity, grid_size);
  const int total = early_iter + n_iter;
  int done = 0, nk = 0;
  for (int phase = 0; phase < 2; ++phase) {
    const int iters = phase == 0 ? early_iter : n_iter;
    const double ex = phase == 0 ? early_exag : exag;
    const double mom = phase == 0 ? m0 : m1;
    const float lr = (float)(lr_auto ? (double)n / (ex > DBL_MIN ? ex : DBL_MIN) : learning_rate);
    const float msn = isfinite(max_step_norm) ? (float)max_step_norm : NAN;
    for (int it = 0; it < iters; ++it) {
      tsne_gradient(s, (float)ex, repulsion == 1);
      orc_update(s->y, s->update, s->gains, s->grad, n, lr, (float)mom, (float)min_gain, msn);
      orc_zero_mean(s->y, n);
      ++done;
      if (kl_trace && nk < kl_cap && (done % 50 == 0 || done == total)) {
        kl_trace[nk] = orc_kl(s->row_ptr, s->col, s->val, s->y, n);
        if (kl_iters) kl_iters[nk] = done;
        ++nk;
      }
    }
  }
  orc_tsne_get_y(s, y_out);
  orc_tsne_free(s);
  return 0;
}
