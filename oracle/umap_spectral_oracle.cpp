// CPU oracle, UMAP spectral start. TEST INFRASTRUCTURE ONLY (see oracle.h).
//
// Restates initialize_layout_csr (fastEmbedR src/fast_knn_umap.cpp:2231-2528) as the CSR driver
// optimize_layout_csr (:3088-3205) calls it for fast_knn_umap_csr_cpp with n_epochs = 0
// (:5291-5321), with the optional scale_embedding_sdev (:2681-2703), sequentially (one worker).
// Written in C++ because the algorithm's random numbers are those of std::mt19937 with
// std::normal_distribution and std::uniform_real_distribution; the same library types
// reproduce them.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <numeric>
#include <random>
#include <vector>

#include "oracle.h"

namespace {

// block subspace iteration on D^-1/2 W D^-1/2 with Rayleigh-Ritz, :2244-2527
void spectral_layout(const int* offsets, const int* neighbors, const float* weights, int n, int n_iter,
                     std::mt19937& rng, double* emb) {
  const int comps = 2;
  std::normal_distribution<double> normal(0.0, 0.0001);
  std::uniform_real_distribution<double> uniform(-10.0, 10.0);
  auto random_layout = [&] {
    for (int c = 0; c < comps; ++c)
      for (int i = 0; i < n; ++i) emb[(size_t)c * n + i] = uniform(rng);
  };
  // edges (row, pos) with row < neighbour
  std::vector<int> erow, epos;
  for (int r = 0; r < n; ++r)
    for (int p = offsets[r]; p < offsets[r + 1]; ++p) {
      const int nb = neighbors[p];
      if (nb >= 0 && nb < n && nb != r && r < nb) {
        erow.push_back(r);
        epos.push_back(p);
      }
    }
  if (offsets[n] == 0 || erow.empty()) {
    random_layout();
    return;
  }
  std::vector<float> deg(n, 0.0f);
  for (int r = 0; r < n; ++r) {
    double s = 0.0;
    for (int p = offsets[r]; p < offsets[r + 1]; ++p) s += weights[p];
    deg[r] = (float)s;
  }
  // symmetric normalised adjacency: both ends of every edge, in edge order
  std::vector<int> cnt(n, 0);
  for (size_t e = 0; e < erow.size(); ++e) {
    ++cnt[erow[e]];
    ++cnt[neighbors[epos[e]]];
  }
  std::vector<int> so(n + 1, 0);
  for (int i = 0; i < n; ++i) so[i + 1] = so[i] + cnt[i];
  std::vector<int> cur(so.begin(), so.end() - 1), snb(so[n]);
  std::vector<float> sw(so[n]);
  for (size_t e = 0; e < erow.size(); ++e) {
    const int h = erow[e], t = neighbors[epos[e]];
    const double den = std::sqrt(std::max((double)deg[h] * (double)deg[t], 1e-24));
    const float w = (float)(weights[epos[e]] / den);
    snb[cur[h]] = t;
    sw[cur[h]++] = w;
    snb[cur[t]] = h;
    sw[cur[t]++] = w;
  }
  std::vector<double> triv(n);
  double tn = 0.0;
  for (int i = 0; i < n; ++i) {
    triv[i] = std::sqrt(std::max((double)deg[i], 0.0));
    tn += triv[i] * triv[i];
  }
  tn = std::sqrt(std::max(tn, 1e-12));
  for (double& v : triv) v /= tn;
  const int B = std::min(n - 1, std::max(comps + 6, 8));
  if (B < comps) {
    random_layout();
    return;
  }
  auto spmm = [&](const std::vector<double>& x, std::vector<double>& y) {
    std::vector<double> s(B);
    for (int r = 0; r < n; ++r) {
      std::fill(s.begin(), s.end(), 0.0);
      for (int p = so[r]; p < so[r + 1]; ++p) {
        const double w = sw[p];
        for (int c = 0; c < B; ++c) s[c] += w * x[(size_t)c * n + snb[p]];
      }
      for (int c = 0; c < B; ++c) y[(size_t)c * n + r] = s[c];
    }
  };
  auto orthonormalize = [&](std::vector<double>& q) {
    for (int c = 0; c < B; ++c) {
      double* qc = &q[(size_t)c * n];
      double d0 = 0.0;
      for (int i = 0; i < n; ++i) d0 += qc[i] * triv[i];
      for (int i = 0; i < n; ++i) qc[i] -= d0 * triv[i];
      for (int pv = 0; pv < c; ++pv) {
        const double* qp = &q[(size_t)pv * n];
        double d = 0.0;
        for (int i = 0; i < n; ++i) d += qc[i] * qp[i];
        for (int i = 0; i < n; ++i) qc[i] -= d * qp[i];
      }
      double nrm = 0.0;
      for (int i = 0; i < n; ++i) nrm += qc[i] * qc[i];
      nrm = std::sqrt(nrm);
      if (nrm < 1e-10) {
        for (int i = 0; i < n; ++i) qc[i] = normal(rng) * 10000.0;
        --c;
      } else {
        for (int i = 0; i < n; ++i) qc[i] /= nrm;
      }
    }
  };
  std::vector<double> q((size_t)n * B), z((size_t)n * B);
  for (double& v : q) v = normal(rng) * 10000.0;
  orthonormalize(q);
  for (int it = 0; it < n_iter; ++it) {
    spmm(q, z);
    orthonormalize(z);
    q.swap(z);
  }
  spmm(q, z);
  std::vector<double> P((size_t)B * B, 0.0);
  for (int r = 0; r < n; ++r)
    for (int a = 0; a < B; ++a) {
      const double qv = q[(size_t)a * n + r];
      for (int b = a; b < B; ++b) P[(size_t)a * B + b] += qv * z[(size_t)b * n + r];
    }
  for (int a = 0; a < B; ++a)
    for (int b = a; b < B; ++b) P[(size_t)b * B + a] = P[(size_t)a * B + b];
  // one Jacobi rotation of the largest off-diagonal entry per sweep, at most 80
  std::vector<double> V((size_t)B * B, 0.0);
  for (int i = 0; i < B; ++i) V[(size_t)i * B + i] = 1.0;
  for (int sweep = 0; sweep < 80; ++sweep) {
    int p = 0, qi = 1;
    double mx = 0.0;
    for (int i = 0; i < B; ++i)
      for (int j = i + 1; j < B; ++j) {
        const double v = std::abs(P[(size_t)i * B + j]);
        if (v > mx) {
          mx = v;
          p = i;
          qi = j;
        }
      }
    if (mx < 1e-10) break;
    const double app = P[(size_t)p * B + p], aqq = P[(size_t)qi * B + qi], apq = P[(size_t)p * B + qi];
    const double tau = (aqq - app) / (2.0 * apq);
    const double t = (tau >= 0.0 ? 1.0 : -1.0) / (std::abs(tau) + std::sqrt(1.0 + tau * tau));
    const double cs = 1.0 / std::sqrt(1.0 + t * t), sn = t * cs;
    for (int k = 0; k < B; ++k) {
      if (k == p || k == qi) continue;
      const double akp = P[(size_t)k * B + p], akq = P[(size_t)k * B + qi];
      P[(size_t)k * B + p] = cs * akp - sn * akq;
      P[(size_t)p * B + k] = P[(size_t)k * B + p];
      P[(size_t)k * B + qi] = sn * akp + cs * akq;
      P[(size_t)qi * B + k] = P[(size_t)k * B + qi];
    }
    P[(size_t)p * B + p] = cs * cs * app - 2.0 * sn * cs * apq + sn * sn * aqq;
    P[(size_t)qi * B + qi] = sn * sn * app + 2.0 * sn * cs * apq + cs * cs * aqq;
    P[(size_t)p * B + qi] = 0.0;
    P[(size_t)qi * B + p] = 0.0;
    for (int k = 0; k < B; ++k) {
      const double vp = V[(size_t)k * B + p], vq = V[(size_t)k * B + qi];
      V[(size_t)k * B + p] = cs * vp - sn * vq;
      V[(size_t)k * B + qi] = sn * vp + cs * vq;
    }
  }
  std::vector<int> order(B);
  std::iota(order.begin(), order.end(), 0);
  std::sort(order.begin(), order.end(),
            [&](int a, int b) { return P[(size_t)a * B + a] > P[(size_t)b * B + b]; });
  for (int c = 0; c < comps; ++c) {
    std::vector<double> v(n, 0.0);
    for (int i = 0; i < n; ++i) {
      double s = 0.0;
      for (int b = 0; b < B; ++b) s += q[(size_t)b * n + i] * V[(size_t)b * B + order[c]];
      v[i] = s;
    }
    const double mean = std::accumulate(v.begin(), v.end(), 0.0) / n;
    for (int i = 0; i < n; ++i) emb[(size_t)c * n + i] = v[i] - mean;
  }
  // scale_embedding_max_abs_and_jitter(embedding, 10, 1e-4), :2705-2730
  double mabs = 0.0;
  for (int c = 0; c < comps; ++c)
    for (int i = 0; i < n; ++i) {
      const double a = std::abs(emb[(size_t)c * n + i]);
      if (std::isfinite(a)) mabs = std::max(mabs, a);
    }
  if (!std::isfinite(mabs) || mabs <= 0.0) return;
  const double ex = 10.0 / mabs;
  std::normal_distribution<double> jitter(0.0, 1e-4);
  for (int c = 0; c < comps; ++c)
    for (int i = 0; i < n; ++i) emb[(size_t)c * n + i] = emb[(size_t)c * n + i] * ex + jitter(rng);
}

}  // namespace

extern "C" void orc_umap_spectral_init(const int* offsets, const int* neighbors, const float* weights, int n,
                                       int n_iter, double init_scale, int seed, double* out) {
  std::mt19937 rng((std::uint32_t)seed);
  spectral_layout(offsets, neighbors, weights, n, n_iter, rng, out);
  // scale_embedding_sdev, :2681-2703
  if (!(std::isfinite(init_scale) && init_scale > 0.0) || n < 2) return;
  for (int c = 0; c < 2; ++c) {
    double* e = out + (size_t)c * n;
    double mean = 0.0;
    for (int i = 0; i < n; ++i) mean += e[i];
    mean /= (double)n;
    double ss = 0.0;
    for (int i = 0; i < n; ++i) {
      const double d = e[i] - mean;
      ss += d * d;
    }
    const double sd = std::sqrt(ss / (double)(n - 1));
    if (!std::isfinite(sd) || sd <= 0.0) continue;
    const double sc = init_scale / sd;
    for (int i = 0; i < n; ++i) e[i] = (e[i] - mean) * sc;
  }
}
