// Spectral start of UMAP on the GPU: the block subspace iteration of the reference's CPU
// initialisation (the start that umap_knn uses on every backend).
#pragma once

#include <future>
#include <random>
#include <vector>

#include "common.cuh"
#include "normal_stream.cuh"

namespace fe {

// The start's random draws for n points, made on the host in the reference's stream order: the
// start block (n x B normal(0, 1e-4) x 1e4 draws) and, speculatively and on another thread, the
// jitter that follows it when no Gram-Schmidt column needs a redraw (drawn from a copy of the
// stream state after the block). `rng` and `normal` hold the live state after the block, for
// redraws. Independent of the graph, so a caller can make them while the GPU builds it.
struct SpectralDraws {
  std::mt19937 rng;
  NormalStream normal{0.0, 0.0001};
  std::vector<double> block;
  std::shared_future<std::vector<double>> jitter;
};
SpectralDraws spectral_draws(int n, int seed);

// Start layout of the symmetric fuzzy graph (device CSR: n + 1 offsets, neighbours 0-based and
// ascending per row, no self entries, w_ij == w_ji) into out: device, column-major n x 2 doubles.
// spectral_n_iter rounds, seed for the std::mt19937 stream of the reference, init_scale > 0
// rescales every column to that standard deviation (NaN: no rescaling). Synchronises s.
// `pre` (may be null): the draws of spectral_draws(n, seed), made ahead.
void umap_spectral_start(const int* offsets, const int* neighbors, const float* weights, int n, long long nnz,
                         int spectral_n_iter, double init_scale, int seed, double* out, cudaStream_t s,
                         SpectralDraws* pre = nullptr);

}  // namespace fe
