// Spectral start of UMAP on the GPU: the block subspace iteration of the reference's CPU
// initialisation (the start that umap_knn uses on every backend).
#pragma once

#include "common.cuh"

namespace fe {

// Start layout of the symmetric fuzzy graph (device CSR: n + 1 offsets, neighbours 0-based and
// ascending per row, no self entries, w_ij == w_ji) into out: device, column-major n x 2 doubles.
// spectral_n_iter rounds, seed for the std::mt19937 stream of the reference, init_scale > 0
// rescales every column to that standard deviation (NaN: no rescaling). Synchronises s.
void umap_spectral_start(const int* offsets, const int* neighbors, const float* weights, int n, long long nnz,
                         int spectral_n_iter, double init_scale, int seed, double* out, cudaStream_t s);

}  // namespace fe
