// PCA start of t-SNE on the GPU (the device PCA initialisation of the reference's
// opentsne_fft_from_device_knn_float_pca_* entry points).
#pragma once

#include "common.cuh"

namespace fe {

// Scores of the two leading principal components of X (device, column-major n x p floats,
// overwritten by the centred data), centred and scaled so the larger column standard deviation
// is 1e-4, written as the row-major float2 start layout `init` (device). p >= 2.
void pca_tsne_start(float* X, int n, int p, float2* init, cudaStream_t s);

}  // namespace fe
