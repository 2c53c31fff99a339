// Exact all-pairs t-SNE quantities (diagnostics, KL, the FP64-normalised exact repulsion).
#pragma once

#include "tsne.cuh"

namespace fe {

// d_rep (2n doubles): -sum_j q_ij^2 (y_i - y_j), not yet divided by Z; d_zrow (n): sum_j q_ij;
// d_ztotal: sum over all ordered pairs i != j.
void exact_repulsion(const float* d_y, int n, double* d_rep, double* d_zrow, double* d_ztotal, cudaStream_t s);

// d_scalars[0] = all-pairs Z, d_scalars[1] = KL. d_zrow, d_work: n doubles each. Row i of P is
// the point y[d_inv[i]] (d_inv null: y[i]); P's columns index d_y.
void exact_kl(const DeviceCsr& P, const float* d_y, const int* d_inv, double* d_zrow, double* d_work,
              double* d_scalars, cudaStream_t s);
// The same for the rows [0, n) of a CSR slice whose points occupy d_y[y_begin, y_begin + n)
// (one instance of a batch; row_ptr holds absolute offsets, columns absolute slots; row i is
// the point y[d_inv[i]], or y[y_begin + i] when d_inv is null).
void exact_kl_range(const int* row_ptr, const int* col, const float* val, int n, const float* d_y, const int* d_inv,
                    int y_begin, double* d_zrow, double* d_work, double* d_scalars, cudaStream_t s);

}  // namespace fe
