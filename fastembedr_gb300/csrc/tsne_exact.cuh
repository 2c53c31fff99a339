// Exact all-pairs t-SNE quantities (diagnostics, KL, the FP64-normalised exact repulsion).
#pragma once

#include "tsne.cuh"

namespace fe {

// d_rep (2n doubles): -sum_j q_ij^2 (y_i - y_j), not yet divided by Z; d_zrow (n): sum_j q_ij;
// d_ztotal: sum over all ordered pairs i != j.
void exact_repulsion(const float* d_y, int n, double* d_rep, double* d_zrow, double* d_ztotal, cudaStream_t s);

// Exact repulsion at selected points: for r < n_rows, the point y[d_inv[d_rows[r]]] (original id
// d_rows[r]) against all n points. d_out (3 x n_rows doubles): -sum_j q^2 dx, -sum_j q^2 dy and
// sum_{j != i} q, unnormalised; d_ztotal: the all-pairs Z (d_zrow: n doubles of scratch). d_part
// holds exact_rows_slices(n, n_rows) x 3 x n_rows doubles.
int exact_rows_slices(int n, int n_rows);
void exact_repulsion_rows(const float* d_y, int n, const int* d_rows, const int* d_inv, int n_rows, double* d_part,
                          double* d_out, double* d_zrow, double* d_ztotal, cudaStream_t s);

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
