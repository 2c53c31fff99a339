// Internal interfaces between the t-SNE translation units (affinities, grid
// repulsion, fused update, C ABI). Device pointers only; the stream is explicit.
#pragma once

#include <vector>

#include "common.cuh"

namespace fe {

// Symmetrised sparse P on the device: CSR with ascending columns per row, the same
// integers and float values as build_tsne_probabilities_float
// (fastEmbedR src/tsne_neighbors.cpp:616-724).
struct DeviceCsr {
  int n = 0;
  long long nnz = 0;
  int* row_ptr = nullptr;  // n + 1
  int* col = nullptr;      // nnz
  float* val = nullptr;    // nnz
  double total_mass = 0.0;
  Arena arena;
};

// Validate KNN input (column-major n x k); throws with the reference CPU messages.
void validate_knn(const int* d_idx, const float* d_dist, int n, int k, int offset, cudaStream_t s);
// Stream-ordered form: ORs the failure bits into *d_flags (bit 0 index range, bit 1 distance)
// without waiting; knn_flags_check throws the matching error for flags read back later.
void validate_knn_async(const int* d_idx, const float* d_dist, int n, int k, int offset, unsigned* d_flags,
                        cudaStream_t s);
void knn_flags_check(unsigned flags);

// Per-row perplexity bisection (FP32 exp, FP64 sums); writes directed P row-major n x k and,
// when non-null, the entropy reached by each row.
void row_probabilities(const int* d_idx, const float* d_dist, int n, int k, float perplexity,
                       float* d_p, double* d_entropy, cudaStream_t s);

// Emit both directions of every non-self directed edge, bucket by row, sort each row by
// column, sum duplicates in double and fill the CSR (allocated inside `out`).
void symmetrise(const int* d_idx, const float* d_p, int n, int k, int offset, DeviceCsr& out,
                cudaStream_t s);
// The same for a batch: instance b owns rows [first[b], first[b + 1]) (first = {0, ..., n}); columns
// of d_idx (minus offset) are global rows and stay inside their instance. Each instance's values
// are normalised by its own total, summed in the order symmetrise uses for one instance, so an
// instance's P equals the P it gets alone. totals (may be null) receives the instance totals.
void symmetrise_batch(const int* d_idx, const float* d_p, int n, int k, int offset, const std::vector<int>& first,
                      DeviceCsr& out, std::vector<double>* totals, cudaStream_t s);

// Device-wide exclusive scan of n int32 counts into n + 1 int64 offsets (out[n] = total);
// tmp holds ceil(n / 1024) int64 values.
void exclusive_scan(const int* in, long long* out, int n, long long* tmp, cudaStream_t s);

// Stable LSD radix sort of (key, value) pairs on the low `bits` key bits. Buffers of n items
// each plus the histogram workspace sized by radix_sort_workspace().
struct RadixWorkspace {
  int* hist = nullptr;          // 256 x blocks
  long long* offs = nullptr;    // 256 x blocks + 1
  long long* scan_tmp = nullptr;
};
int radix_sort_blocks(int n);
void radix_sort_pairs(unsigned* keys, int* vals, unsigned* keys_tmp, int* vals_tmp, int n, int bits,
                      const RadixWorkspace& ws, cudaStream_t s);

// Grid policy of the reference CUDA path (src/embedding_cuda_kernels.cpp:5610-5623), including
// the FASTEMBEDR_TSNE_FFT_GRID override.
int cuda_fft_grid_size(int n);
int cpu_fft_grid_size(int n);

// Interpolation scheme of the grid repulsion.
enum InterpMode { kInterpBilinear = 0, kInterpLagrange3 = 1 };
int interp_mode_from_env();

}  // namespace fe
