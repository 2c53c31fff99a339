// Fixed-reference t-SNE transform: device layout and launch interface shared by the one-shot
// C ABI (transform.cu) and the resident serving loop (transform_server.cu).
//
// One warp owns one query for all of its iterations: the lanes split the repulsion samples (or
// the exact reference sweep) and the k attractive neighbours, reduce with shuffles, and every
// lane carries the same optimizer state in registers. Queries never interact, so a launch may
// hold the queries of several requests (segments) and each result is independent of the mix.
#pragma once

#include <cstdint>

#include "common.cuh"

namespace fe {

// Options shared by every query of a launch (transform_tsne_cpp arguments).
struct TransformParams {
  int n_ref = 0;
  int exact = 0;          // 1: repulsion from every reference row; 0: n_negatives samples
  int n_negatives = 0;
  int iter_total = 0;     // early_exaggeration_iter + n_iter
  int early_iter = 0;
  int init_mode = 1;      // 0 supplied, 1 median, 2 weighted
  int seed = 0;
  int hash_sampler = 0;   // 1: samples by the landmark path's per-(iteration, query, sample) hash
  float lr = 0.1f, early_exag = 4.0f, exag = 1.5f, m0 = 0.8f, m1 = 0.8f;
  float max_grad = 0.25f, max_step = 3.4e38f;
  double perplexity = 5.0;
};

// The queries of one request inside a launch. Per-query arrays are row-major [query][k].
struct TransformSegment {
  const int* idx;          // column-major n_query x k (R layout), index_offset applied in-kernel
  const float* dist_f;     // column-major n_query x k float distances, or
  const double* dist_d;    // column-major n_query x k double distances
  const double* y_init;    // column-major n_query x 2, or null
  float2* nb;              // [query][k] neighbour reference coordinates
  float* p;                // [query][k] conditional probabilities
  float4* state;           // [query] (y_hi.x, y_hi.y, y_lo.x, y_lo.y)
  float4* opt;             // [query] (gain.x, gain.y, update.x, update.y)
  double* out;             // column-major n_query x 2 result
  long long query_begin;   // first warp of this segment within the launch
  int nq, k, offset;
};

// Lane l of a warp draws samples [l*n/32, (l+1)*n/32) of the reference's per-query xorshift32
// stream; its start state is T^(l*n/32) applied to the stream seed, T the xorshift32 step as a
// 32x32 matrix over GF(2). Columns of the 32 lane matrices, 32 words each.
struct XorshiftJump {
  std::uint32_t col[32][32];
};
XorshiftJump xorshift_jump_table(int n_negatives);

// Bytes of device memory one query of width k needs in a segment (excluding inputs).
std::size_t transform_query_bytes(int k);

// Prepare: per-query P (FP64 bisection of compute_row_probabilities_flat), neighbour
// coordinates and the initial layout. `segs` is a device array of `nseg` segments covering
// `total_q` queries.
void transform_prepare(const float2* ref, const double2* ref_d, const TransformSegment* segs, int nseg,
                       long long total_q, const TransformParams& tp, cudaStream_t s);
// Iterations [it_begin, it_end) for every query; writes `out` when it_end == iter_total.
void transform_iterate(const float2* ref, const TransformSegment* segs, int nseg, long long total_q,
                       const TransformParams& tp, const XorshiftJump* jump, int it_begin, int it_end,
                       cudaStream_t s);
// Largest reference the exact sweep keeps wholly in shared memory.
constexpr int kTransformSmemRefs = 12288;

}  // namespace fe
