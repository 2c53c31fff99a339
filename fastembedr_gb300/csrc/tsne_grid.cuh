// Per-iteration state and kernels of the t-SNE gradient loop on the GPU, for one instance or a
// batch of independent instances that share every launch.
#pragma once

#include <vector>

#include "tsne.cuh"

namespace fe {

// Grid placement and normalisation shared by the kernels of one iteration. `next` is
// produced by the update epilogue from the freshly written layout; the scatter of the next
// iteration promotes it to `cur`, the FFT stage adds z / inv_z to `cur`.
struct GridState {
  float x0, y0;        // lower-left corner of the node grid
  float h, inv_h;      // node spacing
  float box, inv_box;  // Lagrange box width (3 nodes per box)
  float cx, cy;        // grid centre; charges are stored relative to it
  double mean_x, mean_y;  // mean of the stored layout (applied lazily as the recentring)
  double z;            // sum_{i != j} q_ij from the grid
  float inv_z;
  int nodes;           // nodes used per side (G for bilinear, 3 * floor(G / 3) for Lagrange)
  // Charges are summed as 64-bit fixed-point integers (value x qscale, qscale a power of two
  // chosen from n and the grid's half-width so no partial sum can overflow): integer addition is
  // associative, so the grid, and with it every later step, is the same whatever order the
  // atomics land in.
  float qscale, inv_qscale;
  // A scatter block (at most kPointBlock points) sums its tile in 32-bit fixed point at scale
  // tscale = qscale / 2^tile_shift (also a power of two, chosen so the block's sums fit in 31
  // bits) and adds each tile node to the grid as (sum << tile_shift).
  float tscale;
  int tile_shift;
};

// Fixed-point charges of one grid node: mass, mass * dx, mass * dy and a pad slot, so a node is
// one 32-byte sector.
constexpr int kChargeStride = 4;

struct StepPartial {
  float min_x, max_x, min_y, max_y;
  double sum_x, sum_y;
};

// One instance of a batch (device table entry). Instances are stored in table order: their
// points occupy consecutive storage slots and their CSR rows consecutive rows.
struct TsneInstance {
  int pt_begin, n;          // storage slots [pt_begin, pt_begin + n)
  int grid, nodes;          // G and the nodes used per side
  int block_begin, blocks;  // point blocks of this instance (and its StepPartial slice)
  float lr_mult;            // learning rate of this instance = run learning rate x lr_mult
  long long* charges;       // G x G x kChargeStride fixed-point (mass, mass*dx, mass*dy, 0)
  float4* potential;        // G x G (phi_q2, phi_x, phi_y, 0)
};

// Instances with the same G, transformed by the same FFT launches (instance members[blockIdx.y]).
struct GridClass {
  int grid = 0, nodes = 0, fft = 0, log_fft = 0;
  int count = 0;
  int* members = nullptr;     // device: the class's instance indices
  int col_blocks = 0;          // M / 2 + 1 conjugate column pairs
  float2* arow = nullptr;      // count x (nodes x M): row spectra of A = x-charge + i y-charge
  float2* brow = nullptr;      // count x (nodes x (M/2 + 1)): half row spectra of the mass plane
  float2* krow = nullptr;      // count x (nodes x (M/2 + 1)): row spectra of the kernel (q + i q^2)
  double* zpart = nullptr;     // count x col_blocks
  float2* twiddle = nullptr;  // M / 2 forward twiddles
  long long* charges = nullptr;  // count x G x G x kChargeStride
  float4* potential = nullptr;
};

constexpr int kPointBlock = 256;  // points per block of the point kernels

// Device buffers of a batch of t-SNE instances (one arena) and the side stream that runs the
// attractive pass concurrently with the grid stage. A single instance is a batch of one.
struct TsneDevice {
  int n = 0;        // points over all instances
  int mode = kInterpBilinear;
  int grid = 0;     // G of instance 0 (single-instance callers)
  int nodes = 0;
  std::vector<TsneInstance> inst;  // host copy of the table
  std::vector<GridClass> classes;
  Arena grid_arena;           // class workspaces; rebuilt when grid sizes change
  TsneInstance* d_inst = nullptr;
  int2* blocks = nullptr;     // point block -> (instance, first storage slot)
  int nblocks = 0;
  float2* y = nullptr;        // layout in storage order (recentred lazily by the update)
  float2* attr = nullptr;     // attractive force of the current iteration
  float2* gains = nullptr;
  float2* update = nullptr;
  GridState* cur = nullptr;   // per instance
  GridState* next = nullptr;  // per instance
  StepPartial* partial = nullptr;  // per point block
  unsigned* counter = nullptr;     // per instance
  // spatial order: storage slot t holds original point perm[t]; inv is the inverse. CSR rows stay
  // in original order; CSR columns hold storage slots (relabelled at every reorder). Points never
  // leave their instance's slot range.
  int* perm = nullptr;
  int* inv = nullptr;
  int2* slot_rows = nullptr;     // CSR segment (begin, end) of the point in each storage slot
  unsigned* attr_ctr = nullptr;  // work counters of the attractive pass (zero between launches)
  int attr_chunk = 8;            // slots per work item of the attractive pass
  struct Tuning {
    int chunk, blocks;
    float ms;
  };
  std::vector<Tuning> tuning;    // timings of the run-time launch tuning (tsne_tune_attractive)
  bool tuned = false;
  unsigned* keys = nullptr;
  unsigned* keys_tmp = nullptr;
  int* order = nullptr;
  int* order_tmp = nullptr;
  int* delta = nullptr;
  float2* scratch = nullptr;  // 3 x n: y, gains, update while permuting
  int* perm_tmp = nullptr;
  RadixWorkspace radix;
  int key_bits = 0;           // Morton bits of the largest grid; instance bits sit above them
  int sort_bits = 0;
  bool reordered = false;
  int attr_blocks = 0;
  cudaStream_t side = nullptr;
  cudaEvent_t fork = nullptr, join = nullptr;
  Arena arena;
  TsneDevice() = default;
  TsneDevice(const TsneDevice&) = delete;
  TsneDevice& operator=(const TsneDevice&) = delete;
  ~TsneDevice();
};

// Nodes per side used for a given size (the reference CUDA policy for either stencil).
int default_grid_size(int n, int mode);

void tsne_device_alloc(TsneDevice& d, int n, int grid, int mode);
// Batch of instances: sizes[b] points on a grids[b] x grids[b] grid, learning rate multipliers
// lr_mult[b].
void tsne_batch_alloc(TsneDevice& d, const std::vector<int>& sizes, const std::vector<int>& grids,
                      const std::vector<float>& lr_mult, int mode);
// Change the instances' grid sizes: rebuild the grid classes and their workspaces, then
// recompute every instance's next grid from the current layout (stream-ordered on s).
void tsne_regrid(TsneDevice& d, const std::vector<int>& grids, cudaStream_t s);
// Current grid extent (2 x half-width of the bounding square) of every instance, from `next`
// (synchronises s).
std::vector<float> tsne_grid_extents(TsneDevice& d, cudaStream_t s);
// Copy a row-major float2 init into the layout, reset gains/update and compute `next`.
void tsne_device_init(TsneDevice& d, const float* d_init, cudaStream_t s);
// Point every storage slot at its CSR row (after init; the reorder keeps it current).
void tsne_bind_rows(TsneDevice& d, const DeviceCsr& P, cudaStream_t s);
// One optimizer iteration: grid stage on `s` concurrently with the attractive pass on the side
// stream, then the update (3 + 3 x grid classes launches).
void tsne_iteration(TsneDevice& d, const DeviceCsr& P, float exaggeration, float learning_rate, float momentum,
                    float min_gain, float max_step_norm, cudaStream_t s);
// Stages, for profiling: scatter + FFT convolution, attractive (1), update (1).
void tsne_grid_stage(TsneDevice& d, cudaStream_t s);
void tsne_attractive_stage(TsneDevice& d, const DeviceCsr& P, float exaggeration, cudaStream_t s);
// Time the attractive pass's launch candidates on the current layout and keep the fastest;
// true when the launch changed.
bool tsne_tune_attractive(TsneDevice& d, const DeviceCsr& P, float exaggeration, cudaStream_t s);
void tsne_update_stage(TsneDevice& d, float learning_rate, float momentum, float min_gain, float max_step_norm,
                       cudaStream_t s);
// Sort each instance's points by the Morton code of their stencil anchor on the current grid and
// permute the point state (storage order) and the CSR column labels accordingly.
void tsne_reorder(TsneDevice& d, DeviceCsr& P, cudaStream_t s);
int tsne_reorder_launches(const TsneDevice& d);
// out[original id] = y - mean(y of its instance), row-major float2.
void tsne_finalize(TsneDevice& d, float* d_out, cudaStream_t s);
// Forces on the current layout without updating it (diagnostics).
void tsne_forces(TsneDevice& d, const DeviceCsr& P, float exaggeration, float* d_attr, float* d_rep,
                 cudaStream_t s);
int tsne_launches_per_iteration(const TsneDevice& d);

}  // namespace fe
