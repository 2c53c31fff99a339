// Per-iteration state and kernels of the t-SNE gradient loop on the GPU.
#pragma once

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
};

struct StepPartial {
  float min_x, max_x, min_y, max_y;
  double sum_x, sum_y;
};

// Device buffers of one t-SNE instance (all inside one arena) and the side stream that runs
// the attractive pass concurrently with the grid stage.
struct TsneDevice {
  int n = 0;
  int grid = 0;     // G: nodes per side of the charge grid
  int fft = 0;      // M = 2G
  int log_fft = 0;
  int mode = kInterpLagrange3;
  int nodes = 0;
  float2* y = nullptr;        // layout in storage order (recentred lazily by the update)
  float2* attr = nullptr;     // attractive force of the current iteration
  float2* gains = nullptr;
  float2* update = nullptr;
  float4* charges = nullptr;  // G x G (mass, mass*dx, mass*dy, 0)
  float2* rows = nullptr;     // 2 planes x nodes x M: row-transformed charges
  float2* krows = nullptr;    // nodes x (G + 1): row-transformed kernel (q, q^2)
  float4* potential = nullptr;  // G x G (phi_q2, phi_x, phi_y, 0)
  float2* twiddle = nullptr;  // M / 2 forward twiddles
  double* zpart = nullptr;    // one per column block
  GridState* cur = nullptr;
  GridState* next = nullptr;
  StepPartial* partial = nullptr;
  unsigned* counter = nullptr;
  // spatial order: storage slot t holds original point perm[t]; inv is the inverse. CSR rows stay
  // in original order; CSR columns hold storage slots (relabelled at every reorder).
  int* perm = nullptr;
  int* inv = nullptr;
  unsigned* keys = nullptr;
  unsigned* keys_tmp = nullptr;
  int* order = nullptr;
  int* order_tmp = nullptr;
  int* delta = nullptr;
  float2* scratch = nullptr;  // 3 x n: y, gains, update while permuting
  int* perm_tmp = nullptr;
  RadixWorkspace radix;
  bool reordered = false;
  int attr_blocks = 0;
  int update_blocks = 0;
  int col_blocks = 0;
  int cols_per_block = 0;
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
// Copy a row-major float2 init into the layout, reset gains/update and compute `next`.
void tsne_device_init(TsneDevice& d, const float* d_init, cudaStream_t s);
// One optimizer iteration: grid stage on `s` concurrently with the attractive pass on the side
// stream, then the update (6 launches).
void tsne_iteration(TsneDevice& d, const DeviceCsr& P, float exaggeration, float learning_rate, float momentum,
                    float min_gain, float max_step_norm, cudaStream_t s);
// Stages, for profiling: scatter + FFT convolution (4 launches), attractive (1), update (1).
void tsne_grid_stage(TsneDevice& d, cudaStream_t s);
void tsne_attractive_stage(TsneDevice& d, const DeviceCsr& P, float exaggeration, cudaStream_t s);
void tsne_update_stage(TsneDevice& d, float learning_rate, float momentum, float min_gain, float max_step_norm,
                       cudaStream_t s);
// Sort points by the Morton code of their stencil anchor on the current grid and permute the
// point state (storage order) and the CSR column labels accordingly.
void tsne_reorder(TsneDevice& d, DeviceCsr& P, cudaStream_t s);
int tsne_reorder_launches();
// out[original id] = y - mean(y), row-major float2.
void tsne_finalize(TsneDevice& d, float* d_out, cudaStream_t s);
// Forces on the current layout without updating it (diagnostics).
void tsne_forces(TsneDevice& d, const DeviceCsr& P, float exaggeration, float* d_attr, float* d_rep,
                 cudaStream_t s);
int tsne_launches_per_iteration();

}  // namespace fe
