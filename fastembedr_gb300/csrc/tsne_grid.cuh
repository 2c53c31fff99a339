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

// Device buffers of one t-SNE instance (all inside one arena).
struct TsneDevice {
  int n = 0;
  int grid = 0;     // G: nodes per side of the charge grid
  int fft = 0;      // M = 2G
  int log_fft = 0;
  int mode = kInterpLagrange3;
  int nodes = 0;
  float2* y = nullptr;      // layout read by the gradient (stored, not recentred)
  float2* ynew = nullptr;   // layout written by the update
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
  int step_blocks = 0;
  int col_blocks = 0;
  int cols_per_block = 0;
  Arena arena;
};

void tsne_device_alloc(TsneDevice& d, int n, int grid, int mode);
// Copy a row-major float2 init into ynew, zero gains/update state and compute `next`.
void tsne_device_init(TsneDevice& d, const float* d_init, cudaStream_t s);
// One optimizer iteration (scatter, FFT convolution, fused attractive + update).
void tsne_iteration(TsneDevice& d, const DeviceCsr& P, float exaggeration, float learning_rate, float momentum,
                    float min_gain, float max_step_norm, cudaStream_t s);
// The two halves of an iteration: scatter + FFT convolution (4 launches), fused step (1).
void tsne_grid_stage(TsneDevice& d, cudaStream_t s);
void tsne_step_stage(TsneDevice& d, const DeviceCsr& P, float exaggeration, float learning_rate, float momentum,
                     float min_gain, float max_step_norm, cudaStream_t s);
// out = ynew - mean(ynew), row-major float2.
void tsne_finalize(TsneDevice& d, float* d_out, cudaStream_t s);
// Forces on the current layout without updating it (diagnostics): attractive and repulsive
// parts separately, plus the grid Z.
void tsne_forces(TsneDevice& d, const DeviceCsr& P, float exaggeration, float* d_attr, float* d_rep,
                 cudaStream_t s);
// Kernel launch counts per iteration (for launch accounting).
int tsne_launches_per_iteration();

}  // namespace fe
