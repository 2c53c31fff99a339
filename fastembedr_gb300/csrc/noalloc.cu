// Exact t-SNE repulsion without any device allocation.
//
// Some callers cannot allocate device memory at the point where they need this result: for
// example an R session that shares the GPU with a framework whose memory pool has already
// reserved the free memory, or a serving loop that reserved its budget up front and does not
// allow cudaMalloc on the request path. For them this entry point takes caller-owned device
// buffers for the input layout and the outputs, and keeps its own working memory in a
// fixed-size array that is part of the library image on every GPU that loads the library
// (kNoAllocMaxPoints points, 1.5 MB, held until the process exits).
//
// The array is shared by every call: a call overwrites the whole region it uses before reading
// it, so nothing needs clearing between calls, but calls that overlap on the GPU (concurrent
// streams or threads) race on it and must be serialised by the caller.
//
// The first call on a device does the set-up for that device: with CUDA's lazy module loading
// (the default since CUDA 12.2) it is the call that loads this file's device code, and with it
// the 1.5 MB array, onto the GPU, and it looks up the array's device address
// (cudaGetSymbolAddress, with that device current), which later calls on the device reuse.
// Make that first call before a memory pool reserves the device's free memory, and before any
// stream capture. The address stays valid for the life of the device's primary context; after
// cudaDeviceReset the library must not be called again in that process.
#include <cstdint>
#include <mutex>

#include "../../include/fastembedr_cuda.h"
#include "tsne_exact.cuh"

namespace fe {
namespace {

constexpr int kNoAllocMaxPoints = 65536;
// per point: 2 doubles of unnormalised force and 1 double row sum of q; then the total
constexpr int kNoAllocScratchDoubles = 3 * kNoAllocMaxPoints + 32;

static __device__ __align__(256) double g_noalloc_scratch[kNoAllocScratchDoubles];

// Device address of the scratch array, resolved once per device with that device current.
// (Host code only sees a host-side stand-in under the array's name, so the address must come
// from cudaGetSymbolAddress.)
constexpr int kMaxDevices = 64;
std::mutex g_scratch_mutex;
double* g_scratch_ptr[kMaxDevices] = {};

double* scratch_on_current_device() {
  int dev = 0;
  FE_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) throw Error("device ordinal out of range for the no-allocation scratch table");
  std::lock_guard<std::mutex> lock(g_scratch_mutex);
  if (g_scratch_ptr[dev] == nullptr) {
    void* p = nullptr;
    const cudaError_t code = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (code != cudaSuccess) {
      cudaGetLastError();
      throw Error(std::string("cudaGetSymbolAddress(no-allocation scratch): ") + cudaGetErrorString(code));
    }
    g_scratch_ptr[dev] = static_cast<double*>(p);
  }
  return g_scratch_ptr[dev];
}

__global__ void normalise_repulsion_kernel(const double* __restrict__ rep, const double* __restrict__ ztot, int n,
                                           float* __restrict__ out, double* __restrict__ sum_q) {
  const double z = *ztot;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < 2 * n; t += gridDim.x * blockDim.x)
    out[t] = (float)(rep[t] / z);
  if (blockIdx.x == 0 && threadIdx.x == 0 && sum_q) *sum_q = z;
}

}  // namespace
}  // namespace fe

extern "C" int fastembedr_cuda_tsne_exact_repulsion_noalloc(const float* layout, int n, float* repulsive,
                                                            double* sum_q, void* stream) {
  return fe::guarded([&] {
    if (!layout || !repulsive) throw fe::Error("null device pointer passed to the no-allocation t-SNE repulsion");
    // the layout is read as float2 pairs
    if ((reinterpret_cast<std::uintptr_t>(layout) & 7u) != 0u)
      throw fe::Error("the no-allocation t-SNE repulsion needs an 8-byte aligned layout pointer");
    if (n < 2) throw fe::Error("the no-allocation t-SNE repulsion needs at least two points");
    if (n > fe::kNoAllocMaxPoints)
      throw fe::Error("n = " + std::to_string(n) + " exceeds the no-allocation scratch capacity of " +
                      std::to_string(fe::kNoAllocMaxPoints) + " points");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    double* scratch = fe::scratch_on_current_device();
    double* rep = scratch;                         // 2n
    double* zrow = scratch + 2 * (std::size_t)n;   // n
    double* ztot = scratch + 3 * (std::size_t)n;   // 1
    fe::exact_repulsion(layout, n, rep, zrow, ztot, s);
    fe::normalise_repulsion_kernel<<<std::max(1, std::min(fe::ceil_div(2LL * n, 256), 1024)), 256, 0, s>>>(
        rep, ztot, n, repulsive, sum_q);
    FE_LAUNCH("normalise_repulsion_kernel");
    FE_CUDA(cudaStreamSynchronize(s));
  });
}
