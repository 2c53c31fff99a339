// Shared runtime pieces of the GB300 embedding library: error state, device arena,
// launch helpers and warp/block reductions. Everything here is host/device plumbing
// for the kernels in this directory; no torch types appear anywhere.
#pragma once

#include <cuda_runtime.h>

#include <algorithm>
#include <cstddef>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

namespace fe {

// ---------------------------------------------------------------- errors
// The C ABI reports failures the way the reference does
// (src/embedding_cuda_kernels.cpp:65-82): return 1 and keep a thread-local message.
void set_error(const std::string& msg);
void clear_error();
const char* last_error();

struct Error : std::runtime_error {
  explicit Error(const std::string& m) : std::runtime_error(m) {}
};

inline void cuda_check(cudaError_t code, const char* what) {
  if (code != cudaSuccess) throw Error(std::string(what) + ": " + cudaGetErrorString(code));
}
#define FE_CUDA(call) ::fe::cuda_check((call), #call)
#define FE_LAUNCH(what) ::fe::cuda_check(cudaGetLastError(), what)

// Run `body` and convert exceptions into the reference's 0/1 status convention.
template <typename F>
int guarded(F&& body) {
  clear_error();
  try {
    body();
    return 0;
  } catch (const std::exception& e) {
    set_error(e.what());
    cudaGetLastError();
    return 1;
  }
}

// ---------------------------------------------------------------- memory
inline std::size_t align256(std::size_t b) { return (b + 255u) & ~std::size_t(255u); }

// Free-memory preflight with the reference's 5% reserve (src/embedding_cuda_kernels.cpp:234-251).
void check_memory_available(std::size_t required, const char* where);

// One cudaMalloc per call, carved into 256-byte aligned pieces (the reference's
// CudaWorkspace arena, src/embedding_cuda_kernels.cpp:88-127). Sizes are collected first so
// that the preflight sees the whole request.
class Arena {
 public:
  Arena() = default;
  Arena(const Arena&) = delete;
  Arena& operator=(const Arena&) = delete;
  ~Arena() { release(); }
  template <typename T>
  void reserve(T** slot, std::size_t count) {
    plan_.push_back({reinterpret_cast<void**>(slot), align256(count * sizeof(T))});
  }
  void commit(const char* where);
  void release();
  std::size_t bytes() const { return total_; }

 private:
  struct Item {
    void** slot;
    std::size_t bytes;
  };
  std::vector<Item> plan_;
  void* base_ = nullptr;
  std::size_t total_ = 0;
};

struct Stream {
  cudaStream_t s = nullptr;
  Stream() { FE_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking)); }
  ~Stream() {
    if (s) cudaStreamDestroy(s);
  }
  Stream(const Stream&) = delete;
  Stream& operator=(const Stream&) = delete;
};

inline int ceil_div(long long a, long long b) { return static_cast<int>((a + b - 1) / b); }

// Entry points that read caller-owned device buffers run on their own non-blocking stream,
// which does not wait for the legacy default stream. Order `s` after everything enqueued so far
// on the legacy stream (and, through it, on every blocking stream) so that the caller's last
// writes to those buffers are complete.
void order_after_legacy_stream(cudaStream_t s);
int sm_count();

// ---------------------------------------------------------------- host uploads
// Host -> device copy of caller memory (pageable or not), ordered on stream s. Copies of at
// least kStagedUploadMin bytes go through a process-wide pair of pinned staging buffers: host
// threads fill one buffer while the copy engine drains the other, so large inputs move at
// pinned-copy speed rather than through the driver's pageable path. The source may be reused
// when the call returns. Smaller copies, and copies from pinned memory, are plain
// cudaMemcpyAsync calls.
constexpr std::size_t kStagedUploadMin = std::size_t(1) << 20;
void upload(void* dst, const void* src, std::size_t bytes, cudaStream_t s);

// ---------------------------------------------------------------- device helpers
__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ float warp_min(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fminf(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}
__device__ __forceinline__ float warp_max(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}
__device__ __forceinline__ double warp_min(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmin(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}
__device__ __forceinline__ double warp_max(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

}  // namespace fe
