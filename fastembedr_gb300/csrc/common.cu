// Error state, arena and device queries shared by the kernels of this library.
#include "common.cuh"

namespace fe {

namespace {
thread_local std::string g_last_error;
}

void set_error(const std::string& msg) { g_last_error = msg; }
void clear_error() { g_last_error.clear(); }
const char* last_error() { return g_last_error.c_str(); }

void check_memory_available(std::size_t required, const char* where) {
  std::size_t free_b = 0, total_b = 0;
  if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) {
    cudaGetLastError();
    return;
  }
  const std::size_t reserve = free_b / 20u;
  if (required > free_b - reserve) {
    throw Error(std::string(where) + ": CUDA memory request exceeds available memory; required " +
                std::to_string(static_cast<unsigned long long>(required)) + " bytes, free " +
                std::to_string(static_cast<unsigned long long>(free_b)) + " bytes");
  }
}

void Arena::commit(const char* where) {
  total_ = 0;
  for (const Item& it : plan_) total_ += it.bytes;
  if (total_ == 0) return;
  check_memory_available(total_, where);
  cuda_check(cudaMalloc(&base_, total_), where);
  std::size_t off = 0;
  for (const Item& it : plan_) {
    *it.slot = it.bytes ? static_cast<unsigned char*>(base_) + off : nullptr;
    off += it.bytes;
  }
  plan_.clear();
}

void Arena::release() {
  if (base_) cudaFree(base_);
  base_ = nullptr;
  total_ = 0;
  plan_.clear();
}

int sm_count() {
  int dev = 0, sms = 0;
  FE_CUDA(cudaGetDevice(&dev));
  FE_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  return sms;
}

}  // namespace fe

void fe::order_after_legacy_stream(cudaStream_t s) {
  cudaEvent_t e = nullptr;
  FE_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  const cudaError_t r1 = cudaEventRecord(e, cudaStreamLegacy);
  const cudaError_t r2 = r1 == cudaSuccess ? cudaStreamWaitEvent(s, e, 0) : r1;
  cudaEventDestroy(e);
  FE_CUDA(r2);
}
