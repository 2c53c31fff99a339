// Error state, arena and device queries shared by the kernels of this library.
#include "common.cuh"

#include <cstring>
#include <mutex>
#include <thread>

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

namespace {
// Two pinned staging buffers of kChunk bytes, allocated on the first large upload and kept for
// the life of the process; a mutex serialises uploads from different host threads.
constexpr std::size_t kChunk = std::size_t(32) << 20;
constexpr int kCopyThreads = 4;

struct Stager {
  std::mutex mu;
  char* buf[2] = {nullptr, nullptr};
  cudaEvent_t done[2] = {nullptr, nullptr};
  int next = 0;
  int device = -1;  // the device whose context holds the events
  void ensure(int dev) {
    device = dev;
    for (int b = 0; b < 2; ++b) {
      if (!buf[b]) FE_CUDA(cudaHostAlloc(reinterpret_cast<void**>(&buf[b]), kChunk, cudaHostAllocDefault));
      if (!done[b]) FE_CUDA(cudaEventCreateWithFlags(&done[b], cudaEventDisableTiming));
    }
  }
};

Stager& stager() {
  static Stager* st = new Stager();  // never destroyed: its pinned memory goes with the CUDA context
  return *st;
}

// memcpy of one staging chunk, split over a few host threads (one memory stream per thread
// reaches only a fraction of the host's bandwidth)
void parallel_copy(char* to, const char* from, std::size_t n) {
  const std::size_t part = (n + kCopyThreads - 1) / kCopyThreads;
  if (n < (std::size_t(4) << 20)) {
    std::memcpy(to, from, n);
    return;
  }
  std::thread th[kCopyThreads - 1];
  int started = 0;
  for (int t = 1; t < kCopyThreads; ++t) {
    const std::size_t off = (std::size_t)t * part;
    if (off >= n) break;
    const std::size_t len = std::min(part, n - off);
    th[started++] = std::thread([=] { std::memcpy(to + off, from + off, len); });
  }
  std::memcpy(to, from, std::min(part, n));
  for (int t = 0; t < started; ++t) th[t].join();
}
}  // namespace

void upload(void* dst, const void* src, std::size_t bytes, cudaStream_t s) {
  if (bytes == 0) return;
  cudaPointerAttributes attr{};
  const bool pinned = cudaPointerGetAttributes(&attr, src) == cudaSuccess && attr.type == cudaMemoryTypeHost;
  cudaGetLastError();
  if (bytes < kStagedUploadMin || pinned) {  // pinned sources are copied by DMA directly
    FE_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, s));
    return;
  }
  int dev = 0;
  FE_CUDA(cudaGetDevice(&dev));
  Stager& st = stager();
  std::lock_guard<std::mutex> lock(st.mu);
  if (st.device >= 0 && st.device != dev) {  // staging lives on the first device that used it
    FE_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, s));
    return;
  }
  st.ensure(dev);
  const char* from = static_cast<const char*>(src);
  char* to = static_cast<char*>(dst);
  for (std::size_t off = 0; off < bytes; off += kChunk) {
    const std::size_t n = std::min(kChunk, bytes - off);
    const int b = st.next;
    st.next ^= 1;
    FE_CUDA(cudaEventSynchronize(st.done[b]));  // the last copy out of this buffer has finished
    parallel_copy(st.buf[b], from + off, n);
    FE_CUDA(cudaMemcpyAsync(to + off, st.buf[b], n, cudaMemcpyHostToDevice, s));
    FE_CUDA(cudaEventRecord(st.done[b], s));
  }
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
