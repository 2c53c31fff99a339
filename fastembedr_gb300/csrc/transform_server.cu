// Resident serving loop for the fixed-reference t-SNE transform (transform_tsne /
// project_landmark_model in serving form). No counterpart in the reference, which re-uploads
// the reference layout and re-derives everything per call
// (src/embedding_cuda_kernels.cpp:3572-3686).
//
// The server keeps the reference layout (FP32 for the pair terms, FP64 for the median/weighted
// start) and the sampling jump table resident on the device. Requests (KNN of a query batch
// into the reference) are copied at submit and queued. A worker thread admits queued requests,
// in arrival order, while their device memory fits a fixed budget and a stream slot is free;
// each admitted group of requests runs as ONE prepare launch pair and ONE iterate launch over
// all of the group's queries (segment table), on its own stream, so groups admitted while
// others run overlap on the device. Completion is signalled from the stream by a host function;
// the worker then releases the group's memory and admits more work.
//
// Every query's computation depends only on its own request (its row inside the request keys
// the sample stream), so a result is bit-identical alone, in any mix, and to the one-shot
// fastembedr_cuda_transform_tsne on the same inputs.
#include <atomic>
#include <chrono>
#include <climits>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "../../include/fastembedr_cuda.h"
#include "transform.cuh"

namespace fe {

TransformParams transform_params(int n_ref, int n_negatives, int exact_repulsion_threshold, double perplexity,
                                 int n_iter, int early_iter, double learning_rate, double early_exaggeration,
                                 double exaggeration, double initial_momentum, double final_momentum,
                                 double max_grad_norm, double max_step_norm, int init_mode, int seed);
void transform_random_init(int seed, int query_begin, int n_query, double* out);
int transform_chunk(long long n_query, const TransformParams& tp, int k);
void transform_upload_reference(const double* d_ref_cm, int n_ref, float2* ref, double2* ref_d, cudaStream_t s);

namespace {

// First-fit allocator over [0, capacity) in 256-byte units; adjacent free blocks coalesce.
class RangeAllocator {
 public:
  explicit RangeAllocator(std::size_t capacity = 0) { reset(capacity); }
  void reset(std::size_t capacity) {
    cap_ = capacity & ~std::size_t(255);
    free_.clear();
    if (cap_) free_[0] = cap_;
    used_ = peak_ = 0;
  }
  bool alloc(std::size_t bytes, std::size_t* off) {
    bytes = align256(std::max<std::size_t>(bytes, 1));
    for (auto it = free_.begin(); it != free_.end(); ++it) {
      if (it->second < bytes) continue;
      *off = it->first;
      const std::size_t rest = it->second - bytes, at = it->first + bytes;
      free_.erase(it);
      if (rest) free_[at] = rest;
      used_ += bytes;
      peak_ = std::max(peak_, used_);
      return true;
    }
    return false;
  }
  void release(std::size_t off, std::size_t bytes) {
    bytes = align256(std::max<std::size_t>(bytes, 1));
    used_ -= bytes;
    auto it = free_.emplace(off, bytes).first;
    auto next = std::next(it);
    if (next != free_.end() && it->first + it->second == next->first) {
      it->second += next->second;
      free_.erase(next);
    }
    if (it != free_.begin()) {
      auto prev = std::prev(it);
      if (prev->first + prev->second == it->first) {
        prev->second += it->second;
        free_.erase(it);
      }
    }
  }
  std::size_t capacity() const { return cap_; }
  std::size_t peak() const { return peak_; }

 private:
  std::map<std::size_t, std::size_t> free_;
  std::size_t cap_ = 0, used_ = 0, peak_ = 0;
};

using Clock = std::chrono::steady_clock;

struct Request {
  unsigned long long id = 0;
  int nq = 0, k = 0, offset = 0;
  std::vector<int> idx;        // column-major n_query x k
  std::vector<float> dist;     // column-major n_query x k
  std::vector<double> init;    // column-major n_query x 2 (random start), or empty
  std::vector<double> result;  // column-major n_query x 2
  Clock::time_point submitted, finished;
  std::size_t dev_off = 0, dev_bytes = 0, host_off = 0, host_bytes = 0;
  int state = 0;  // 0 queued, 1 running, 2 done, 3 failed
  std::string error;
};

struct Slot {
  cudaStream_t stream = nullptr;
  TransformSegment* d_segs = nullptr;  // device segment table
  TransformSegment* h_segs = nullptr;  // pinned staging of the table
  std::vector<Request*> reqs;
  std::atomic<bool> done{false};
  bool busy = false;
  void* server = nullptr;
  cudaEvent_t ev_begin = nullptr, ev_iterate = nullptr, ev_end = nullptr;  // device time of the group
  long long group_queries = 0;
};

constexpr int kMaxSegments = 4096;
constexpr long long kMaxGroupQueries = 1 << 17;

}  // namespace

class TransformServer {
 public:
  TransformParams tp;
  int init_mode = 1;  // 1 median, 2 weighted, 3 random
  int n_ref = 0;
  float2* ref = nullptr;
  double2* ref_d = nullptr;
  XorshiftJump* jump = nullptr;
  char* dev_pool = nullptr;
  char* host_pool = nullptr;
  RangeAllocator dev_alloc, host_alloc;
  std::vector<std::unique_ptr<Slot>> slots;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<Request*> queue;
  std::unordered_map<unsigned long long, std::unique_ptr<Request>> requests;
  unsigned long long next_id = 1;
  bool stopping = false;
  bool head_waits = false;  // the queue head did not fit the budget; set until memory is released
  std::thread worker;
  int device = 0;
  // statistics
  unsigned long long completed = 0, queries_done = 0, groups = 0, launches = 0;
  double device_ms = 0.0, iterate_ms = 0.0, max_group_iterate_ms = 0.0;
  long long max_group_queries = 0;

  ~TransformServer() { shutdown(); }

  std::size_t request_device_bytes(int nq, int k, bool with_init) const {
    const std::size_t items = (std::size_t)nq * k;
    std::size_t b = align256(items * sizeof(int)) + align256(items * sizeof(float)) +
                    align256(items * sizeof(float2)) + align256(items * sizeof(float)) +
                    2 * align256((std::size_t)nq * sizeof(float4)) + align256((std::size_t)nq * 2 * sizeof(double));
    if (with_init) b += align256((std::size_t)nq * 2 * sizeof(double));
    return b;
  }
  std::size_t request_host_bytes(int nq, int k, bool with_init) const {
    const std::size_t items = (std::size_t)nq * k;
    std::size_t b = align256(items * sizeof(int)) + align256(items * sizeof(float)) +
                    align256((std::size_t)nq * 2 * sizeof(double));
    if (with_init) b += align256((std::size_t)nq * 2 * sizeof(double));
    return b;
  }

  static void CUDART_CB on_done(void* p) {
    Slot* slot = static_cast<Slot*>(p);
    TransformServer* self = static_cast<TransformServer*>(slot->server);
    {
      std::lock_guard<std::mutex> lk(self->mu);
      slot->done.store(true);
    }
    self->cv_work.notify_one();
  }

  // Launch one admitted group on `slot` (called by the worker without the lock held).
  void launch(Slot& slot) {
    cudaStream_t s = slot.stream;
    long long total = 0;
    int nseg = 0;
    for (Request* r : slot.reqs) {
      const std::size_t items = (std::size_t)r->nq * r->k;
      const bool with_init = !r->init.empty();
      char* h = host_pool + r->host_off;
      char* d = dev_pool + r->dev_off;
      // host staging layout: idx | dist | out | init ; device layout: idx | dist | nb | p | state | opt | out | init
      int* h_idx = reinterpret_cast<int*>(h);
      float* h_dist = reinterpret_cast<float*>(h + align256(items * sizeof(int)));
      char* h_tail = h + align256(items * sizeof(int)) + align256(items * sizeof(float));
      double* h_init = reinterpret_cast<double*>(h_tail + align256((std::size_t)r->nq * 2 * sizeof(double)));
      std::memcpy(h_idx, r->idx.data(), items * sizeof(int));
      std::memcpy(h_dist, r->dist.data(), items * sizeof(float));
      if (with_init) std::memcpy(h_init, r->init.data(), (std::size_t)r->nq * 2 * sizeof(double));
      TransformSegment sg{};
      std::size_t at = 0;
      auto carve = [&](std::size_t bytes) {
        char* p = d + at;
        at += align256(bytes);
        return p;
      };
      sg.idx = reinterpret_cast<int*>(carve(items * sizeof(int)));
      sg.dist_f = reinterpret_cast<float*>(carve(items * sizeof(float)));
      sg.dist_d = nullptr;
      sg.nb = reinterpret_cast<float2*>(carve(items * sizeof(float2)));
      sg.p = reinterpret_cast<float*>(carve(items * sizeof(float)));
      sg.state = reinterpret_cast<float4*>(carve((std::size_t)r->nq * sizeof(float4)));
      sg.opt = reinterpret_cast<float4*>(carve((std::size_t)r->nq * sizeof(float4)));
      sg.out = reinterpret_cast<double*>(carve((std::size_t)r->nq * 2 * sizeof(double)));
      sg.y_init = with_init ? reinterpret_cast<double*>(carve((std::size_t)r->nq * 2 * sizeof(double))) : nullptr;
      sg.query_begin = total;
      sg.nq = r->nq;
      sg.k = r->k;
      sg.offset = r->offset;
      FE_CUDA(cudaMemcpyAsync(const_cast<int*>(sg.idx), h_idx, items * sizeof(int), cudaMemcpyHostToDevice, s));
      FE_CUDA(cudaMemcpyAsync(const_cast<float*>(sg.dist_f), h_dist, items * sizeof(float), cudaMemcpyHostToDevice,
                              s));
      if (with_init)
        FE_CUDA(cudaMemcpyAsync(const_cast<double*>(sg.y_init), h_init, (std::size_t)r->nq * 2 * sizeof(double),
                                cudaMemcpyHostToDevice, s));
      slot.h_segs[nseg++] = sg;
      total += r->nq;
    }
    FE_CUDA(cudaMemcpyAsync(slot.d_segs, slot.h_segs, sizeof(TransformSegment) * nseg, cudaMemcpyHostToDevice, s));
    slot.group_queries = total;
    FE_CUDA(cudaEventRecord(slot.ev_begin, s));
    transform_prepare(ref, ref_d, slot.d_segs, nseg, total, tp, s);
    FE_CUDA(cudaEventRecord(slot.ev_iterate, s));
    int max_k = 1;
    for (Request* r : slot.reqs) max_k = std::max(max_k, r->k);
    const int chunk = transform_chunk(total, tp, max_k);
    int n_launch = 2;
    for (int it = 0; it < tp.iter_total; it += chunk, ++n_launch)
      transform_iterate(ref, slot.d_segs, nseg, total, tp, jump, it, std::min(tp.iter_total, it + chunk), s);
    FE_CUDA(cudaEventRecord(slot.ev_end, s));
    for (int g = 0; g < nseg; ++g) {
      Request* r = slot.reqs[g];
      const std::size_t items = (std::size_t)r->nq * r->k;
      double* h_out = reinterpret_cast<double*>(host_pool + r->host_off + align256(items * sizeof(int)) +
                                                align256(items * sizeof(float)));
      FE_CUDA(cudaMemcpyAsync(h_out, slot.h_segs[g].out, (std::size_t)r->nq * 2 * sizeof(double),
                              cudaMemcpyDeviceToHost, s));
    }
    FE_CUDA(cudaLaunchHostFunc(s, &TransformServer::on_done, &slot));
    launches += n_launch;
  }

  // Worker: retire finished groups, admit queued requests, launch. Runs until shutdown.
  void run() {
    cudaSetDevice(device);
    std::unique_lock<std::mutex> lk(mu);
    for (;;) {
      const bool woke = cv_work.wait_for(lk, std::chrono::milliseconds(50), [&] {
        if (stopping) return true;
        for (auto& sl : slots)
          if (sl->busy && sl->done.load()) return true;
        if (queue.empty() || head_waits) return false;
        for (auto& sl : slots)
          if (!sl->busy) return true;
        return false;
      });
      if (!woke) {
        // a failed launch never reaches its completion host function: look for stream errors
        for (auto& sl : slots) {
          if (!sl->busy || sl->done.load()) continue;
          const cudaError_t e = cudaStreamQuery(sl->stream);
          if (e != cudaSuccess && e != cudaErrorNotReady) sl->done.store(true);
        }
      }
      // retire
      bool retired = false;
      for (auto& slp : slots) {
        Slot& sl = *slp;
        if (!sl.busy || !sl.done.load()) continue;
        const cudaError_t e = cudaStreamQuery(sl.stream);
        float g_ms = 0.0f, i_ms = 0.0f;
        if ((e == cudaSuccess || e == cudaErrorNotReady) &&
            cudaEventElapsedTime(&g_ms, sl.ev_begin, sl.ev_end) == cudaSuccess &&
            cudaEventElapsedTime(&i_ms, sl.ev_iterate, sl.ev_end) == cudaSuccess) {
          device_ms += g_ms;
          iterate_ms += i_ms;
          if (sl.group_queries >= max_group_queries) {
            max_group_queries = sl.group_queries;
            max_group_iterate_ms = i_ms;
          }
        }
        cudaGetLastError();
        for (Request* r : sl.reqs) {
          const std::size_t items = (std::size_t)r->nq * r->k;
          const double* h_out = reinterpret_cast<const double*>(host_pool + r->host_off + align256(items * sizeof(int)) +
                                                                align256(items * sizeof(float)));
          if (e == cudaSuccess || e == cudaErrorNotReady) {
            r->result.assign(h_out, h_out + (std::size_t)r->nq * 2);
            r->state = 2;
            ++completed;
            queries_done += (unsigned long long)r->nq;
          } else {
            r->state = 3;
            r->error = std::string("CUDA t-SNE transform server: ") + cudaGetErrorString(e);
          }
          r->finished = Clock::now();
          std::vector<int>().swap(r->idx);
          std::vector<float>().swap(r->dist);
          dev_alloc.release(r->dev_off, r->dev_bytes);
          host_alloc.release(r->host_off, r->host_bytes);
        }
        sl.reqs.clear();
        sl.busy = false;
        sl.done.store(false);
        retired = true;
        head_waits = false;
      }
      if (retired) cv_done.notify_all();
      if (stopping) {
        bool any_busy = false;
        for (auto& sl : slots) any_busy |= sl->busy;
        if (!any_busy) break;
        cv_work.wait_for(lk, std::chrono::milliseconds(1));
        continue;
      }
      // admit into free slots, in arrival order
      for (auto& slp : slots) {
        Slot& sl = *slp;
        if (sl.busy || queue.empty()) continue;
        long long total = 0;
        while (!queue.empty() && (int)sl.reqs.size() < kMaxSegments) {
          Request* r = queue.front();
          if (!sl.reqs.empty() && total + r->nq > kMaxGroupQueries) break;
          const bool with_init = !r->init.empty();
          std::size_t doff = 0, hoff = 0;
          const std::size_t db = request_device_bytes(r->nq, r->k, with_init);
          const std::size_t hb = request_host_bytes(r->nq, r->k, with_init);
          if (!dev_alloc.alloc(db, &doff)) break;
          if (!host_alloc.alloc(hb, &hoff)) {
            dev_alloc.release(doff, db);
            break;
          }
          r->dev_off = doff;
          r->dev_bytes = db;
          r->host_off = hoff;
          r->host_bytes = hb;
          r->state = 1;
          queue.pop_front();
          sl.reqs.push_back(r);
          total += r->nq;
        }
        if (sl.reqs.empty()) {
          // the head of the queue waits for memory; with nothing in flight it never will fit
          bool any_busy = false;
          for (auto& other : slots) any_busy |= other->busy;
          if (any_busy) {
            head_waits = true;
          } else {
            Request* r = queue.front();
            queue.pop_front();
            r->state = 3;
            r->error = "CUDA t-SNE transform request does not fit the server's memory budget";
            r->finished = Clock::now();
            cv_done.notify_all();
          }
          break;
        }
        sl.busy = true;
        ++groups;
        lk.unlock();
        std::string err;
        try {
          launch(sl);
        } catch (const std::exception& ex) {
          err = ex.what();
        }
        if (!err.empty()) cudaStreamSynchronize(sl.stream);
        lk.lock();
        if (!err.empty()) {
          for (Request* r : sl.reqs) {
            r->state = 3;
            r->error = err;
            r->finished = Clock::now();
            dev_alloc.release(r->dev_off, r->dev_bytes);
            host_alloc.release(r->host_off, r->host_bytes);
          }
          sl.reqs.clear();
          sl.busy = false;
          sl.done.store(false);
          head_waits = false;
          cv_done.notify_all();
        }
      }
    }
    for (Request* r : queue) {
      r->state = 3;
      r->error = "CUDA t-SNE transform server was shut down";
    }
    queue.clear();
    cv_done.notify_all();
  }

  void shutdown() {
    {
      std::lock_guard<std::mutex> lk(mu);
      stopping = true;
    }
    cv_work.notify_all();
    if (worker.joinable()) worker.join();
    for (auto& sl : slots) {
      if (sl->stream) cudaStreamDestroy(sl->stream);
      if (sl->h_segs) cudaFreeHost(sl->h_segs);
      if (sl->d_segs) cudaFree(sl->d_segs);
      for (cudaEvent_t ev : {sl->ev_begin, sl->ev_iterate, sl->ev_end})
        if (ev) cudaEventDestroy(ev);
      sl->stream = nullptr;
      sl->h_segs = nullptr;
    }
    slots.clear();
    if (dev_pool) cudaFree(dev_pool);
    if (host_pool) cudaFreeHost(host_pool);
    if (ref) cudaFree(ref);
    dev_pool = host_pool = nullptr;
    ref = nullptr;
  }
};

}  // namespace fe

struct fastembedr_transform_server {
  fe::TransformServer impl;
};

namespace {
fe::TransformServer* impl(fastembedr_transform_server* s) {
  if (!s) throw fe::Error("null CUDA t-SNE transform server");
  return &s->impl;
}
}  // namespace

extern "C" int fastembedr_transform_server_create(const double* reference_layout, int n_reference, double perplexity,
                                                  int n_iter, int early_exaggeration_iter, double learning_rate,
                                                  double early_exaggeration, double exaggeration,
                                                  double initial_momentum, double final_momentum,
                                                  double max_grad_norm, double max_step_norm, int n_negatives,
                                                  int exact_repulsion_threshold, int seed, const char* initialization,
                                                  unsigned long long memory_budget_bytes, int max_inflight,
                                                  fastembedr_transform_server** out) {
  return fe::guarded([&] {
    if (!reference_layout || !out) throw fe::Error("null CUDA t-SNE transform server argument");
    *out = nullptr;
    const std::string ini = initialization ? initialization : "median";
    if (ini != "median" && ini != "weighted" && ini != "random")
      throw fe::Error("`initialization` must be 'median', 'weighted', or 'random'.");
    const int mode = ini == "median" ? 1 : (ini == "weighted" ? 2 : 3);
    std::unique_ptr<fastembedr_transform_server> h(new fastembedr_transform_server());
    fe::TransformServer& sv = h->impl;
    sv.tp = fe::transform_params(n_reference, n_negatives, exact_repulsion_threshold, perplexity, n_iter,
                                 early_exaggeration_iter, learning_rate, early_exaggeration, exaggeration,
                                 initial_momentum, final_momentum, max_grad_norm, max_step_norm,
                                 mode == 3 ? 0 : mode, seed);
    sv.init_mode = mode;
    sv.n_ref = n_reference;
    FE_CUDA(cudaGetDevice(&sv.device));
    std::size_t free_b = 0, total_b = 0;
    FE_CUDA(cudaMemGetInfo(&free_b, &total_b));
    // resident part: FP32 + FP64 reference, jump table, staging of the FP64 input
    const std::size_t ref_bytes = fe::align256((std::size_t)n_reference * sizeof(float2)) +
                                  fe::align256((std::size_t)n_reference * sizeof(double2)) +
                                  fe::align256(sizeof(fe::XorshiftJump));
    std::size_t budget = memory_budget_bytes ? (std::size_t)memory_budget_bytes : (std::size_t)40 << 30;
    const std::size_t reserve = free_b / 20u;
    if (ref_bytes + budget + 2 * (std::size_t)n_reference * sizeof(double) > free_b - reserve)
      budget = free_b > reserve + ref_bytes + ((std::size_t)64 << 20)
                   ? free_b - reserve - ref_bytes - 2 * (std::size_t)n_reference * sizeof(double) -
                         ((std::size_t)32 << 20)
                   : 0;
    if (budget < ((std::size_t)1 << 20)) throw fe::Error("CUDA t-SNE transform server: not enough free device memory");
    char* base = nullptr;
    FE_CUDA(cudaMalloc(&base, ref_bytes));
    sv.ref = reinterpret_cast<float2*>(base);
    sv.ref_d = reinterpret_cast<double2*>(base + fe::align256((std::size_t)n_reference * sizeof(float2)));
    sv.jump = reinterpret_cast<fe::XorshiftJump*>(base + fe::align256((std::size_t)n_reference * sizeof(float2)) +
                                                  fe::align256((std::size_t)n_reference * sizeof(double2)));
    {
      fe::Stream st;
      double* d_cm = nullptr;
      FE_CUDA(cudaMalloc(&d_cm, 2 * (std::size_t)n_reference * sizeof(double)));
      FE_CUDA(cudaMemcpyAsync(d_cm, reference_layout, 2 * (std::size_t)n_reference * sizeof(double),
                              cudaMemcpyHostToDevice, st.s));
      const fe::XorshiftJump jump = fe::xorshift_jump_table(sv.tp.n_negatives);
      FE_CUDA(cudaMemcpyAsync(sv.jump, &jump, sizeof(jump), cudaMemcpyHostToDevice, st.s));
      fe::transform_upload_reference(d_cm, n_reference, sv.ref, sv.ref_d, st.s);
      FE_CUDA(cudaStreamSynchronize(st.s));
      FE_CUDA(cudaFree(d_cm));
    }
    FE_CUDA(cudaMalloc(&sv.dev_pool, budget));
    sv.dev_alloc.reset(budget);
    const std::size_t host_bytes = std::min<std::size_t>(budget, (std::size_t)2 << 30);
    FE_CUDA(cudaHostAlloc(&sv.host_pool, host_bytes, cudaHostAllocDefault));
    sv.host_alloc.reset(host_bytes);
    const int n_slots = std::max(1, std::min(max_inflight > 0 ? max_inflight : 4, 16));
    for (int i = 0; i < n_slots; ++i) {
      std::unique_ptr<fe::Slot> sl(new fe::Slot());
      FE_CUDA(cudaStreamCreateWithFlags(&sl->stream, cudaStreamNonBlocking));
      FE_CUDA(cudaHostAlloc(&sl->h_segs, sizeof(fe::TransformSegment) * fe::kMaxSegments, cudaHostAllocDefault));
      FE_CUDA(cudaMalloc(&sl->d_segs, sizeof(fe::TransformSegment) * fe::kMaxSegments));
      FE_CUDA(cudaEventCreate(&sl->ev_begin));
      FE_CUDA(cudaEventCreate(&sl->ev_iterate));
      FE_CUDA(cudaEventCreate(&sl->ev_end));
      sl->server = &sv;
      sv.slots.push_back(std::move(sl));
    }
    sv.worker = std::thread([&sv] { sv.run(); });
    *out = h.release();
  });
}

extern "C" int fastembedr_transform_server_submit(fastembedr_transform_server* server, const int* indices,
                                                  const float* distances, int n_query, int k,
                                                  unsigned long long* request_id) {
  return fe::guarded([&] {
    fe::TransformServer* sv = impl(server);
    if (!indices || !distances || !request_id) throw fe::Error("null CUDA t-SNE transform request pointer");
    if (n_query < 1 || k < 1) throw fe::Error("`knn` must have at least one row and one neighbor column.");
    std::unique_ptr<fe::Request> r(new fe::Request());
    const std::size_t items = (std::size_t)n_query * k;
    r->nq = n_query;
    r->k = k;
    r->idx.assign(indices, indices + items);
    r->dist.assign(distances, distances + items);
    int lo = INT_MAX, hi = INT_MIN;
    for (int v : r->idx) {
      lo = std::min(lo, v);
      hi = std::max(hi, v);
    }
    r->offset = (lo >= 1 && hi <= sv->n_ref) ? 1 : 0;
    for (std::size_t t = 0; t < items; ++t) {
      const int ref = r->idx[t] - r->offset;
      if (ref < 0 || ref >= sv->n_ref) throw fe::Error("KNN indices are out of range for `reference_layout`.");
      if (!std::isfinite(r->dist[t]) || r->dist[t] < 0.0f)
        throw fe::Error("KNN distances must be finite and non-negative.");
    }
    if (sv->init_mode == 3) {
      r->init.resize(2 * (std::size_t)n_query);
      fe::transform_random_init(sv->tp.seed, 0, n_query, r->init.data());
    }
    const bool with_init = !r->init.empty();
    if (sv->request_device_bytes(n_query, k, with_init) > sv->dev_alloc.capacity() ||
        sv->request_host_bytes(n_query, k, with_init) > sv->host_alloc.capacity())
      throw fe::Error("CUDA t-SNE transform request is larger than the server's memory budget");
    r->submitted = fe::Clock::now();
    {
      std::lock_guard<std::mutex> lk(sv->mu);
      if (sv->stopping) throw fe::Error("CUDA t-SNE transform server was shut down");
      r->id = sv->next_id++;
      *request_id = r->id;
      sv->queue.push_back(r.get());
      sv->requests.emplace(r->id, std::move(r));
    }
    sv->cv_work.notify_one();
  });
}

extern "C" int fastembedr_transform_server_wait(fastembedr_transform_server* server, unsigned long long request_id,
                                                int timeout_ms, double* out, double* latency_ms) {
  int status = 0;
  const int rc = fe::guarded([&] {
    fe::TransformServer* sv = impl(server);
    std::unique_lock<std::mutex> lk(sv->mu);
    auto it = sv->requests.find(request_id);
    if (it == sv->requests.end()) throw fe::Error("unknown CUDA t-SNE transform request id");
    fe::Request* r = it->second.get();
    auto ready = [&] { return r->state >= 2; };
    if (timeout_ms < 0) sv->cv_done.wait(lk, ready);
    else sv->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), ready);
    if (!ready()) {
      status = 2;
      return;
    }
    if (r->state == 3) {
      const std::string e = r->error;
      sv->requests.erase(it);
      throw fe::Error(e);
    }
    if (latency_ms)
      *latency_ms = std::chrono::duration<double, std::milli>(r->finished - r->submitted).count();
    if (out) {
      std::memcpy(out, r->result.data(), r->result.size() * sizeof(double));
      sv->requests.erase(it);
    }
  });
  return rc ? rc : status;
}

extern "C" int fastembedr_transform_server_stats(fastembedr_transform_server* server, unsigned long long* completed,
                                                 unsigned long long* queries, unsigned long long* groups,
                                                 unsigned long long* launches, unsigned long long* peak_bytes,
                                                 unsigned long long* budget_bytes, double* device_ms,
                                                 double* iterate_ms, long long* largest_group_queries,
                                                 double* largest_group_iterate_ms) {
  return fe::guarded([&] {
    fe::TransformServer* sv = impl(server);
    std::lock_guard<std::mutex> lk(sv->mu);
    if (completed) *completed = sv->completed;
    if (queries) *queries = sv->queries_done;
    if (groups) *groups = sv->groups;
    if (launches) *launches = sv->launches;
    if (peak_bytes) *peak_bytes = sv->dev_alloc.peak();
    if (budget_bytes) *budget_bytes = sv->dev_alloc.capacity();
    if (device_ms) *device_ms = sv->device_ms;
    if (iterate_ms) *iterate_ms = sv->iterate_ms;
    if (largest_group_queries) *largest_group_queries = sv->max_group_queries;
    if (largest_group_iterate_ms) *largest_group_iterate_ms = sv->max_group_iterate_ms;
  });
}

extern "C" void fastembedr_transform_server_destroy(fastembedr_transform_server* server) { delete server; }
