// nq_handle.h -- the handle behind the C ABI (include/nqueens_gb300.h) and the
// device buffers it owns; shared by the translation units that implement the
// ABI (nq_capi.cu, nq_unique.cu).  Not installed.
#pragma once
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/nqueens_gb300.h"

namespace nq {

// Device buffer.  With a stream set, allocation and release are stream-ordered
// (cudaMallocAsync / cudaFreeAsync on that stream), so building or freeing one
// batch never waits for kernels of other batches still running.
struct DevBuf {
  void* p = nullptr;
  size_t cap = 0;
  cudaStream_t ordered = nullptr;
  cudaError_t ensure(size_t n) {
    if (n <= cap) return cudaSuccess;
    release();
    size_t want = std::max<size_t>(n, 256);
    cudaError_t e = ordered ? cudaMallocAsync(&p, want, ordered) : cudaMalloc(&p, want);
    if (e == cudaSuccess) cap = want; else p = nullptr;
    return e;
  }
  void release() {
    if (p) { if (ordered) cudaFreeAsync(p, ordered); else cudaFree(p); }
    p = nullptr; cap = 0;
  }
};

// Control block of a batch run: totals (u64 per job), then the queue cursor
// (u64) and the error word (u32) at totals_bytes + 0 / + 8.
struct Ctrl {
  static size_t bytes(int njobs) { return (size_t)njobs * 8 + 16; }
};

// Control block of a single-N run (device, zeroed before each run):
//   job total (u64), queue cursor (u64), error word (u32), deepest schedule (u32),
//   split counters (u64 subtasks, u64 allocation cursor).
namespace ctl {
constexpr size_t kTotal = 0, kCursor = 8, kErr = 16, kTmax = 20, kSplit = 24, kBytes = 40;
}

}  // namespace nq

struct nq_handle {
  int device = 0;
  int sms = 0;
  cudaStream_t stream = nullptr;
  int block = 64, grid = 0, split = -1;    // split: -1 automatic, 0..3 fixed depth
  std::string err;
  nq::DevBuf rec, root, info, sched, per_task, ctrl, nsub, sroot, sinfo;
  nq::DevBuf utasks, uconfs, uctl;       // unique counter (nq_count_unique)
  nq::DevBuf okeys, oorder, ohist;       // queue order (nq_set_queue_order)
  int queue_order = 0;                   // 0: generator / split order, 1: largest estimated subtree first
  int64_t chunk_records = 0;             // records per chunk of nq_count (0: the library default)
  int64_t last_chunks = 0, last_records = 0;   // chunks and records of the last nq_count
  cudaEvent_t done = nullptr;            // recorded after the last asynchronous count (nq_sync waits on it)
  uint64_t* h_ctrl = nullptr;   // pinned read-back of the control block
  size_t h_ctrl_cap = 0;
  // pinned read-back blocks for batches, reused (freeing pinned memory can
  // synchronise the device, which would stall other batches in flight)
  std::mutex pin_mu;
  std::vector<std::pair<void*, size_t>> pin_free;
  void* pin_get(size_t bytes) {
    {
      std::lock_guard<std::mutex> lk(pin_mu);
      for (size_t i = 0; i < pin_free.size(); i++)
        if (pin_free[i].second >= bytes) {
          void* q = pin_free[i].first;
          pin_free.erase(pin_free.begin() + (long)i);
          pinned_sizes[q] = bytes;
          return q;
        }
    }
    const size_t want = std::max<size_t>(bytes, 65536);
    void* q = nullptr;
    if (cudaMallocHost(&q, want) != cudaSuccess) return nullptr;
    std::lock_guard<std::mutex> lk(pin_mu);
    pinned_cap[q] = want;
    pinned_sizes[q] = bytes;
    return q;
  }
  void pin_put(void* q) {
    if (!q) return;
    std::lock_guard<std::mutex> lk(pin_mu);
    pin_free.push_back({q, pinned_cap[q]});
  }
  std::map<void*, size_t> pinned_cap, pinned_sizes;
  bool pending = false;
  int last_split = 0;        // split depth and queue length of the last run
  int64_t last_queue = 0;
  // events around the last run's kernels (same stream as the launches)
  cudaEvent_t ev[3] = {nullptr, nullptr, nullptr};

  int fail(int status, const char* fmt, ...) {
    char buf[512];
    va_list ap; va_start(ap, fmt); vsnprintf(buf, sizeof buf, fmt, ap); va_end(ap);
    err = buf;
    return status;
  }
  int cuda_fail(cudaError_t e, const char* where) {
    return fail(e == cudaErrorMemoryAllocation ? NQ_ENOMEM : NQ_ECUDA, "%s: %s", where, cudaGetErrorString(e));
  }
  int ensure_pinned(size_t bytes) {
    if (bytes <= h_ctrl_cap) return NQ_OK;
    if (h_ctrl) cudaFreeHost(h_ctrl);
    h_ctrl = nullptr; h_ctrl_cap = 0;
    cudaError_t e = cudaMallocHost((void**)&h_ctrl, bytes);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMallocHost");
    h_ctrl_cap = bytes;
    return NQ_OK;
  }
};

#define NQ_CUDA(h, call)                                     \
  do {                                                       \
    cudaError_t _e = (call);                                 \
    if (_e != cudaSuccess) return (h)->cuda_fail(_e, #call); \
  } while (0)

#define NQ_CUDA(h, call)                                     \
  do {                                                       \
    cudaError_t _e = (call);                                 \
    if (_e != cudaSuccess) return (h)->cuda_fail(_e, #call); \
  } while (0)
