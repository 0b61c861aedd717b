// nq_noalloc.cu -- exec_solutions for callers that cannot allocate device memory.
//
// Some callers of this library must not call cudaMalloc/cudaFree after they
// start: a serving process whose device memory is owned and pre-reserved by
// another allocator (a framework's caching allocator, a fixed per-tenant
// budget), or a latency-critical loop where an allocation's implicit device
// synchronisation would stall every other stream.  This entry point runs the
// same prepare and DFS kernels as nq_exec_solutions_device, but its scratch
// (control words, task roots, task info, per-depth schedules) lives in one
// file-scope __device__ array of fixed size, which every GPU that loads the
// library holds until the process exits.  Nothing here allocates.
//
// Limits: at most kMaxRecords records per call (N <= 17 at the default
// presets) and schedules of at most kMaxWords depths.  All calls share the
// one array, so calls that overlap on the GPU (different streams or host
// threads at the same time) race: the caller must serialise them.
#include <cuda_runtime.h>

#include <mutex>

#include "../../include/nqueens_gb300.h"
#include "nq_common.cuh"
#include "nq_internal.h"

namespace {

constexpr int64_t kMaxRecords = 131072;
constexpr int kMaxWords = 24;                        // schedule words per task (depths 0..23)
constexpr size_t kCtrlBytes = 256;                   // totals, queue cursor, error word
constexpr size_t kRootBytes = (size_t)kMaxRecords * sizeof(uint4);
constexpr size_t kInfoBytes = (size_t)kMaxRecords * sizeof(uint2);
constexpr size_t kSchedBytes = (size_t)kMaxRecords * kMaxWords * sizeof(uint32_t);
constexpr size_t kScratchBytes = kCtrlBytes + kRootBytes + kInfoBytes + kSchedBytes;   // 15.0 MiB + 256 B
constexpr int kMaxDevices = 64;

std::mutex g_setup_mu;
void* g_scratch[kMaxDevices] = {nullptr};

}  // namespace

// The scratch itself.  In host code this name is only a stand-in for the
// symbol, not a device address: the address each device uses comes from
// cudaGetSymbolAddress below.
static __device__ __align__(256) unsigned char nq_noalloc_scratch[kScratchBytes];

namespace {

// Set-up, once per device, with that device current.
int scratch_for_current_device(void** out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return NQ_ECUDA;
  std::lock_guard<std::mutex> lk(g_setup_mu);
  if (!g_scratch[dev]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, nq_noalloc_scratch);
    if (e != cudaSuccess || p == nullptr) return NQ_ECUDA;
    g_scratch[dev] = p;
  }
  *out = g_scratch[dev];
  return NQ_OK;
}

}  // namespace

extern "C" int nq_exec_solutions_noalloc(int N, const nq_record* d_records, int64_t m, int start_min,
                                         uint64_t* d_solutions, uint64_t* d_total, void* stream) {
  using namespace nq;
  if (N < 6 || N > kMaxN || m < 0 || !d_total || (m > 0 && !d_records)) return NQ_EINVAL;
  if (m > kMaxRecords) return NQ_EINVAL;                // beyond the fixed scratch: rejected, never truncated
  const int s = start_min < 0 ? 1 : start_min;
  const int maxt = N - 2 - s < 1 ? 1 : N - 2 - s;       // stack frames; schedule words maxt + 1
  if (maxt + 1 > kMaxWords) return NQ_EINVAL;
  void* base = nullptr;
  if (int st = scratch_for_current_device(&base)) return st;
  cudaStream_t st = (cudaStream_t)stream;
  unsigned char* c = (unsigned char*)base;
  unsigned long long* totals = (unsigned long long*)c;
  unsigned long long* cursor = (unsigned long long*)(c + 8);
  unsigned int* err = (unsigned int*)(c + 16);
  // the array keeps the previous call's contents: clear what must start at zero
  if (cudaMemsetAsync(c, 0, 24, st) != cudaSuccess) return NQ_ECUDA;
  if (m > 0) {
    TaskArrays ta;
    ta.root = (uint4*)(c + kCtrlBytes);
    ta.info = (uint2*)(c + kCtrlBytes + kRootBytes);
    ta.sched = (void*)(c + kCtrlBytes + kRootBytes + kInfoBytes);
    ta.sw = maxt + 1;
    ta.wide = false;
    if (launch_prepare(N, m, (const uint4*)d_records, ta, 0, 0, err, st) != cudaSuccess) return NQ_ECUDA;
    DfsLaunch L;
    L.tasks = ta; L.m = m; L.cursor = cursor; L.job_totals = totals;
    L.per_task = (unsigned long long*)d_solutions; L.err = err; L.maxt = maxt; L.block = 128; L.grid = 0;
    L.big = counts_need_u64(N, m);
    if (launch_dfs(L, st) != cudaSuccess) return NQ_ECUDA;
  }
  if (cudaMemcpyAsync(d_total, totals, 8, cudaMemcpyDeviceToDevice, st) != cudaSuccess) return NQ_ECUDA;
  uint32_t herr = 0;
  if (cudaMemcpyAsync(&herr, err, 4, cudaMemcpyDeviceToHost, st) != cudaSuccess) return NQ_ECUDA;
  if (cudaStreamSynchronize(st) != cudaSuccess) return NQ_ECUDA;
  if (herr & DERR_DEPTH) return NQ_ESTACK;
  if (herr & DERR_SHIFT) return NQ_EPRESET;
  if (herr) return NQ_EINVAL;
  return NQ_OK;
}
