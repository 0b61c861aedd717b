// nq_capi.cu -- the extern "C" boundary of libnqgpu.so (include/nqueens_gb300.h).
//
// Owns device memory, streams, error reporting and the launch sequence:
//   records (host or device) -> prepare_kernel -> dfs_kernel -> totals.
// The library has no CPU counting path: every count is computed by the
// kernels in nq_kernels.cu.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <map>
#include <mutex>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <thread>
#include <vector>

#include "../../include/nqueens_gb300.h"
#include "nq_common.cuh"
#include "nq_host.h"
#include "nq_handle.h"
#include "nq_internal.h"

using namespace nq;

namespace {

int preset_for(int N) {
  if (N >= 5 && N <= 17) return 5;
  if (N >= 18 && N <= 21) return 6;
  if (N >= 22 && N <= 24) return 7;
  if (N >= 25 && N <= 27) return 8;
  return 5;
}

int derr_to_status(uint32_t e) {
  if (e & DERR_DEPTH) return NQ_ESTACK;
  if (e & DERR_SHIFT) return NQ_EPRESET;
  if (e) return NQ_EINVAL;
  return NQ_OK;
}

const char* derr_text(uint32_t e) {
  if (e & DERR_DEPTH) return "a task's schedule is deeper than the launch's stack";
  if (e & DERR_SHIFT) return "a record needs a negative shift (preset too deep for N)";
  if (e & DERR_NOTERM) return "a task's schedule never reaches a base frame";
  if (e & DERR_BADN) return "task with N outside 6..27";
  if (e & DERR_FORMAT) return "a schedule op does not fit the compact schedule word";
  return "ok";
}

// Expand tasks until the queue holds at least 13 items per resident DFS lane
// (the DFS kernel keeps about 768 lanes per SM), at most 3 levels.  Each level
// multiplies the queue by about 7 (measured: 6.2x at N=16 to 8x at N=20).
// Task lists of a million or more are split at least once: their largest
// tasks set the tail (GB300, N=21: D=0 7466 ms, D=1 6983 ms, D=2 6914 ms).
// This rule picks the depth the autotuner found fastest on GB300 for
// N=16..21 (2, 2, 1, 1, 1-2, 1-2).
int choose_split(int64_t m, int sms) {
  const double target = 13.0 * 768.0 * (double)sms;
  int D = 0;
  double est = (double)m;
  while (D < 3 && est < target) { est *= 7.0; D++; }
  // ~7 subtasks per task must stay within the u32 subtask queue
  return (D == 0 && m >= 1000000 && m <= 400000000) ? 1 : D;
}

// Records per chunk of a whole-board count (nq_count): one chunk up to N=21
// (2.0 M records), four at N=22 (28.7 M), about 32 MB of host records each.
constexpr int64_t kChunkRecords = 8 << 20;

int maxt_for(int N, int start_min) {
  // Terminal-parent depth T <= N - 3 - start; one frame of margin.
  int s = start_min < 0 ? 1 : start_min;
  int m = N - 2 - s;
  return std::max(1, std::min(m, kMaxDepth - 1));
}

}  // namespace

namespace {


// records (device) -> counts on st; totals land in ctrl[0].  Launches
// prepare, then (when splitting) the split count pass, one read-back of the
// control block (subtask count and deepest schedule), the split write pass,
// and the DFS with a stack sized to the deepest subtask.
int run_records(nq_handle* h, int N, const uint4* d_rec, int64_t m, int start_min, unsigned long long* d_per_task,
                cudaStream_t st) {
  const int maxt = maxt_for(N, start_min);
  const int sw = maxt + 1;
  NQ_CUDA(h, cudaSetDevice(h->device));
  NQ_CUDA(h, h->root.ensure((size_t)m * sizeof(uint4)));
  NQ_CUDA(h, h->info.ensure((size_t)m * sizeof(uint2)));
  NQ_CUDA(h, h->sched.ensure((size_t)m * sw * sizeof(uint32_t)));
  NQ_CUDA(h, h->ctrl.ensure(ctl::kBytes));
  unsigned char* c = (unsigned char*)h->ctrl.p;
  NQ_CUDA(h, cudaMemsetAsync(c, 0, ctl::kBytes, st));
  TaskArrays ta;
  ta.root = (uint4*)h->root.p; ta.info = (uint2*)h->info.p; ta.sched = h->sched.p; ta.sw = sw; ta.wide = false;
  unsigned long long* totals = (unsigned long long*)(c + ctl::kTotal);
  unsigned long long* cursor = (unsigned long long*)(c + ctl::kCursor);
  unsigned int* err = (unsigned int*)(c + ctl::kErr);
  unsigned long long* sctr = (unsigned long long*)(c + ctl::kSplit);   // split: [0] subtasks, [1] allocation cursor
  unsigned int* tmax = (unsigned int*)(c + ctl::kTmax);                 // deepest schedule of the launch
  NQ_CUDA(h, cudaEventRecord(h->ev[0], st));
  NQ_CUDA(h, launch_prepare(N, m, d_rec, ta, 0, 0, err, st, tmax));
  const int D = h->split >= 0 ? h->split : choose_split(m, h->sms);
  DfsLaunch L;
  L.tasks = ta; L.m = m; L.order = nullptr; L.cursor = cursor; L.job_totals = totals;
  L.per_task = d_per_task; L.err = err; L.maxt = maxt; L.block = h->block; L.grid = h->grid;
  if (D > 0) {
    NQ_CUDA(h, h->nsub.ensure((size_t)m * sizeof(uint32_t)));
    NQ_CUDA(h, launch_split(0, D, 0, m, ta, (uint32_t*)h->nsub.p, nullptr, nullptr, sctr, nullptr, totals, 0, st));
  }
  // One read-back: the split size and the deepest schedule T.  Subtasks start
  // at depth D with an empty stack, so the DFS needs T - D frames and T - D + 1
  // schedule words per lane; the kernel still rejects any task deeper than that.
  if (int s = h->ensure_pinned(ctl::kBytes)) return s;
  NQ_CUDA(h, cudaMemcpyAsync(h->h_ctrl, c, ctl::kBytes, cudaMemcpyDeviceToHost, st));
  NQ_CUDA(h, cudaStreamSynchronize(st));
  const unsigned char* hc = (const unsigned char*)h->h_ctrl;
  const int t_deep = (int)*(const uint32_t*)(hc + ctl::kTmax);
  L.maxt = std::max(1, std::min(maxt, t_deep - D));
  if (D > 0) {
    const int64_t ns = (int64_t)*(const uint64_t*)(hc + ctl::kSplit);
    if (ns > (int64_t)0xFFFFFFFF) return h->fail(NQ_ENOMEM, "split: %lld subtasks", (long long)ns);
    NQ_CUDA(h, h->sroot.ensure((size_t)std::max<int64_t>(ns, 1) * sizeof(uint4)));
    NQ_CUDA(h, h->sinfo.ensure((size_t)std::max<int64_t>(ns, 1) * sizeof(uint2)));
    NQ_CUDA(h, launch_split(1, D, 0, m, ta, (uint32_t*)h->nsub.p, (uint4*)h->sroot.p, (uint2*)h->sinfo.p, sctr,
                            d_per_task, totals, 0, st));
    L.sroot = (const uint4*)h->sroot.p; L.sinfo = (const uint2*)h->sinfo.p; L.m = ns;
  }
  L.big = counts_need_u64(N, L.m);
  if (h->queue_order == 1) {
    NQ_CUDA(h, h->okeys.ensure((size_t)std::max<int64_t>(L.m, 1)));
    NQ_CUDA(h, h->oorder.ensure((size_t)std::max<int64_t>(L.m, 1) * sizeof(uint32_t)));
    NQ_CUDA(h, h->ohist.ensure(512 * sizeof(unsigned int)));
    NQ_CUDA(h, launch_order(L.m, L.sroot, L.sinfo, ta, (uint8_t*)h->okeys.p, (unsigned int*)h->ohist.p,
                            (uint32_t*)h->oorder.p, st));
    L.order = (const uint32_t*)h->oorder.p;
  }
  h->last_split = D; h->last_queue = L.m;
  NQ_CUDA(h, cudaEventRecord(h->ev[1], st));
  NQ_CUDA(h, launch_dfs(L, st));
  NQ_CUDA(h, cudaEventRecord(h->ev[2], st));
  return NQ_OK;
}

int read_ctrl(nq_handle* h, cudaStream_t st, uint64_t* total) {
  if (int s = h->ensure_pinned(ctl::kBytes)) return s;
  NQ_CUDA(h, cudaMemcpyAsync(h->h_ctrl, h->ctrl.p, ctl::kBytes, cudaMemcpyDeviceToHost, st));
  NQ_CUDA(h, cudaStreamSynchronize(st));
  const unsigned char* hc = (const unsigned char*)h->h_ctrl;
  const uint32_t e = *(const uint32_t*)(hc + ctl::kErr);
  if (e) return h->fail(derr_to_status(e), "device: %s", derr_text(e));
  if (total) *total = *(const uint64_t*)(hc + ctl::kTotal);
  return NQ_OK;
}

}  // namespace

// ---------------------------------------------------------------------------
extern "C" {

const char* nq_version(void) { return "nqueens-gb300 0.1 (sm_103a)"; }

const char* nq_strerror(int s) {
  switch (s) {
    case NQ_OK: return "ok";
    case NQ_EINVAL: return "invalid argument";
    case NQ_ESTACK: return "task deeper than the launch's stack";
    case NQ_ETIMEOUT: return "bounded wait ran out";
    case NQ_ECUDA: return "CUDA error";
    case NQ_ENOMEM: return "out of memory";
    case NQ_EPRESET: return "preset too deep for N";
    case NQ_EBUSY: return "still running";
    default: return "unknown status";
  }
}

int nq_create(nq_handle** out, int device) {
  if (!out) return NQ_EINVAL;
  *out = nullptr;
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || device < 0 || device >= n) return NQ_ECUDA;
  nq_handle* h = new (std::nothrow) nq_handle();
  if (!h) return NQ_ENOMEM;
  h->device = device;
  if (cudaSetDevice(device) != cudaSuccess || cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaDeviceGetAttribute(&h->sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess ||
      cudaEventCreate(&h->ev[0]) != cudaSuccess || cudaEventCreate(&h->ev[1]) != cudaSuccess ||
      cudaEventCreate(&h->ev[2]) != cudaSuccess ||
      cudaEventCreateWithFlags(&h->done, cudaEventDisableTiming) != cudaSuccess) {
    nq_destroy(h);
    return NQ_ECUDA;
  }
  *out = h;
  return NQ_OK;
}

void nq_destroy(nq_handle* h) {
  if (!h) return;
  cudaSetDevice(h->device);
  if (h->stream) cudaStreamSynchronize(h->stream);
  h->rec.release(); h->root.release(); h->info.release(); h->sched.release(); h->per_task.release(); h->ctrl.release();
  h->nsub.release(); h->sroot.release(); h->sinfo.release();
  h->okeys.release(); h->oorder.release(); h->ohist.release();
  h->utasks.release(); h->uconfs.release(); h->uctl.release();
  if (h->h_ctrl) cudaFreeHost(h->h_ctrl);
  for (auto& q : h->pinned_cap) cudaFreeHost(q.first);
  for (auto& e : h->ev) if (e) cudaEventDestroy(e);
  if (h->done) cudaEventDestroy(h->done);
  if (h->stream) cudaStreamDestroy(h->stream);
  delete h;
}

int nq_int32_peak(nq_handle* h, int kind, double* ops_per_s) {
  if (!h || !ops_per_s || kind < 0 || kind > 3) return NQ_EINVAL;
  NQ_CUDA(h, cudaSetDevice(h->device));
  NQ_CUDA(h, h->ctrl.ensure(Ctrl::bytes(1)));
  int per = 0;
  NQ_CUDA(h, cudaDeviceGetAttribute(&per, cudaDevAttrMaxThreadsPerMultiProcessor, h->device));
  const int grid = h->sms * std::max(1, per / 256);
  const int iters = 4096;
  cudaStream_t st = h->stream;
  NQ_CUDA(h, int_peak(kind, 64, grid, (uint32_t*)h->ctrl.p, st));   // warm-up
  double best = 0.0;
  for (int rep = 0; rep < 3; rep++) {
    NQ_CUDA(h, cudaEventRecord(h->ev[0], st));
    NQ_CUDA(h, int_peak(kind, iters, grid, (uint32_t*)h->ctrl.p, st));
    NQ_CUDA(h, cudaEventRecord(h->ev[1], st));
    NQ_CUDA(h, cudaEventSynchronize(h->ev[1]));
    float ms = 0.f;
    NQ_CUDA(h, cudaEventElapsedTime(&ms, h->ev[0], h->ev[1]));
    const double ops = (double)grid * 256.0 * (double)iters * 128.0;
    best = std::max(best, ops / (ms * 1e-3));
  }
  *ops_per_s = best;
  return NQ_OK;
}

int nq_last_run_info(const nq_handle* h, int* split_depth, int64_t* queued) {
  if (!h) return NQ_EINVAL;
  if (split_depth) *split_depth = h->last_split;
  if (queued) *queued = h->last_queue;
  return NQ_OK;
}

int nq_last_kernel_ms(nq_handle* h, float* prepare_ms, float* dfs_ms) {
  if (!h) return NQ_EINVAL;
  NQ_CUDA(h, cudaSetDevice(h->device));
  NQ_CUDA(h, cudaEventSynchronize(h->ev[2]));
  float a = 0.f, b = 0.f;
  NQ_CUDA(h, cudaEventElapsedTime(&a, h->ev[0], h->ev[1]));
  NQ_CUDA(h, cudaEventElapsedTime(&b, h->ev[1], h->ev[2]));
  if (prepare_ms) *prepare_ms = a;
  if (dfs_ms) *dfs_ms = b;
  return NQ_OK;
}

int nq_device_sms(const nq_handle* h, int* sms) {
  if (!h || !sms) return NQ_EINVAL;
  *sms = h->sms;
  return NQ_OK;
}

int nq_device_name(const nq_handle* h, char* buf, size_t cap) {
  if (!h || !buf || cap == 0) return NQ_EINVAL;
  cudaDeviceProp p;
  if (cudaGetDeviceProperties(&p, h->device) != cudaSuccess) return NQ_ECUDA;
  snprintf(buf, cap, "%s", p.name);
  return NQ_OK;
}

int nq_last_error(const nq_handle* h, char* buf, size_t cap) {
  if (!h || !buf || cap == 0) return NQ_EINVAL;
  snprintf(buf, cap, "%s", h->err.c_str());
  return NQ_OK;
}

int nq_set_config(nq_handle* h, int block, int grid, int split_depth) {
  if (!h) return NQ_EINVAL;
  if (block != 64 && block != 128 && block != 256) return h->fail(NQ_EINVAL, "block must be 64, 128 or 256");
  if (grid < 0 || split_depth < -1 || split_depth > 3) return h->fail(NQ_EINVAL, "bad grid or split depth");
  h->block = block; h->grid = grid; h->split = split_depth;
  return NQ_OK;
}

int nq_set_queue_order(nq_handle* h, int mode) {
  if (!h) return NQ_EINVAL;
  if (mode != 0 && mode != 1) return h->fail(NQ_EINVAL, "queue order must be 0 or 1");
  h->queue_order = mode;
  return NQ_OK;
}

int nq_get_queue_order(const nq_handle* h, int* mode) {
  if (!h || !mode) return NQ_EINVAL;
  *mode = h->queue_order;
  return NQ_OK;
}

int nq_get_config(const nq_handle* h, int* block, int* grid, int* split_depth) {
  if (!h) return NQ_EINVAL;
  if (block) *block = h->block;
  if (grid) *grid = h->grid;
  if (split_depth) *split_depth = h->split;
  return NQ_OK;
}

int nq_preset_for(int N) { return preset_for(N); }

int64_t nq_gen_constellations(int N, int preset, nq_record* out, int64_t cap) {
  std::vector<GenRecord> v;
  const int s = gen_constellations(N, preset, v, 0);
  if (s == -1) return NQ_EINVAL;
  if (s == -2) return NQ_EPRESET;
  const int64_t n = (int64_t)v.size();
  if (out && cap >= n)
    for (int64_t i = 0; i < n; i++)
      out[i] = nq_record{(uint32_t)v[i].ld, (uint32_t)v[i].rd, (uint32_t)v[i].col, v[i].startijkl};
  return n;
}

int64_t nq_gen_constellations_wide(int N, int preset, uint64_t* ld, uint64_t* rd, uint64_t* col, uint32_t* sijkl,
                                   int64_t cap) {
  std::vector<GenRecord> v;
  const int s = gen_constellations(N, preset, v, 0);
  if (s == -1) return NQ_EINVAL;
  if (s == -2) return NQ_EPRESET;
  const int64_t n = (int64_t)v.size();
  if (ld && rd && col && sijkl && cap >= n)
    for (int64_t i = 0; i < n; i++) { ld[i] = v[i].ld; rd[i] = v[i].rd; col[i] = v[i].col; sijkl[i] = v[i].startijkl; }
  return n;
}

int nq_exec_solutions(nq_handle* h, int N, const nq_record* records, int64_t m, uint64_t* solutions, uint64_t* total) {
  if (!h || !total || m < 0 || (m > 0 && !records)) return h ? h->fail(NQ_EINVAL, "null argument") : NQ_EINVAL;
  if (N < 6 || N > kMaxN) return h->fail(NQ_EINVAL, "exec_solutions: N=%d outside 6..27", N);
  if (m > (int64_t)0x7FFFFFFF) return h->fail(NQ_EINVAL, "too many records");
  *total = 0;
  if (m == 0) return NQ_OK;
  cudaStream_t st = h->stream;
  NQ_CUDA(h, cudaSetDevice(h->device));
  const int smin = (int)start_row_min(&records[0].startijkl, m, 4);
  NQ_CUDA(h, h->rec.ensure((size_t)m * sizeof(nq_record)));
  NQ_CUDA(h, cudaMemcpyAsync(h->rec.p, records, (size_t)m * sizeof(nq_record), cudaMemcpyHostToDevice, st));
  unsigned long long* pt = nullptr;
  if (solutions) {
    NQ_CUDA(h, h->per_task.ensure((size_t)m * 8));
    pt = (unsigned long long*)h->per_task.p;
  }
  if (int s = run_records(h, N, (const uint4*)h->rec.p, m, smin, pt, st)) return s;
  if (solutions) NQ_CUDA(h, cudaMemcpyAsync(solutions, pt, (size_t)m * 8, cudaMemcpyDeviceToHost, st));
  return read_ctrl(h, st, total);
}

int nq_exec_solutions_device(nq_handle* h, int N, const nq_record* d_records, int64_t m, int start_min,
                             uint64_t* d_solutions, uint64_t* d_total, void* stream) {
  if (!h || !d_total || m < 0 || (m > 0 && !d_records)) return h ? h->fail(NQ_EINVAL, "null argument") : NQ_EINVAL;
  if (N < 6 || N > kMaxN) return h->fail(NQ_EINVAL, "exec_solutions: N=%d outside 6..27", N);
  if (m > (int64_t)0x7FFFFFFF) return h->fail(NQ_EINVAL, "too many records");
  cudaStream_t st = stream ? (cudaStream_t)stream : h->stream;
  NQ_CUDA(h, cudaSetDevice(h->device));
  if (m == 0) {
    NQ_CUDA(h, cudaMemsetAsync(d_total, 0, 8, st));
    return NQ_OK;
  }
  if (int s = run_records(h, N, (const uint4*)d_records, m, start_min, (unsigned long long*)d_solutions, st)) return s;
  NQ_CUDA(h, cudaMemcpyAsync(d_total, h->ctrl.p, 8, cudaMemcpyDeviceToDevice, st));
  NQ_CUDA(h, cudaEventRecord(h->done, st));
  h->pending = true;
  return NQ_OK;
}

int nq_sync(nq_handle* h) {
  if (!h) return NQ_EINVAL;
  NQ_CUDA(h, cudaSetDevice(h->device));
  if (!h->pending) {                      // nothing asynchronous outstanding: the handle's own stream
    NQ_CUDA(h, cudaStreamSynchronize(h->stream));
    return NQ_OK;
  }
  // waits for this handle's last count only (its event), not for other handles, batches or streams
  NQ_CUDA(h, cudaEventSynchronize(h->done));
  h->pending = false;
  uint32_t e = 0;
  NQ_CUDA(h, cudaMemcpyAsync(&e, (unsigned char*)h->ctrl.p + ctl::kErr, 4, cudaMemcpyDeviceToHost, h->stream));
  NQ_CUDA(h, cudaStreamSynchronize(h->stream));
  if (e) return h->fail(derr_to_status(e), "device: %s", derr_text(e));
  return NQ_OK;
}

int nq_debug_task_schedule(int N, nq_record rec, uint32_t root[4], uint32_t* info, uint32_t* words, int cap) {
  if (N < 6 || N > kMaxN || !root || !info || (cap > 0 && !words) || cap < 0) return NQ_EINVAL;
  const TaskHead t = decode_record(N, rec.ld, rec.rd, rec.col, rec.startijkl);
  if (t.status != TS_OK) return NQ_EPRESET;
  Root rt;
  uint32_t rc = 0;
  Op ops[kMaxDepth];
  const int T = walk_schedule(N, t, &rt, &rc, ops, std::min(cap, kMaxDepth));
  if (T == -2) return NQ_ESTACK;
  root[0] = rt.ld; root[1] = rt.rd; root[2] = rt.col; root[3] = (T < 0) ? 0u : rt.avail;
  *info = info_pack(T < 0 ? INFO_NO_DFS : (uint32_t)T, (uint32_t)t.wexp, rc, (uint32_t)N, TS_OK);
  if (T < 0) return 0;
  for (int d = 0; d <= T; d++) {
    if (!compact_fits(ops[d], N)) return NQ_EINVAL;
    words[d] = pack_compact(ops[d]);
  }
  return T + 1;
}

int64_t nq_debug_completion_tasks(int N, int k, const int* rows, const int* cols, int min_tasks, uint32_t* roots,
                                  uint32_t* infos, uint32_t* words, int stride, int64_t cap, uint64_t* fixed_count) {
  if (k < 0 || k > 8 || (k > 0 && (!rows || !cols)) || stride < 1) return NQ_EINVAL;
  std::vector<HostTask> v;
  int mt = 0;
  const int s = build_completion_tasks(N, k, rows, cols, min_tasks, 0, v, &mt);
  if (s < 0) return NQ_EINVAL;
  if (fixed_count) *fixed_count = (s == 2) ? 1 : 0;
  const int64_t n = (int64_t)v.size();
  if (cap >= n && n > 0) {
    if (!roots || !infos || !words) return NQ_EINVAL;
    for (int64_t i = 0; i < n; i++) {
      if (v[i].T + 1 > stride) return NQ_ESTACK;
      for (int q = 0; q < 4; q++) roots[i * 4 + q] = v[i].root[q];
      infos[i] = v[i].info;
      for (int d = 0; d <= v[i].T; d++) {
        words[(i * stride + d) * 2] = v[i].sched[2 * d];
        words[(i * stride + d) * 2 + 1] = v[i].sched[2 * d + 1];
      }
    }
  }
  return n;
}

int nq_count_completions(nq_handle* h, int N, int k, const int* rows, const int* cols, uint64_t* count);

int nq_tune(nq_handle* h, int N, int repeats, int* best_block, int* best_split, float* best_ms) {
  if (!h || repeats < 1) return h ? h->fail(NQ_EINVAL, "tune: bad arguments") : NQ_EINVAL;
  if (N < 6 || N > kMaxN) return h->fail(NQ_EINVAL, "tune: N=%d outside 6..27", N);
  std::vector<GenRecord> v;
  const int g = gen_constellations(N, preset_for(N), v, 0);
  if (g != 0) return h->fail(g == -2 ? NQ_EPRESET : NQ_EINVAL, "tune: generator failed for N=%d", N);
  const int64_t m = (int64_t)v.size();
  if (m == 0) return h->fail(NQ_EINVAL, "tune: no tasks for N=%d", N);
  std::vector<nq_record> r((size_t)m);
  for (int64_t i = 0; i < m; i++) r[i] = nq_record{(uint32_t)v[i].ld, (uint32_t)v[i].rd, (uint32_t)v[i].col, v[i].startijkl};
  cudaStream_t st = h->stream;
  NQ_CUDA(h, cudaSetDevice(h->device));
  const int smin = (int)start_row_min(&r[0].startijkl, m, 4);
  NQ_CUDA(h, h->rec.ensure((size_t)m * sizeof(nq_record)));
  NQ_CUDA(h, cudaMemcpyAsync(h->rec.p, r.data(), (size_t)m * sizeof(nq_record), cudaMemcpyHostToDevice, st));
  const int old_block = h->block, old_split = h->split;
  float best = 1e30f;
  int bb = old_block, bs = old_split;
  uint64_t want = 0;
  bool have_total = false;
  for (int b : {64, 128, 256})
    for (int s = 0; s <= 3; s++) {
      h->block = b; h->split = s;
      for (int k = 0; k <= repeats; k++) {           // first run warms up, then `repeats` timed runs
        uint64_t total = 0;
        int st_run = run_records(h, N, (const uint4*)h->rec.p, m, smin, nullptr, st);
        if (st_run == NQ_OK) st_run = read_ctrl(h, st, &total);
        if (st_run != NQ_OK) { h->block = old_block; h->split = old_split; return st_run; }
        if (!have_total) { want = total; have_total = true; }
        if (total != want) {
          h->block = old_block; h->split = old_split;
          return h->fail(NQ_ECUDA, "tune: N=%d count changed between configurations", N);
        }
        if (k == 0) continue;
        float ms = 0.f;
        NQ_CUDA(h, cudaEventElapsedTime(&ms, h->ev[0], h->ev[2]));
        if (ms < best) { best = ms; bb = b; bs = s; }
      }
    }
  h->block = bb; h->split = bs;                       // the handle keeps the fastest configuration
  if (best_block) *best_block = bb;
  if (best_split) *best_split = bs;
  if (best_ms) *best_ms = best;
  return NQ_OK;
}

int nq_set_chunk_records(nq_handle* h, int64_t records) {
  if (!h) return NQ_EINVAL;
  if (records < 0) return h->fail(NQ_EINVAL, "chunk size must be >= 0");
  h->chunk_records = records;
  return NQ_OK;
}

}  // extern "C"

namespace {

// The records of start constellations [s_begin, s_end), generated and counted
// chunk by chunk so host memory stays bounded for the largest boards (the
// reference streams its task list to a .bin file for the same reason,
// gen_constellations_stream_to_bin, 356Py_savesp_narrow.py:2988-3084): each
// chunk of starts is expanded into records on the host threads while the
// previous chunk's DFS runs on the GPU.
int count_start_range(nq_handle* h, int N, int p, const std::vector<int>& starts, size_t s_begin, size_t s_end,
                      uint64_t* total) {
  const int64_t chunk = h->chunk_records > 0 ? h->chunk_records : kChunkRecords;
  size_t next = s_begin;
  double per_start = 0.0;                  // records per start constellation seen so far
  std::vector<GenRecord> g;
  // Blocks of starts are expanded and packed into 16-byte records at once, so the
  // 32-byte generator records of at most an eighth of a chunk are alive at a time.
  auto gen_chunk = [&](std::vector<nq_record>& out) -> int {
    out.clear();
    if (per_start > 0.0)   // expected size of this chunk, so the vector does not double past it
      out.reserve((size_t)std::min((double)(chunk + chunk / 8), per_start * (double)(s_end - next) + 1024.0));
    while (next < s_end && (int64_t)out.size() < chunk) {
      const double want = std::min((double)(chunk - (int64_t)out.size()), (double)chunk / 8.0);
      const size_t take = per_start > 0.0 ? (size_t)std::max(1.0, want / per_start) : (size_t)16;
      const size_t s1 = std::min(s_end, next + take);
      g.clear();
      const int e = expand_starts(N, p, starts, next, s1, g, 0);
      if (e == -1) return h->fail(NQ_EINVAL, "generator: bad arguments N=%d preset=%d", N, p);
      if (e == -2) return h->fail(NQ_EPRESET, "generator: preset %d too deep for N=%d", p, N);
      per_start = 0.5 * per_start + 0.5 * (double)g.size() / (double)(s1 - next);
      if (per_start <= 0.0) per_start = 0.25;
      next = s1;
      const size_t o = out.size();
      out.resize(o + g.size());
      for (size_t i = 0; i < g.size(); i++)
        out[o + i] = nq_record{(uint32_t)g[i].ld, (uint32_t)g[i].rd, (uint32_t)g[i].col, g[i].startijkl};
    }
    std::vector<GenRecord>().swap(g);
    return NQ_OK;
  };
  cudaStream_t st = h->stream;
  NQ_CUDA(h, cudaSetDevice(h->device));
  std::vector<nq_record> cur, nxt;
  if (int e = gen_chunk(cur)) return e;
  uint64_t acc = 0;
  int64_t chunks = 0, records = 0;
  while (!cur.empty()) {
    const int64_t m = (int64_t)cur.size();
    const int smin = (int)start_row_min(&cur[0].startijkl, m, 4);
    NQ_CUDA(h, h->rec.ensure((size_t)m * sizeof(nq_record)));
    NQ_CUDA(h, cudaMemcpyAsync(h->rec.p, cur.data(), (size_t)m * sizeof(nq_record), cudaMemcpyHostToDevice, st));
    if (int s = run_records(h, N, (const uint4*)h->rec.p, m, smin, nullptr, st)) return s;
    if (int e = gen_chunk(nxt)) { cudaStreamSynchronize(st); return e; }   // overlaps the DFS just launched
    uint64_t t = 0;
    if (int s = read_ctrl(h, st, &t)) return s;
    acc += t; chunks++; records += m;
    cur.swap(nxt);
  }
  h->last_chunks = chunks;
  h->last_records = records;
  *total = acc;
  return NQ_OK;
}

}  // namespace

extern "C" {

// Whole-board count: the start constellations are listed first (cheap), then
// counted as one range.
int nq_count(nq_handle* h, int N, int preset, uint64_t* total) {
  if (!h || !total) return NQ_EINVAL;
  if (N < 1 || N > kMaxN) return h->fail(NQ_EINVAL, "N=%d outside 1..27", N);
  if (N <= 5) return nq_count_completions(h, N, 0, nullptr, nullptr, total);
  const int p = preset > 0 ? preset : preset_for(N);
  if (p < 4) return h->fail(NQ_EPRESET, "generator: preset %d below 4", p);
  std::vector<int> starts;
  if (start_constellations(N, starts) != 0) return h->fail(NQ_EINVAL, "generator: bad arguments N=%d", N);
  return count_start_range(h, N, p, starts, 0, starts.size(), total);
}

int64_t nq_start_constellations(int N, int32_t* out, int64_t cap) {
  if (N < 6 || N > kMaxN) return NQ_EINVAL;
  std::vector<int> starts;
  if (start_constellations(N, starts) != 0) return NQ_EINVAL;
  const int64_t n = (int64_t)starts.size();
  if (out && cap >= n)
    for (int64_t i = 0; i < n; i++) out[i] = (int32_t)starts[i];
  return n;
}

int64_t nq_gen_constellations_starts(int N, int preset, int64_t first, int64_t count, nq_record* out, int64_t cap) {
  if (N < 6 || N > kMaxN) return NQ_EINVAL;
  const int p = preset > 0 ? preset : preset_for(N);
  if (p < 4) return NQ_EPRESET;
  std::vector<int> starts;
  if (start_constellations(N, starts) != 0) return NQ_EINVAL;
  const int64_t ns = (int64_t)starts.size();
  if (first < 0 || count < 0 || first > ns || count > ns - first) return NQ_EINVAL;
  std::vector<GenRecord> v;
  const int e = expand_starts(N, p, starts, (size_t)first, (size_t)(first + count), v, 0);
  if (e == -1) return NQ_EINVAL;
  if (e == -2) return NQ_EPRESET;
  const int64_t n = (int64_t)v.size();
  if (out && cap >= n)
    for (int64_t i = 0; i < n; i++)
      out[i] = nq_record{(uint32_t)v[i].ld, (uint32_t)v[i].rd, (uint32_t)v[i].col, v[i].startijkl};
  return n;
}

int nq_count_starts(nq_handle* h, int N, int preset, int64_t first, int64_t count, uint64_t* total) {
  if (!h || !total) return NQ_EINVAL;
  if (N < 6 || N > kMaxN) return h->fail(NQ_EINVAL, "count_starts: N=%d outside 6..27", N);
  const int p = preset > 0 ? preset : preset_for(N);
  if (p < 4) return h->fail(NQ_EPRESET, "generator: preset %d below 4", p);
  std::vector<int> starts;
  if (start_constellations(N, starts) != 0) return h->fail(NQ_EINVAL, "generator: bad arguments N=%d", N);
  const int64_t ns = (int64_t)starts.size();
  if (first < 0 || count < 0 || first > ns || count > ns - first)
    return h->fail(NQ_EINVAL, "count_starts: range [%lld, +%lld) outside the %lld start constellations",
                   (long long)first, (long long)count, (long long)ns);
  return count_start_range(h, N, p, starts, (size_t)first, (size_t)(first + count), total);
}

int nq_last_count_info(const nq_handle* h, int64_t* chunks, int64_t* records) {
  if (!h) return NQ_EINVAL;
  if (chunks) *chunks = h->last_chunks;
  if (records) *records = h->last_records;
  return NQ_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// batches
// ---------------------------------------------------------------------------
struct nq_batch {
  nq_handle* h = nullptr;
  std::vector<nq_job> jobs;
  cudaStream_t stream = nullptr;
  cudaEvent_t done = nullptr;
  DevBuf rec, root, info, sched, ctrl, nsub, sroot, sinfo;
  int64_t m = 0;        // tasks
  int64_t ms = 0;       // queued subtasks (every job's split output, job after job)
  int maxt = 1, sw = 2, grid = 0, block = 128;
  bool big = false;                        // some job's queue items may count 2^32: u64 per-lane counters
  bool wide = true;                        // 8-byte schedule words (completion tasks); compact otherwise
  std::vector<int64_t> job_off, job_m;     // task range per job
  std::vector<int64_t> sub_off, sub_m;     // subtask range per job
  std::vector<int> job_maxt, job_split;
  std::vector<uint64_t> fixed_total;       // counts settled at build time (small tasks, full boards)
  uint64_t* h_out = nullptr;               // pinned: totals per job + cursor/err
  cudaGraphExec_t graph = nullptr;
  bool submitted = false;
  int64_t device_bytes = 0;
  int64_t h2d_bytes = 0;                   // host->device bytes of the build (records, host-built tasks)
  cudaError_t set_ordered() {
    for (DevBuf* d : {&rec, &root, &info, &sched, &ctrl, &nsub, &sroot, &sinfo}) d->ordered = stream;
    return cudaSuccess;
  }
};

namespace {

int batch_enqueue(nq_batch* b, int use_graph) {
  nq_handle* h = b->h;
  const int nj = (int)b->jobs.size();
  const size_t cb = Ctrl::bytes(nj);
  unsigned char* c = (unsigned char*)b->ctrl.p;
  auto enqueue = [&](cudaStream_t st) -> cudaError_t {
    cudaError_t e = cudaMemsetAsync(c, 0, cb, st);
    if (e != cudaSuccess) return e;
    TaskArrays ta;
    ta.root = (uint4*)b->root.p; ta.info = (uint2*)b->info.p; ta.sched = b->sched.p; ta.sw = b->sw; ta.wide = b->wide;
    DfsLaunch L;
    L.tasks = ta; L.sroot = (const uint4*)b->sroot.p; L.sinfo = (const uint2*)b->sinfo.p;
    L.m = b->ms; L.cursor = (unsigned long long*)(c + (size_t)nj * 8);
    L.job_totals = (unsigned long long*)c; L.err = (unsigned int*)(c + (size_t)nj * 8 + 8);
    L.maxt = b->maxt; L.block = b->block; L.grid = b->grid; L.big = b->big;
    e = launch_dfs(L, st);
    if (e != cudaSuccess) return e;
    return cudaMemcpyAsync(b->h_out, c, cb, cudaMemcpyDeviceToHost, st);
  };
  NQ_CUDA(h, cudaSetDevice(h->device));
  if (use_graph) {
    if (!b->graph) {
      cudaGraph_t g = nullptr;
      NQ_CUDA(h, cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
      cudaError_t e = enqueue(b->stream);
      cudaError_t e2 = cudaStreamEndCapture(b->stream, &g);
      if (e != cudaSuccess) { if (g) cudaGraphDestroy(g); return h->cuda_fail(e, "batch capture"); }
      if (e2 != cudaSuccess) return h->cuda_fail(e2, "cudaStreamEndCapture");
      e = cudaGraphInstantiate(&b->graph, g, 0);
      cudaGraphDestroy(g);
      if (e != cudaSuccess) { b->graph = nullptr; return h->cuda_fail(e, "cudaGraphInstantiate"); }
    }
    NQ_CUDA(h, cudaGraphLaunch(b->graph, b->stream));
  } else {
    NQ_CUDA(h, enqueue(b->stream));
  }
  NQ_CUDA(h, cudaEventRecord(b->done, b->stream));
  b->submitted = true;
  return NQ_OK;
}

int batch_collect(nq_batch* b, uint64_t* totals) {
  nq_handle* h = b->h;
  const int nj = (int)b->jobs.size();
  const uint32_t e = ((const uint32_t*)(b->h_out + nj))[2];
  b->submitted = false;
  if (e) return h->fail(derr_to_status(e), "device: %s", derr_text(e));
  if (totals)
    for (int j = 0; j < nj; j++) totals[j] = b->h_out[j] + b->fixed_total[j];
  return NQ_OK;
}

}  // namespace

extern "C" {

void nq_batch_destroy(nq_batch* b) {
  if (!b) return;
  cudaSetDevice(b->h->device);
  if (b->stream) cudaStreamSynchronize(b->stream);
  if (b->graph) cudaGraphExecDestroy(b->graph);
  b->rec.release(); b->root.release(); b->info.release(); b->sched.release(); b->ctrl.release();
  b->nsub.release(); b->sroot.release(); b->sinfo.release();
  if (b->stream) cudaStreamSynchronize(b->stream);   // this batch's own frees only
  b->h->pin_put(b->h_out);
  if (b->done) cudaEventDestroy(b->done);
  if (b->stream) cudaStreamDestroy(b->stream);
  delete b;
}

int nq_batch_create(nq_handle* h, const nq_job* jobs, int njobs, nq_batch** out) {
  if (!h || !out || njobs <= 0 || !jobs) return h ? h->fail(NQ_EINVAL, "batch: bad arguments") : NQ_EINVAL;
  *out = nullptr;
  NQ_CUDA(h, cudaSetDevice(h->device));
  nq_batch* b = new (std::nothrow) nq_batch();
  if (!b) return NQ_ENOMEM;
  b->h = h;
  b->jobs.assign(jobs, jobs + njobs);
  b->block = h->block;
  b->job_off.assign(njobs, 0); b->job_m.assign(njobs, 0); b->job_maxt.assign(njobs, 1); b->fixed_total.assign(njobs, 0);
  // Build: count jobs (N >= 6) become constellation records prepared on the
  // device; count jobs with N <= 5 and completion jobs become host tasks.
  struct Seg { int job, N; int64_t rec_off, m; };
  std::vector<Seg> segs;
  std::vector<nq_record> recs;
  std::vector<HostTask> htasks;
  std::vector<int64_t> job_host_begin(njobs, -1), job_host_end(njobs, -1);
  // The generator is deterministic in (N, preset): jobs that repeat a pair reuse
  // its records (each job still gets its own task segment and job id).
  struct Gen { std::vector<GenRecord> v; int smin; };
  std::map<std::pair<int, int>, Gen> generated;
  int maxt = 1;
  for (int j = 0; j < njobs; j++) {
    const nq_job& J = jobs[j];
    if (J.N < 1 || J.N > kMaxN || J.k < 0 || J.k > 8) { nq_batch_destroy(b); return h->fail(NQ_EINVAL, "batch job %d: bad N or k", j); }
    if (J.kind == NQ_JOB_COUNT && J.N >= 6) {
      const int p = J.preset > 0 ? J.preset : preset_for(J.N);
      auto it = generated.find({J.N, p});
      if (it == generated.end()) {
        Gen g;
        const int s = gen_constellations(J.N, p, g.v, 0);
        if (s != 0) { nq_batch_destroy(b); return h->fail(s == -2 ? NQ_EPRESET : NQ_EINVAL, "batch job %d: generator failed", j); }
        g.smin = 64;
        for (auto& r : g.v) g.smin = std::min<int>(g.smin, (int)(r.startijkl >> 20));
        it = generated.emplace(std::make_pair(J.N, p), std::move(g)).first;
      }
      const std::vector<GenRecord>& v = it->second.v;
      Seg sg{j, J.N, (int64_t)recs.size(), (int64_t)v.size()};
      for (auto& g : v) recs.push_back(nq_record{(uint32_t)g.ld, (uint32_t)g.rd, (uint32_t)g.col, g.startijkl});
      segs.push_back(sg);
      b->job_maxt[j] = maxt_for(J.N, it->second.smin);
      maxt = std::max(maxt, b->job_maxt[j]);
    } else if (J.kind == NQ_JOB_COUNT || J.kind == NQ_JOB_COMPLETION) {
      int rows[8], cols[8];
      const int k = (J.kind == NQ_JOB_COUNT) ? 0 : J.k;
      for (int q = 0; q < k; q++) { rows[q] = J.rows[q]; cols[q] = J.cols[q]; }
      int mt = 0;
      const int64_t before = (int64_t)htasks.size();
      const int s = build_completion_tasks(J.N, k, rows, cols, 4096, (uint32_t)j, htasks, &mt);
      if (s < 0) { nq_batch_destroy(b); return h->fail(NQ_EINVAL, "batch job %d: bad pre-placed queens", j); }
      if (s == 2) b->fixed_total[j] = 1;
      job_host_begin[j] = before; job_host_end[j] = (int64_t)htasks.size();
      b->job_maxt[j] = std::max(1, mt);
      maxt = std::max(maxt, b->job_maxt[j]);
    } else {
      nq_batch_destroy(b);
      return h->fail(NQ_EINVAL, "batch job %d: unknown kind %d", j, J.kind);
    }
  }
  if (maxt >= kMaxDepth) { nq_batch_destroy(b); return h->fail(NQ_ESTACK, "batch: schedule too deep"); }
  b->maxt = maxt; b->sw = maxt + 1;
  b->wide = !htasks.empty();             // constellation-only batches keep the compact 4-byte words
  const int64_t m_rec = (int64_t)recs.size(), m_host = (int64_t)htasks.size();
  b->m = m_rec + m_host;
  for (auto& sg : segs) { b->job_off[sg.job] = sg.rec_off; b->job_m[sg.job] = sg.m; }
  for (int j = 0; j < njobs; j++)
    if (job_host_begin[j] >= 0) { b->job_off[j] = m_rec + job_host_begin[j]; b->job_m[j] = job_host_end[j] - job_host_begin[j]; }
  const size_t cb = Ctrl::bytes(njobs);
  cudaError_t e;
  if ((e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking)) != cudaSuccess ||
      (e = cudaEventCreateWithFlags(&b->done, cudaEventDisableTiming)) != cudaSuccess ||
      (e = b->set_ordered()) != cudaSuccess ||
      (e = ((b->h_out = (uint64_t*)h->pin_get(cb)) ? cudaSuccess : cudaErrorMemoryAllocation)) != cudaSuccess ||
      (e = b->ctrl.ensure(cb)) != cudaSuccess ||
      (e = b->root.ensure((size_t)std::max<int64_t>(b->m, 1) * sizeof(uint4))) != cudaSuccess ||
      (e = b->info.ensure((size_t)std::max<int64_t>(b->m, 1) * sizeof(uint2))) != cudaSuccess ||
      (e = b->sched.ensure((size_t)std::max<int64_t>(b->m, 1) * b->sw * (b->wide ? sizeof(uint2) : sizeof(uint32_t)))) !=
          cudaSuccess ||
      (e = b->rec.ensure((size_t)std::max<int64_t>(m_rec, 1) * sizeof(nq_record))) != cudaSuccess) {
    int st = h->cuda_fail(e, "batch allocation");
    nq_batch_destroy(b);
    return st;
  }
  b->device_bytes = (int64_t)(b->root.cap + b->info.cap + b->sched.cap + b->rec.cap + b->ctrl.cap);
  TaskArrays ta;
  ta.root = (uint4*)b->root.p; ta.info = (uint2*)b->info.p; ta.sched = b->sched.p; ta.sw = b->sw; ta.wide = b->wide;
  unsigned char* c = (unsigned char*)b->ctrl.p;
  unsigned int* derr = (unsigned int*)(c + (size_t)njobs * 8 + 8);
  cudaStream_t st = b->stream;
  int status = NQ_OK;
  DevBuf jt;                                   // deepest schedule per job (constellation jobs)
  jt.ordered = st;
  std::vector<uint32_t> job_deep(njobs, 0);
  do {
    if ((e = cudaMemsetAsync(c, 0, cb, st)) != cudaSuccess) break;
    if ((e = jt.ensure((size_t)njobs * sizeof(uint32_t))) != cudaSuccess) break;
    if ((e = cudaMemsetAsync(jt.p, 0, (size_t)njobs * sizeof(uint32_t), st)) != cudaSuccess) break;
    if (m_rec && (e = cudaMemcpyAsync(b->rec.p, recs.data(), (size_t)m_rec * sizeof(nq_record), cudaMemcpyHostToDevice, st)) != cudaSuccess) break;
    b->h2d_bytes = m_rec * (int64_t)sizeof(nq_record) +
                   m_host * (int64_t)(sizeof(uint4) + sizeof(uint2) + (size_t)b->sw * sizeof(uint2));
    for (auto& sg : segs)
      if ((e = launch_prepare(sg.N, sg.m, (const uint4*)b->rec.p + sg.rec_off, ta, sg.rec_off, (uint32_t)sg.job, derr, st,
                              (unsigned int*)jt.p + sg.job)) != cudaSuccess) break;
    if (e != cudaSuccess) break;
    if ((e = cudaMemcpyAsync(job_deep.data(), jt.p, (size_t)njobs * sizeof(uint32_t), cudaMemcpyDeviceToHost, st)) !=
        cudaSuccess) break;
    if (m_host) {
      std::vector<uint4> hr(m_host);
      std::vector<uint2> hi(m_host);
      std::vector<uint2> hs((size_t)m_host * b->sw, make_uint2(0, 0));
      for (int64_t i = 0; i < m_host; i++) {
        const HostTask& t = htasks[i];
        hr[i] = make_uint4(t.root[0], t.root[1], t.root[2], t.root[3]);
        hi[i] = make_uint2(t.info, t.job);
        for (int d = 0; d <= t.T; d++) hs[(size_t)i * b->sw + d] = make_uint2(t.sched[2 * d], t.sched[2 * d + 1]);
      }
      if ((e = cudaMemcpyAsync((uint4*)b->root.p + m_rec, hr.data(), m_host * sizeof(uint4), cudaMemcpyHostToDevice, st)) != cudaSuccess) break;
      if ((e = cudaMemcpyAsync((uint2*)b->info.p + m_rec, hi.data(), m_host * sizeof(uint2), cudaMemcpyHostToDevice, st)) != cudaSuccess) break;
      if ((e = cudaMemcpyAsync((uint2*)b->sched.p + (size_t)m_rec * b->sw, hs.data(), hs.size() * sizeof(uint2),
                               cudaMemcpyHostToDevice, st)) != cudaSuccess) break;
      if ((e = cudaStreamSynchronize(st)) != cudaSuccess) break;   // host staging vectors go out of scope
    }
    if ((e = cudaMemcpyAsync(b->h_out, c, cb, cudaMemcpyDeviceToHost, st)) != cudaSuccess) break;
    if ((e = cudaStreamSynchronize(st)) != cudaSuccess) break;
    const uint32_t de = ((const uint32_t*)(b->h_out + njobs))[2];
    if (de) { status = h->fail(derr_to_status(de), "batch prepare: %s", derr_text(de)); break; }
    // Split each job on its own (tiny boards are not split), so every job's
    // subtasks form one contiguous queue range: pass 0 counts per job, then
    // pass 1 writes job after job behind one allocation cursor.
    b->job_split.assign(njobs, 0);
    b->sub_off.assign(njobs, 0); b->sub_m.assign(njobs, 0);
    if ((e = b->nsub.ensure((size_t)std::max<int64_t>(b->m, 1) * sizeof(uint32_t))) != cudaSuccess) break;
    DevBuf sctr;
    sctr.ordered = st;
    if ((e = sctr.ensure((size_t)(njobs + 1) * 16)) != cudaSuccess) break;
    unsigned long long* sc = (unsigned long long*)sctr.p;   // [2j] subtasks of job j, [2*njobs+1] cursor
    if ((e = cudaMemsetAsync(sc, 0, (size_t)(njobs + 1) * 16, st)) != cudaSuccess) { sctr.release(); break; }
    for (int j = 0; j < njobs && e == cudaSuccess; j++) {
      b->job_split[j] = (jobs[j].N <= 12) ? 0 : (h->split >= 0 ? h->split : choose_split(b->job_m[j], h->sms));
      e = launch_split(0, b->job_split[j], b->job_off[j], b->job_m[j], ta, (uint32_t*)b->nsub.p, nullptr, nullptr,
                       sc + 2 * j, nullptr, nullptr, 0, st);
    }
    std::vector<unsigned long long> cnts((size_t)(njobs + 1) * 2, 0);
    if (e == cudaSuccess) e = cudaMemcpyAsync(cnts.data(), sc, cnts.size() * 8, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) { sctr.release(); break; }
    int64_t total_sub = 0;
    for (int j = 0; j < njobs; j++) { b->sub_off[j] = total_sub; b->sub_m[j] = (int64_t)cnts[2 * j]; total_sub += b->sub_m[j]; }
    for (int j = 0; j < njobs; j++) b->big = b->big || (b->sub_m[j] > 0 && counts_need_u64(jobs[j].N, b->sub_m[j]));
    b->ms = total_sub;
    // Stacks sized to the deepest subtask: a job's subtasks start at depth
    // job_split[j], so they need (deepest T) - job_split[j] frames.
    b->maxt = 1;
    for (int j = 0; j < njobs; j++) {
      const int deep = (job_host_begin[j] >= 0) ? b->job_maxt[j] : (int)job_deep[j];
      b->job_maxt[j] = std::max(1, std::min(b->job_maxt[j], deep - b->job_split[j]));
      b->maxt = std::max(b->maxt, b->job_maxt[j]);
    }
    if ((e = b->sroot.ensure((size_t)std::max<int64_t>(total_sub, 1) * sizeof(uint4))) != cudaSuccess ||
        (e = b->sinfo.ensure((size_t)std::max<int64_t>(total_sub, 1) * sizeof(uint2))) != cudaSuccess) { sctr.release(); break; }
    // settled counts of small tasks land in the control block's totals (zeroed above)
    for (int j = 0; j < njobs && e == cudaSuccess; j++)
      e = launch_split(1, b->job_split[j], b->job_off[j], b->job_m[j], ta, (uint32_t*)b->nsub.p, (uint4*)b->sroot.p,
                       (uint2*)b->sinfo.p, sc + 2 * njobs, nullptr, (unsigned long long*)c, 0, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(b->h_out, c, cb, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    sctr.release();
    if (e != cudaSuccess) break;
    for (int j = 0; j < njobs; j++) b->fixed_total[j] += b->h_out[j];
    b->device_bytes = (int64_t)(b->root.cap + b->info.cap + b->sched.cap + b->rec.cap + b->ctrl.cap + b->nsub.cap +
                                b->sroot.cap + b->sinfo.cap);
  } while (0);
  jt.release();
  if (e != cudaSuccess) status = h->cuda_fail(e, "batch build");
  if (status != NQ_OK) { nq_batch_destroy(b); return status; }
  *out = b;
  return NQ_OK;
}

int64_t nq_job_device_bytes(const nq_job* job, int sms, int split_depth) {
  if (!job || sms < 1 || split_depth < -1 || split_depth > 3) return NQ_EINVAL;
  const nq_job& J = *job;
  if (J.N < 1 || J.N > kMaxN || J.k < 0 || J.k > 8) return NQ_EINVAL;
  int64_t m = 0;
  size_t word = 0;
  int maxt = 1;
  if (J.kind == NQ_JOB_COUNT && J.N >= 6) {
    // the generator's record count, as nq_batch_create builds the job (compact schedule words)
    const int p = J.preset > 0 ? J.preset : preset_for(J.N);
    std::vector<GenRecord> v;
    const int s = gen_constellations(J.N, p, v, 0);
    if (s != 0) return s == -2 ? NQ_EPRESET : NQ_EINVAL;
    m = (int64_t)v.size();
    int smin = 64;
    for (const GenRecord& r : v) smin = std::min<int>(smin, (int)(r.startijkl >> 20));
    maxt = maxt_for(J.N, smin);
    word = sizeof(uint32_t);
  } else if (J.kind == NQ_JOB_COUNT || J.kind == NQ_JOB_COMPLETION) {
    int rows[8], cols[8];
    const int k = (J.kind == NQ_JOB_COUNT) ? 0 : J.k;
    for (int q = 0; q < k; q++) { rows[q] = J.rows[q]; cols[q] = J.cols[q]; }
    std::vector<HostTask> t;
    int mt = 0;
    if (build_completion_tasks(J.N, k, rows, cols, 4096, 0, t, &mt) < 0) return NQ_EINVAL;
    m = (int64_t)t.size();
    maxt = std::max(1, mt);
    word = sizeof(uint2);
  } else {
    return NQ_EINVAL;
  }
  // split queue: each level multiplies the items by at most ~8 (measured 6.2-8x)
  const int D = (J.N <= 12) ? 0 : (split_depth >= 0 ? split_depth : choose_split(m, sms));
  int64_t ns = m;
  for (int d = 0; d < D; d++) ns *= 8;
  const int64_t per_task = 16 /*record*/ + 16 /*root*/ + 8 /*info*/ + 4 /*split count*/ + (int64_t)(maxt + 1) * (int64_t)word;
  return m * per_task + ns * (16 + 8) + (int64_t)Ctrl::bytes(1) + 4096;
}

int nq_batch_set_grid(nq_batch* b, int grid) {
  if (!b || grid < 0) return NQ_EINVAL;
  if (b->submitted) return b->h->fail(NQ_EBUSY, "batch is running");
  if (b->graph) { cudaGraphExecDestroy(b->graph); b->graph = nullptr; }   // the captured launch used the old grid
  b->grid = grid;
  return NQ_OK;
}

int nq_resident_blocks(nq_handle* h, int wide, int maxt, int* blocks) {
  if (!h || !blocks || maxt < 1 || maxt >= kMaxDepth) return NQ_EINVAL;
  *blocks = h->sms * std::max(1, dfs_blocks_per_sm(wide != 0, h->block, maxt));
  return NQ_OK;
}

int nq_batch_resident_blocks(const nq_batch* b, int* blocks) {
  if (!b || !blocks) return NQ_EINVAL;
  *blocks = b->h->sms * std::max(1, dfs_blocks_per_sm(b->wide, b->block, b->maxt));
  return NQ_OK;
}

int64_t nq_batch_tasks(const nq_batch* b) { return b ? b->m : NQ_EINVAL; }
int64_t nq_batch_device_bytes(const nq_batch* b) { return b ? b->device_bytes : NQ_EINVAL; }
int64_t nq_batch_h2d_bytes(const nq_batch* b) { return b ? b->h2d_bytes : NQ_EINVAL; }

int nq_batch_submit(nq_batch* b, int use_graph) {
  if (!b) return NQ_EINVAL;
  if (b->submitted) return b->h->fail(NQ_EBUSY, "batch already submitted");
  return batch_enqueue(b, use_graph);
}

int nq_batch_poll(nq_batch* b, uint64_t* totals, int64_t max_wait_us) {
  if (!b) return NQ_EINVAL;
  if (!b->submitted) return b->h->fail(NQ_EINVAL, "batch not submitted");
  const auto t0 = std::chrono::steady_clock::now();
  for (;;) {
    cudaError_t q = cudaEventQuery(b->done);
    if (q == cudaSuccess) break;
    if (q != cudaErrorNotReady) return b->h->cuda_fail(q, "cudaEventQuery");
    const int64_t us = std::chrono::duration_cast<std::chrono::microseconds>(std::chrono::steady_clock::now() - t0).count();
    if (us >= max_wait_us) return NQ_EBUSY;
    std::this_thread::sleep_for(std::chrono::microseconds(20));
  }
  return batch_collect(b, totals);
}

int nq_batch_run(nq_batch* b, int use_graph, uint64_t* totals) {
  if (!b) return NQ_EINVAL;
  if (int s = nq_batch_submit(b, use_graph)) return s;
  NQ_CUDA(b->h, cudaEventSynchronize(b->done));
  return batch_collect(b, totals);
}

int nq_batch_run_plain(nq_batch* b, uint64_t* totals) {
  if (!b) return NQ_EINVAL;
  nq_handle* h = b->h;
  const int nj = (int)b->jobs.size();
  unsigned char* c = (unsigned char*)b->ctrl.p;
  NQ_CUDA(h, cudaSetDevice(h->device));
  for (int j = 0; j < nj; j++) {
    uint64_t t = 0;
    if (b->sub_m[j] > 0) {
      NQ_CUDA(h, cudaMemsetAsync(c, 0, 24, b->stream));
      TaskArrays ta;
      ta.root = (uint4*)b->root.p; ta.info = (uint2*)b->info.p; ta.sched = b->sched.p; ta.sw = b->sw; ta.wide = b->wide;
      // One job per launch over its subtask range; its tasks carry job id j, which lands in slot 0.
      DfsLaunch L;
      L.tasks = ta; L.sroot = (const uint4*)b->sroot.p + b->sub_off[j]; L.sinfo = (const uint2*)b->sinfo.p + b->sub_off[j];
      L.m = b->sub_m[j]; L.cursor = (unsigned long long*)(c + 8);
      L.job_totals = (unsigned long long*)c; L.job_base = (uint32_t)j; L.err = (unsigned int*)(c + 16);
      L.maxt = b->job_maxt[j]; L.block = b->block; L.grid = b->grid; L.big = counts_need_u64(b->jobs[j].N, b->sub_m[j]);
      NQ_CUDA(h, launch_dfs(L, b->stream));
      NQ_CUDA(h, cudaMemcpyAsync(b->h_out, c, 24, cudaMemcpyDeviceToHost, b->stream));
      NQ_CUDA(h, cudaStreamSynchronize(b->stream));
      const uint32_t e = ((const uint32_t*)b->h_out)[4];
      if (e) return h->fail(derr_to_status(e), "device: %s", derr_text(e));
      t = b->h_out[0];
    }
    if (totals) totals[j] = t + b->fixed_total[j];
  }
  return NQ_OK;
}

int nq_count_completions(nq_handle* h, int N, int k, const int* rows, const int* cols, uint64_t* count) {
  if (!h || !count || k < 0 || k > 8 || (k > 0 && (!rows || !cols))) return h ? h->fail(NQ_EINVAL, "bad arguments") : NQ_EINVAL;
  if (N < 1 || N > kMaxN) return h->fail(NQ_EINVAL, "N=%d outside 1..27", N);
  nq_job J;
  std::memset(&J, 0, sizeof J);
  J.kind = NQ_JOB_COMPLETION; J.N = N; J.k = k;
  for (int q = 0; q < k; q++) {
    if (rows[q] < 0 || rows[q] >= N || cols[q] < 0 || cols[q] >= N) return h->fail(NQ_EINVAL, "queen outside the board");
    J.rows[q] = (int8_t)rows[q]; J.cols[q] = (int8_t)cols[q];
  }
  nq_batch* b = nullptr;
  if (int s = nq_batch_create(h, &J, 1, &b)) return s;
  const int s = nq_batch_run(b, 0, count);
  nq_batch_destroy(b);
  return s;
}

}  // extern "C"
