// nq_internal.h -- internal interface between the C-ABI layer (nq_capi.cu),
// the host task builders (nq_host.cpp) and the sm_103a kernels
// (nq_kernels.cu).  Not installed; the public interface is
// include/nqueens_gb300.h.
#pragma once
#include <stdint.h>
#include <cuda_runtime.h>

namespace nq {

// Device-side error bits (OR-ed into a device word, read back by the host).
constexpr uint32_t DERR_SHIFT = 1u;      // a record needs a negative shift (reference would raise)
constexpr uint32_t DERR_DEPTH = 2u;      // a task's schedule is deeper than the launch's stack
constexpr uint32_t DERR_NOTERM = 4u;     // a schedule never reaches a base frame
constexpr uint32_t DERR_BADN = 8u;       // N outside 6..27 in a task
constexpr uint32_t DERR_FORMAT = 16u;    // a schedule op does not fit the compact word's fields

// Prepared task arrays (structure of arrays, one entry per task).
struct TaskArrays {
  uint4* root = nullptr;      // {ld, rd, col, avail} of the root frame
  uint2* info = nullptr;      // {info word (T, wexp, root count, N, status), job id}
  void* sched = nullptr;      // per-task schedule words, stride `sw` words
  int sw = 0;                 // schedule words per task (>= T+1 of every task)
  bool wide = false;          // uint2 words (mixed batches) instead of uint32
};

struct DfsLaunch {
  TaskArrays tasks;
  const uint4* sroot = nullptr;         // split queue: subtask frames ...
  const uint2* sinfo = nullptr;         // ... and {task, depth}; nullptr: the queue holds tasks
  int64_t m = 0;                        // queue length
  const uint32_t* order = nullptr;      // optional queue order (task index per slot)
  unsigned long long* cursor = nullptr; // queue cursor (device, zeroed before launch; 64-bit, so it never wraps)
  unsigned long long* job_totals = nullptr;  // weighted totals, slot (job id - job_base) (device)
  uint32_t job_base = 0;
  unsigned long long* per_task = nullptr;    // optional weighted count per task (device)
  unsigned int* err = nullptr;          // device error word
  int maxt = 0;                         // stack frames per lane (>= T of every task; words: maxt+1)
  bool big = false;                     // u64 per-task counters (some task has N >= 24)
  int block = 128;
  int grid = 0;                         // 0: one wave of resident blocks
};

// Prepare: records {ld, rd, col, startijkl} (the reference's 16-byte task
// record) -> task arrays.  job/offset place the tasks of one job inside a
// larger queue.
// tmax (optional): atomicMax of the schedule depth T over the launch's tasks.
cudaError_t launch_prepare(int N, int64_t m, const uint4* records, const TaskArrays& out, int64_t offset,
                           uint32_t job, unsigned int* err, cudaStream_t st, unsigned int* tmax = nullptr);

cudaError_t launch_dfs(const DfsLaunch& L, cudaStream_t st);

// Split tasks t0..t0+m-1 to depth D (0..3; 0 queues the tasks themselves).
// pass 0: nsub[t] and ctr[0] += subtasks; pass 1: writes subtasks at the
// allocation cursor ctr[1], initialises per_task (nullable) and adds counts
// settled above depth D to job_totals.
cudaError_t launch_split(int pass, int D, int64_t t0, int64_t m, const TaskArrays& ta, uint32_t* nsub, uint4* sroot,
                         uint2* sinfo, unsigned long long* ctr, unsigned long long* per_task,
                         unsigned long long* job_totals, uint32_t job_base, cudaStream_t st);

// Queue order, largest estimated subtree first: order[0..m) receives the queue
// indices (subtasks when sinfo is set, else tasks); keys: m bytes of scratch,
// hist_offs: 512 u32 of scratch.
cudaError_t launch_order(int64_t m, const uint4* sroot, const uint2* sinfo, const TaskArrays& ta, uint8_t* keys,
                         unsigned int* hist_offs, uint32_t* order, cudaStream_t st);

// Largest block count per SM for a given stack depth (occupancy query).
int dfs_blocks_per_sm(bool wide, int block, int maxt);

// INT32 throughput probe: grid x 256 threads x iters x 128 instructions of
// one kind (0 lop3, 1 add, 2 shf, 3 mix).
cudaError_t int_peak(int kind, int iters, int grid, uint32_t* out, cudaStream_t st);
size_t dfs_smem_bytes(bool wide, int block, int maxt);

}  // namespace nq
