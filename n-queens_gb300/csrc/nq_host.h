// nq_host.h -- host task builders (see nq_host.cpp).
#pragma once
#include <stdint.h>
#include <vector>

#include "nq_common.cuh"

namespace nq {

// One generated constellation with full-width masks (the reference keeps
// them as Python ints; bits above 31 only matter for its 40-byte
// solution-file layout).
struct GenRecord {
  uint64_t ld, rd, col;
  uint32_t startijkl;
};

// A host-built task in the wide schedule format.
struct HostTask {
  uint32_t root[4];                 // ld, rd, col, avail
  uint32_t info;                    // info word (T, wexp, root count, N, status)
  uint32_t job;
  int T;
  uint32_t sched[2 * kMaxDepth];    // wide words (x, RA) for depths 0..T
};

// Returns 0, -1 (bad arguments) or -2 (the reference would raise: a preset too
// deep for N).  threads <= 0: all hardware threads.
int gen_constellations(int N, int preset, std::vector<GenRecord>& out, int threads);

// The same in two parts, for generating a large board chunk by chunk with
// bounded host memory: the canonical start constellations (packed ijkl,
// ascending; cheap), then the records of starts[s0..s1) appended to `out` in
// start order (the expansion runs on `threads` host threads).
int start_constellations(int N, std::vector<int>& starts);
int expand_starts(int N, int preset, const std::vector<int>& starts, size_t s0, size_t s1,
                  std::vector<GenRecord>& out, int threads);

// Tasks whose counts sum to the number of N-queens solutions containing the
// k pre-placed queens (rows[q], cols[q]); no symmetry weight.  Returns 0 with
// tasks appended, 1 when the count is 0 without any task (attacking queens or
// two queens in one row), 2 when the count is 1 without any task (the queens
// fill every row), -1 on bad arguments.  *max_T is raised to the deepest
// task's terminal depth.
int build_completion_tasks(int N, int k, const int* rows, const int* cols, int min_tasks, uint32_t job,
                           std::vector<HostTask>& out, int* max_T);

// Smallest start row over m records (startijkl >> 20), reading every
// stride_words-th uint32 (4 for packed 16-byte records).
int64_t start_row_min(const uint32_t* startijkl, int64_t m, int stride_words);

}  // namespace nq
