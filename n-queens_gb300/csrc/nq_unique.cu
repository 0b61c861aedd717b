// nq_unique.cu -- unique and total counts by the symmetry method on sm_103a.
//
// Restates the classic symmetry-elimination search of the reference
// (11Bit_Python/07Py_bit_symmetry.py:65-200; GPU form 10Bit_CUDA/
// 01CUDA_Bit_Symmetry.cu:627-960):
//   * corner solutions: queen at row 0 column 0, row 1 at column bound1
//     (2 <= bound1 <= N-2); rows below bound1 may not use column 1; every
//     solution counts x8 (backTrack1, :152-170);
//   * the rest: row 0 at column bound1 with bound2 = N-1-bound1 and
//     bound1 < bound2; rows above bound1 avoid the side columns, row bound2 is
//     gated on the side columns used so far, the last row must avoid lastmask
//     (backTrack2, :126-151); each solution is classified by its rotations as
//     x2, x4 or x8 or dropped as a non-canonical copy (symmetryops, :65-125).
// Unique = c2 + c4 + c8, total = 2 c2 + 4 c4 + 8 c8.
//
// The host expands the first rows of every (part, bound1) start into tasks;
// the kernel is persistent, queue-fed and explicit-stack like the
// constellation DFS (one candidate per lane per step, predicated pop/push,
// the row carried in `down`'s high bits), keeping each lane's board (one bit
// per row) in shared memory for the leaf classification.
#include <cuda_runtime.h>

#include <algorithm>
#include <vector>

#include "../../include/nqueens_gb300.h"
#include "nq_common.cuh"
#include "nq_handle.h"
#include "nq_internal.h"

namespace nq {
namespace {

constexpr unsigned FULLM = 0xFFFFFFFFu;
constexpr int kBoardWords = 8;   // rows of the board prefix carried by a task
constexpr int kUniqueSteps = 16;   // steps per lane between checks for finished lanes

// One start configuration (symmetry part and its bounds).
struct UConf {
  uint32_t part;       // 1 corner, 2 no corner
  uint32_t bound1, bound2, endbit, lastmask, sidemask, topbit;
};

// A task: the search state at `row` plus the board rows above it.
struct UTask {
  uint32_t left, down, right, avail;
  uint32_t row, conf;
  uint32_t board[kBoardWords];
};

// symmetryops (07Py_bit_symmetry.py:65-125): 2, 4 or 8 for a canonical
// solution, 0 for a rotated copy.  `b(k)` reads board row k.
template <typename B>
__device__ __forceinline__ uint32_t classify(const B& b, int size, const UConf& c) {
  int own, you;
  uint32_t bit, ptn;
  if (b(c.bound2) == 1u) {                        // 90 degrees
    own = 1; ptn = 2;
    while (own <= size - 1) {
      bit = 1; you = size - 1;
      while (b(you) != ptn && b(own) >= bit) { bit <<= 1; you--; }
      if (b(own) > bit) return 0;
      if (b(own) < bit) break;
      own++; ptn <<= 1;
    }
    if (own > size - 1) return 2;
  }
  if (b(size - 1) == c.endbit) {                  // 180 degrees
    own = 1; you = size - 2;
    while (own <= size - 1) {
      bit = 1; ptn = c.topbit;
      while (b(you) != ptn && b(own) >= bit) { bit <<= 1; ptn >>= 1; }
      if (b(own) > bit) return 0;
      if (b(own) < bit) break;
      own++; you--;
    }
    if (own > size - 1) return 4;
  }
  if (b(c.bound1) == c.topbit) {                  // 270 degrees
    own = 1; ptn = c.topbit >> 1;
    while (own <= size - 1) {
      bit = 1; you = 0;
      while (b(you) != ptn && b(own) >= bit) { bit <<= 1; you++; }
      if (b(own) > bit) return 0;
      if (b(own) < bit) break;
      own++; ptn >>= 1;
    }
  }
  return 8;
}

// Row rules of backTrack1/backTrack2 applied to the candidate set of `row`.
__host__ __device__ __forceinline__ uint32_t row_filter(uint32_t bitmap, uint32_t row, uint32_t down, const UConf& c) {
  if (c.part == 1) return row < c.bound1 ? (bitmap & ~2u) : bitmap;
  if (row < c.bound1) return bitmap & ~c.sidemask;
  if (row == c.bound2) {
    const uint32_t ds = down & c.sidemask;
    if (ds == 0u) return 0u;
    if (ds != c.sidemask) return bitmap & c.sidemask;
  }
  return bitmap;
}

struct UArgs {
  const UTask* tasks;
  const UConf* confs;
  int64_t m;
  int N;
  int maxf;                     // stack frames per lane: N - 2 - (smallest task row)
  unsigned int* cursor;
  unsigned long long* counts;   // c2, c4, c8
  unsigned int* err;
};

// Predicated shared-memory stores (32-bit shared-window addresses), so the push is
// a single predicated instruction, not a branch.
__device__ __forceinline__ void sts_frame_if(uint32_t p, uint32_t a, uint32_t x, uint32_t y, uint32_t z, uint32_t w) {
  asm volatile("{\n\t.reg .pred q;\n\tsetp.ne.u32 q, %0, 0;\n\t@q st.shared.v4.u32 [%1], {%2, %3, %4, %5};\n\t}"
               :: "r"(p), "r"(a), "r"(x), "r"(y), "r"(z), "r"(w) : "memory");
}
__device__ __forceinline__ void sts_word_if(uint32_t p, uint32_t a, uint32_t x) {
  asm volatile("{\n\t.reg .pred q;\n\tsetp.ne.u32 q, %0, 0;\n\t@q st.shared.u32 [%1], %2;\n\t}"
               :: "r"(p), "r"(a), "r"(x) : "memory");
}

// One lane per task, one candidate per step, all lanes on the same predicated
// sequence: resume a saved frame, take the lowest candidate, record it in the
// board, build the next row with the part's row rules, then count (last row)
// or descend.  The row of a frame rides in `down` bits 27-31 (columns use bits
// 0..N-1, N <= 27), so a saved frame is exactly {left, down, right, avail}.
template <int BLOCK>
__global__ void __launch_bounds__(BLOCK) unique_kernel(const UArgs a) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int N = a.N;
  constexpr uint32_t F = BLOCK * (uint32_t)sizeof(uint4);          // frame stride of one lane's stack
  constexpr uint32_t RB = BLOCK * (uint32_t)sizeof(uint32_t);      // board row stride
  // a lane pushes at most one frame per row from its task's row to N - 3
  uint4* stk = reinterpret_cast<uint4*>(smem) + threadIdx.x;                            // maxf frames, stride BLOCK
  uint32_t* brd = reinterpret_cast<uint32_t*>(smem + (size_t)a.maxf * BLOCK * sizeof(uint4)) + threadIdx.x;  // N rows
  const uint32_t sbase = (uint32_t)__cvta_generic_to_shared(stk);
  const uint32_t bbase = (uint32_t)__cvta_generic_to_shared(brd);
  const unsigned lane = threadIdx.x & 31u;
  const uint32_t mask = (1u << N) - 1u;
  const uint32_t last_row = (uint32_t)N - 1u;
  uint32_t left = 0, down = 0, right = 0, avail = 0, sp = sbase;
  UConf cf = {0, 0, 0, 0, 0, 0, 0};
  uint32_t lowmask = ~0u, b2 = ~0u;      // row rules of the task's part
  unsigned long long c2 = 0, c4 = 0, c8 = 0;
  bool exhausted = false;
  for (;;) {
    const bool idle = (avail | (sp - sbase)) == 0u;
    if (__ballot_sync(FULLM, idle)) {
      const bool want = idle && !exhausted;
      const unsigned need = __ballot_sync(FULLM, want);
      if (need) {
        const int leader = __ffs(need) - 1;
        unsigned base = 0;
        if ((int)lane == leader) base = atomicAdd(a.cursor, (unsigned)__popc(need));
        base = __shfl_sync(FULLM, base, leader);
        if (want) {
          const uint64_t slot = (uint64_t)base + (uint64_t)__popc(need & ((1u << lane) - 1u));
          if (slot < (uint64_t)a.m) {
            const UTask t = a.tasks[slot];
            cf = a.confs[t.conf];
            // part 1: rows above bound1 avoid column 1; part 2: they avoid the side
            // columns, and row bound2 is gated on the side columns used so far
            lowmask = (cf.part == 1) ? ~2u : ~cf.sidemask;
            b2 = (cf.part == 1) ? ~0u : cf.bound2;
            left = t.left; down = (t.down & mask) | (t.row << 27); right = t.right; avail = t.avail; sp = sbase;
            for (uint32_t r = 0; r < t.row && r < (uint32_t)kBoardWords; r++) brd[r * BLOCK] = t.board[r];
          } else {
            exhausted = true;
          }
        }
      }
      if (__all_sync(FULLM, exhausted && (avail | (sp - sbase)) == 0u)) break;
      asm volatile("" ::: "memory");   // board stores of the refill before the steps' accesses
    }
    // kUniqueSteps steps between two checks for finished lanes (two ballots each)
#pragma unroll 1
    for (int s = 0; s < kUniqueSteps; ++s) {
      // pop with its condition formed in a predicate register inside the block (no 0/1 value for it)
      asm volatile("{\n\t.reg .pred q;\n\tsetp.eq.u32 q, %3, 0;\n\tsetp.ne.and.u32 q, %4, %5, q;\n\t"
                   "@q sub.u32 %4, %4, %6;\n\t@q ld.shared.v4.u32 {%0, %1, %2, %3}, [%4];\n\t}"
                   : "+r"(left), "+r"(down), "+r"(right), "+r"(avail), "+r"(sp) : "r"(sbase), "n"(F));
      const uint32_t row = __umulhi(down, 32u);                 // down >> 27
      const bool act = avail != 0u;
      const uint32_t bit = avail & (0u - avail);
      avail -= bit;
      sts_word_if(act ? 1u : 0u, bbase + row * RB, bit);        // board row `row` = the queen taken
      const uint32_t nl = (left + bit) * 2u;
      const uint32_t nd = down + bit;
      const uint32_t nr = __umulhi(right + bit, 0x80000000u);   // (right | bit) >> 1
      const uint32_t nrow = row + 1u;
      const uint32_t nb = mask & ~(nl | nd | nr);
      const bool last = nrow == last_row;
      // row rules of backTrack1/backTrack2 (row_filter) as selects
      uint32_t nbf = nb & ((nrow < cf.bound1) ? lowmask : ~0u);
      const uint32_t ds = nd & cf.sidemask;
      const uint32_t at_b2 = (ds == 0u) ? 0u : ((ds != cf.sidemask) ? (nbf & cf.sidemask) : nbf);
      nbf = (nrow == b2) ? at_b2 : nbf;
      // last row: a solution (part 1: x8) or a board to classify (part 2)
      if (act && last && nb != 0u) {
        if (cf.part == 1) {
          c8++;
        } else if ((nb & cf.lastmask) == 0u) {
          brd[nrow * BLOCK] = nb;
          const uint32_t k = classify([&](int r) { return brd[r * BLOCK]; }, N, cf);
          c2 += (k == 2); c4 += (k == 4); c8 += (k == 8);
        }
      }
      const bool desc = act && !last && nbf != 0u;
      const uint32_t push = (desc && avail != 0u) ? 1u : 0u;
      sts_frame_if(push, sp, left, down, right, avail);
      sp += push ? F : 0u;
      if (desc) { left = nl; down = nd + (1u << 27); right = nr; avail = nbf; }
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    c2 += __shfl_xor_sync(FULLM, c2, o);
    c4 += __shfl_xor_sync(FULLM, c4, o);
    c8 += __shfl_xor_sync(FULLM, c8, o);
  }
  if (lane == 0) {
    if (c2) atomicAdd(a.counts + 0, c2);
    if (c4) atomicAdd(a.counts + 1, c4);
    if (c8) atomicAdd(a.counts + 2, c8);
  }
}

// Host: every (part, bound1) start of 07Py_bit_symmetry.py NQueens() (:171-200),
// expanded breadth-first over its first rows until there are enough tasks.
int build_unique_tasks(int N, int64_t min_tasks, std::vector<UConf>& confs, std::vector<UTask>& tasks) {
  const uint32_t mask = (1u << N) - 1u;
  // Search states are kept in the task layout itself (avail is filled in at the
  // end), so the last level becomes the task list without another copy.
  std::vector<UTask> cur;
  // part 1: corner queen
  for (int b1 = 2; b1 < N - 1; b1++) {
    UConf c = {1, (uint32_t)b1, 0, 0, 0, 0, 1u << (N - 1)};
    confs.push_back(c);
    const uint32_t bit = 1u << b1;
    UTask s{};
    s.left = (2u | bit) << 1; s.down = 1u | bit; s.right = (2u | bit) >> 1; s.row = 2;
    s.board[0] = 1; s.board[1] = bit; s.conf = (uint32_t)confs.size() - 1;
    cur.push_back(s);
  }
  // part 2: no corner queen
  {
    const uint32_t topbit = 1u << (N - 1);
    uint32_t endbit = topbit >> 1, lastmask = topbit | 1u;
    const uint32_t sidemask = topbit | 1u;
    for (int b1 = 1, b2 = N - 2; b1 > 0 && b2 < N - 1 && b1 < b2; b1++, b2--) {
      UConf c = {2, (uint32_t)b1, (uint32_t)b2, endbit, lastmask, sidemask, topbit};
      confs.push_back(c);
      const uint32_t bit = 1u << b1;
      UTask s{};
      s.left = bit << 1; s.down = bit; s.right = bit >> 1; s.row = 1; s.board[0] = bit;
      s.conf = (uint32_t)confs.size() - 1;
      cur.push_back(s);
      endbit >>= 1;
      lastmask = (lastmask << 1) | lastmask | (lastmask >> 1);
    }
  }
  // expand whole rows breadth-first (tasks of one row are of similar size) while
  // the tasks stay above the last row and fit the board prefix
  std::vector<UTask> nxt;
  while ((int64_t)cur.size() < min_tasks) {
    bool grew = false;
    nxt.clear();
    nxt.reserve(cur.size() * (size_t)N);
    for (const UTask& s : cur) {
      if ((int)s.row + 1 >= N - 1 || s.row + 1 >= (uint32_t)kBoardWords) { nxt.push_back(s); continue; }
      uint32_t bm = row_filter(mask & ~(s.left | s.down | s.right), s.row, s.down, confs[s.conf]);
      while (bm) {
        const uint32_t bit = bm & (0u - bm);
        bm ^= bit;
        UTask t = s;
        t.board[s.row] = bit;
        t.left = (s.left | bit) << 1; t.down = s.down | bit; t.right = (s.right | bit) >> 1; t.row = s.row + 1;
        nxt.push_back(t);
        grew = true;
      }
    }
    cur.swap(nxt);
    if (!grew) break;
  }
  // each state's candidate set; states without one are dropped (in place)
  size_t k = 0;
  for (size_t q = 0; q < cur.size(); q++) {
    UTask& t = cur[q];
    t.avail = row_filter(mask & ~(t.left | t.down | t.right), t.row, t.down, confs[t.conf]);
    if (t.avail) cur[k++] = t;
  }
  cur.resize(k);
  if (tasks.empty()) tasks.swap(cur);
  else tasks.insert(tasks.end(), cur.begin(), cur.end());
  return 0;
}

}  // namespace
}  // namespace nq

using namespace nq;

extern "C" int nq_count_unique(nq_handle* h, int N, uint64_t* unique, uint64_t* total) {
  if (!h) return NQ_EINVAL;
  if (!unique || !total) return h->fail(NQ_EINVAL, "count_unique: null output");
  if (N < 4 || N > kMaxN) return h->fail(NQ_EINVAL, "count_unique: N=%d outside 4..27", N);
  // the handle's device and stream, and buffers the handle keeps between calls
  NQ_CUDA(h, cudaSetDevice(h->device));
  const int dev = h->device, sms = h->sms;
  cudaStream_t st = h->stream;
  std::vector<UConf> confs;
  std::vector<UTask> tasks;
  // About 8 tasks per resident lane (the kernel keeps ~512 lanes per SM): fewer
  // leave a tail at N=20 (+35 % with 4 per lane), more cost host time (N=19:
  // 0.66 s with 32 per lane against 0.48 s, the same kernel time).
  build_unique_tasks(N, (int64_t)sms * 2048 * 2, confs, tasks);
  const int64_t m = (int64_t)tasks.size();
  uint32_t min_row = (uint32_t)N;
  for (const UTask& t : tasks) min_row = std::min(min_row, t.row);
  const int maxf = std::max(1, N - 2 - (int)min_row);
  constexpr int B = 128;
  const size_t smem = (size_t)B * ((size_t)maxf * sizeof(uint4) + (size_t)N * sizeof(uint32_t));
  NQ_CUDA(h, h->utasks.ensure(std::max<size_t>(1, (size_t)m * sizeof(UTask))));
  NQ_CUDA(h, h->uconfs.ensure(std::max<size_t>(1, confs.size() * sizeof(UConf))));
  NQ_CUDA(h, h->uctl.ensure(64));
  unsigned char* ctl = (unsigned char*)h->uctl.p;
  NQ_CUDA(h, cudaMemsetAsync(ctl, 0, 64, st));
  if (m > 0) NQ_CUDA(h, cudaMemcpyAsync(h->utasks.p, tasks.data(), (size_t)m * sizeof(UTask), cudaMemcpyHostToDevice, st));
  if (!confs.empty())
    NQ_CUDA(h, cudaMemcpyAsync(h->uconfs.p, confs.data(), confs.size() * sizeof(UConf), cudaMemcpyHostToDevice, st));
  if (m > 0) {
    int optin = 0;   // the cap is process-wide: set it to the device maximum, never to one launch's size
    NQ_CUDA(h, cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    NQ_CUDA(h, cudaFuncSetAttribute(unique_kernel<B>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin));
    int per = 0;
    NQ_CUDA(h, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, unique_kernel<B>, B, smem));
    if (per <= 0) return h->fail(NQ_ECUDA, "count_unique: N=%d does not fit on an SM", N);
    UArgs a;
    a.tasks = (const UTask*)h->utasks.p; a.confs = (const UConf*)h->uconfs.p; a.m = m; a.N = N; a.maxf = maxf;
    a.counts = (unsigned long long*)ctl; a.cursor = (unsigned int*)(ctl + 32);
    a.err = (unsigned int*)(ctl + 36);
    unique_kernel<B><<<sms * per, B, smem, st>>>(a);
    NQ_CUDA(h, cudaGetLastError());
  }
  // the host task vectors stay alive until the stream has consumed them (synchronised below)
  if (int s = h->ensure_pinned(64)) return s;
  NQ_CUDA(h, cudaMemcpyAsync(h->h_ctrl, ctl, 64, cudaMemcpyDeviceToHost, st));
  NQ_CUDA(h, cudaStreamSynchronize(st));
  const unsigned long long* hc = (const unsigned long long*)h->h_ctrl;
  const uint32_t herr = ((const uint32_t*)h->h_ctrl)[9];
  if (herr) return h->fail(NQ_EINVAL, "count_unique: device error word %u", herr);
  *unique = hc[0] + hc[1] + hc[2];
  *total = 2 * hc[0] + 4 * hc[1] + 8 * hc[2];
  return NQ_OK;
}
