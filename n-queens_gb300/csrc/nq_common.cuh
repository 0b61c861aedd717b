// nq_common.cuh -- task decoding and per-depth schedules shared by the host
// library code and the sm_103a kernels.
//
// A constellation record {ld, rd, col, startijkl} (the reference's 16-byte
// task record, 14Bit_codon_GPU/356Py_savesp_narrow.py:2981-2986) becomes one
// DFS task.  The reference walks an SQ* state machine (func_meta,
// 356Py:2255-2284) inside its DFS; because a task's rows advance
// deterministically, the SQ* function in force at each depth depends only on
// the depth (the reference's kernel exploits the same fact, 356Py:689-756).
// This file turns that state machine into a per-depth schedule of words once
// per task, so the DFS inner loop is the same branch-free step for every
// SQ* variant: no per-node function-id dispatch and no divergence on it.
//
// Per-depth op of a frame at depth d producing a child at depth d+1:
//   nld  = ((ld | bit) << s) | LA        (LA: queens of skipped rows, jmark)
//   nrd  = ((rd | bit) >> s) | RA        (RA: blockK of 356Py:2586-2589)
//   ncol = col | bit
//   nf   = bm & ~(nld | nrd | ncol)
//   FC:   drop the child when bm & ~((nld<<1)|(nrd>>1)|ncol) == 0 (look-ahead,
//         356Py:1935-1965; see extend_lookahead for where it applies)
//   TERM: the child is a base frame (356Py:1855-1860): count it instead of
//         descending (for SQd2B, whose base counts only when a square other
//         than column 0 is free, the word's LA carries bit 0);
//         TALL: count every candidate (completion queries, last free row)
//
// Compact word (4 B, constellation tasks), laid out so the DFS forms the
// child masks with two funnel shifts and no field extraction:
//   bits 0-4     s (1..3): the count of both shifts (a funnel shift reads
//                only the low 5 bits of its count)
//   RA << s      at its own position, bits N-1..N: or-ed into rd | bit before
//                the right shift, ((rd | bit) | RA << s) >> s = nrd
//   bit 28       FC
//   top s bits   LA: shf.l(lo = w, hi = x, n = w) = (x << s) | (w >> (32 - s))
//                = (x << s) | LA
// TERM is not stored: it is the task's terminal depth T (info word); TALL
// never occurs in constellation tasks.  compact_fits() checks the fields do
// not overlap (la < 2^s, RA << s within bits N-1..N).
// Wide word (8 B, mixed batches and completion queries), the same funnel-shift
// layout for nld with RA in a word of its own (any bits):
//   x: bits 0-4 s | 5 FC | 6 TERM | 7 TALL | top s bits LA (la < 2^s);  y: RA
#pragma once
#include <stdint.h>

#ifdef __CUDACC__
#define NQ_HD __host__ __device__ __forceinline__
#else
#define NQ_HD inline
#endif

namespace nq {

constexpr int kMaxN = 27;        // columns in bits 0-26, a frame's depth in bits 27-31; u64 totals
constexpr int kMaxDepth = 28;    // schedule words per task (depths 0..T)

// compact word fields
constexpr uint32_t C_S = 0x1Fu;
constexpr uint32_t C_FC = 1u << 28;
NQ_HD uint32_t compact_ra_mask(int N) { return 3u << (N - 1); }   // where RA << s may sit
// wide word fields (x)
constexpr uint32_t W_S = 0x1Fu;
constexpr uint32_t W_FC = 1u << 5;
constexpr uint32_t W_TERM = 1u << 6;
constexpr uint32_t W_TALL = 1u << 7;

// Known whole-board totals (the reference's known-answer table,
// 356Py_savesp_narrow.py:5775), index N.  Used only as an upper bound when
// sizing counters, never as a result.
NQ_HD uint64_t known_total(int N) {
  constexpr uint64_t t[28] = {1ull, 1ull, 0ull, 0ull, 2ull, 10ull, 4ull, 40ull, 92ull, 352ull, 724ull, 2680ull, 14200ull,
                              73712ull, 365596ull, 2279184ull, 14772512ull, 95815104ull, 666090624ull, 4968057848ull,
                              39029188884ull, 314666222712ull, 2691008701644ull, 24233937684440ull,
                              227514171973736ull, 2207893435808352ull, 22317699616364044ull, 234907967154122528ull};
  return (N >= 0 && N <= 27) ? t[N] : ~0ull;
}

// Per-lane counts of the DFS are u32 unless a queue item could count 2^32
// solutions.  An item's share of the board total, measured with the oracle at
// N=14..17 and presets 4-5, is at most ~2.2x the average (total / 2 / items);
// a factor of 32 on the average leaves ~15x margin.
inline bool counts_need_u64(int N, int64_t items) {
  const double avg = (double)known_total(N) / (double)(items > 0 ? items : 1);
  return avg * 32.0 >= 4294967296.0;
}

// Task info word: T (terminal depth, 0..31) | wexp<<5 | root_count<<7 | N<<8 |
// status<<13.  T == 31 marks a task with no DFS work (root handled in prepare).
constexpr uint32_t INFO_NO_DFS = 31u;
NQ_HD uint32_t info_pack(uint32_t T, uint32_t wexp, uint32_t root_count, uint32_t N, uint32_t status) {
  return (T & 31u) | ((wexp & 3u) << 5) | ((root_count & 1u) << 7) | ((N & 31u) << 8) | ((status & 7u) << 13);
}
NQ_HD uint32_t info_T(uint32_t x) { return x & 31u; }
NQ_HD uint32_t info_wexp(uint32_t x) { return (x >> 5) & 3u; }
NQ_HD uint32_t info_root(uint32_t x) { return (x >> 7) & 1u; }
NQ_HD uint32_t info_N(uint32_t x) { return (x >> 8) & 31u; }
NQ_HD uint32_t info_status(uint32_t x) { return (x >> 13) & 7u; }
// task status codes stored in the info word
constexpr uint32_t TS_OK = 0, TS_BAD_SHIFT = 1, TS_DEPTH = 2, TS_NOTERM = 3, TS_BADN = 4, TS_FORMAT = 5;

// ---------------------------------------------------------------------------
// SQ* state machine tables (356Py:2236-2289, 2586-2589).
// ptn: 0,1,2 = mark patterns (step 2 at mark1 / step 2 at mark2 / step 3 at
// mark1), 3 = jmark, 4 = P5, 5 = base.  av = look-ahead flag.  cat selects
// blockK (3 -> 1<<(N-3), 4 -> 1<<(N-4)).  bl = blockL.
// ---------------------------------------------------------------------------
// Each fid packs as next | ptn<<5 | av<<8 | cat<<9 | bl<<12; a switch keeps
// the table out of memory on both host and device.
struct FidRow { uint32_t next, ptn, av, cat, bl; };
NQ_HD uint32_t fid_code(int f) {
  switch (f) {
    case 0: return 0x0601u;  case 1: return 0x1022u;  case 2: return 0x0163u;  case 3: return 0x01a3u;
    case 4: return 0x1842u;  case 5: return 0x1006u;  case 6: return 0x0622u;  case 7: return 0x2642u;
    case 8: return 0x0180u;  case 9: return 0x0184u;  case 10: return 0x0185u; case 11: return 0x0187u;
    case 12: return 0x060du; case 13: return 0x102eu; case 14: return 0x01aeu; case 15: return 0x184eu;
    case 16: return 0x1011u; case 17: return 0x062eu; case 18: return 0x264eu; case 19: return 0x0614u;
    case 20: return 0x0035u; case 21: return 0x01b5u; case 22: return 0x1855u; case 23: return 0x1019u;
    case 24: return 0x2655u; case 25: return 0x0635u; case 26: return 0x01bau; default: return 0x061au;
  }
}
NQ_HD FidRow fid_row(int f) {
  const uint32_t c = fid_code(f);
  FidRow r;
  r.next = c & 31u; r.ptn = (c >> 5) & 7u; r.av = (c >> 8) & 1u; r.cat = (c >> 9) & 7u; r.bl = (c >> 12) & 3u;
  return r;
}

// Decoded task: build_soa_for_range (356Py:1971-2169) for one record.
struct TaskHead {
  uint32_t ld, rd, col, free_;
  int fid, start, jmark, endmark, mark1, mark2, ijkl, wexp;
  uint32_t status;
};

NQ_HD int geti(int x) { return (x >> 15) & 0x1F; }
NQ_HD int getj(int x) { return (x >> 10) & 0x1F; }
NQ_HD int getk(int x) { return (x >> 5) & 0x1F; }
NQ_HD int getl(int x) { return x & 0x1F; }

// symmetry weight exponent: w = 2, 4, 8 -> 1, 2, 3 (356Py:2723-2724)
NQ_HD int weight_exp(int x, int N) {
  int r90 = ((N - 1 - getk(x)) << 15) + ((N - 1 - getl(x)) << 10) + (getj(x) << 5) + geti(x);
  if (x == r90) return 1;
  if (geti(x) == N - 1 - getj(x) && getk(x) == N - 1 - getl(x)) return 2;
  return 3;
}

// Record -> task head.  ld/rd/col are the record's low 32 bits (the .bin
// layout); only bits below N matter after the reference's >>1 and masking,
// and the rd high bit it adds is kept below bit 31 by its own gate.
NQ_HD TaskHead decode_record(int N, uint32_t rld, uint32_t rrd, uint32_t rcol, uint32_t sijkl) {
  TaskHead t;
  const uint64_t bm = (1ull << N) - 1;
  const uint64_t small = (1ull << (N - 2)) - 1;
  const int N1 = N - 1, N2 = N - 2;
  int jmark = 0, mark1 = 0, mark2 = 0, endmark = 0, target = 0;
  const int start = (int)(sijkl >> 20);
  const int ijkl = (int)(sijkl & 0xFFFFFu);
  const int j = getj(ijkl), k = getk(ijkl), l = getl(ijkl);
  t.status = TS_OK;
  uint64_t ld = (uint64_t)(rld >> 1), rd = (uint64_t)(rrd >> 1);
  uint64_t col = (((uint64_t)(rcol >> 1)) | ~small) & bm;
  const uint64_t LD = (1ull << (N1 - j)) | (1ull << (N1 - l));
  if (start > N || start < 0) { t.status = TS_BAD_SHIFT; }
  else ld |= LD >> (N - start);
  if (start > k) {
    const int sh = N1 - (start - k + 1);
    if (sh < 0) t.status = TS_BAD_SHIFT; else rd |= 1ull << sh;
  }
  if (j >= 2 * N - 33 - start) {
    if (N2 - start < 0) t.status = TS_BAD_SHIFT;
    else rd |= (1ull << (N1 - j)) << (N2 - start);
  }
  const uint64_t fr = bm & ~(ld | rd | col);
  const bool k_lt_l = k < l, s_lt_k = start < k, s_lt_l = start < l;
  const bool l_eq_kp1 = l == k + 1, k_eq_lp1 = k == l + 1;
  const bool j_gate = j > 2 * N - 34 - start;
  if (j < N - 3) {
    jmark = j + 1; endmark = N2;
    if (j_gate) {
      if (k_lt_l) { mark1 = k - 1; mark2 = l - 1; target = s_lt_l ? (s_lt_k ? (l_eq_kp1 ? 4 : 0) : 1) : 2; }
      else { mark1 = l - 1; mark2 = k - 1; target = s_lt_k ? (s_lt_l ? (k_eq_lp1 ? 7 : 5) : 6) : 2; }
    } else {
      if (k_lt_l) { mark1 = k - 1; mark2 = l - 1; target = l_eq_kp1 ? 9 : 8; }
      else { mark1 = l - 1; mark2 = k - 1; target = k_eq_lp1 ? 11 : 10; }
    }
  } else if (j == N - 3) {
    endmark = N2;
    if (k_lt_l) { mark1 = k - 1; mark2 = l - 1; target = s_lt_l ? (s_lt_k ? (l_eq_kp1 ? 15 : 12) : 13) : 14; }
    else { mark1 = l - 1; mark2 = k - 1; target = s_lt_k ? (s_lt_l ? (k_eq_lp1 ? 18 : 16) : 17) : 14; }
  } else if (j == N - 2) {
    if (k_lt_l) {
      endmark = N2;
      if (s_lt_l) {
        if (s_lt_k) { mark1 = k - 1; if (!l_eq_kp1) { mark2 = l - 1; target = 19; } else target = 22; }
        else { mark2 = l - 1; target = 20; }           // mark1 stays 0 (356Py:2109-2111)
      } else target = 21;
    } else {
      if (s_lt_k) {
        if (s_lt_l) {
          if (k < N2) { mark1 = l - 1; endmark = N2; if (!k_eq_lp1) { mark2 = k - 1; target = 23; } else target = 24; }
          else if (l != N - 3) { mark2 = l - 1; endmark = N - 3; target = 20; }
          else { endmark = N - 4; target = 21; }
        } else {
          if (k != N2) { mark2 = k - 1; endmark = N2; target = 25; }
          else { endmark = N - 3; target = 21; }
        }
      } else { endmark = N2; target = 21; }
    }
  } else {
    endmark = N2;
    if (start > k) target = 26; else { mark1 = k - 1; target = 27; }
  }
  t.ld = (uint32_t)ld; t.rd = (uint32_t)rd; t.col = (uint32_t)col; t.free_ = (uint32_t)fr;
  t.fid = target; t.start = start; t.jmark = jmark; t.endmark = endmark; t.mark1 = mark1; t.mark2 = mark2;
  t.ijkl = ijkl; t.wexp = weight_exp(ijkl, N);
  return t;
}

// One schedule entry before packing.
struct Op { uint32_t s, la, ra, fc, term, tall; };

// Look-ahead wherever it is sound, not only where the reference applies it
// (fr.av == 1 frames).  A word's look-ahead prunes the child frame when the
// row after the child has no square free of the child's ld << 1, rd >> 1 and
// col.  If the child's own step is a single row (s == 1) that set contains
// every grandchild's free set, whatever square the child takes and whatever
// the child's word adds through la/ra, so an empty set means every child
// candidate dies (or, at a terminal parent, counts nothing): pruning there
// changes no count.  A tall terminal counts its candidates without looking
// at a further row, so a child with a tall word is never pruned.
NQ_HD void extend_lookahead(Op* ops, int T) {
  for (int d = 0; d < T; d++)
    if (ops[d + 1].s == 1 && !ops[d + 1].tall) ops[d].fc = 1;
}

// Walk the SQ* state machine from the task's root frame and emit one Op per
// depth 0..T (dfs_iter, 356Py:1846-1965, with rows advancing by the op's
// step).  Root adjustments (the root frame's own jmark, 356Py:1889-1897, or
// a root that is already a base frame) are applied to *root / *root_count.
// Returns T (terminal-parent depth), -1 when the root itself is terminal or
// empty, or -2 on a schedule longer than max_depth / without a terminal.
struct Root { uint32_t ld, rd, col, avail; };

NQ_HD int walk_schedule(int N, const TaskHead& t, Root* root, uint32_t* root_count, Op* ops, int max_depth) {
  const uint32_t n3 = 1u << (N - 3), n4 = 1u << (N - 4);
  root->ld = t.ld; root->rd = t.rd; root->col = t.col; root->avail = t.free_;
  *root_count = 0;
  if (root->avail == 0) return -1;                       // dfs_iter: `if not free: continue`
  int fid = t.fid, row = t.start;
  for (int d = 0;; d++) {
    FidRow fr = fid_row(fid);
    if (fr.ptn == 4 && row == t.mark1) { fid = fr.next; fr = fid_row(fid); }   // P5: re-push with next fid
    if (fr.ptn == 5 && row == t.endmark) {                                      // base frame
      if (d == 0) {
        *root_count = (fid == 14) ? ((root->avail >> 1) ? 1u : 0u) : 1u;
        return -1;
      }
      ops[d - 1].term = 1;
      // The terminal-parent frame never descends, so its LA bits only feed the
      // child row's free set: LA bit 0 there removes column 0, which is the
      // SQd2B base rule "count only if a square other than column 0 is free"
      // (356Py:1855-1860).
      if (fid == 14) ops[d - 1].la |= 1u;
      extend_lookahead(ops, d - 1);
      return d - 1;
    }
    if (d >= max_depth || row > 31) return -2;
    Op op = {1, 0, 0, 0, 0, 0};
    int nfid = fid;
    bool at_mark = false;
    if (fr.ptn <= 2) at_mark = (fr.ptn == 1) ? (row == t.mark2) : (row == t.mark1);
    if (at_mark) {
      op.s = (fr.ptn == 2) ? 3u : 2u;
      op.la = ((fr.ptn == 1 && fid == 20) ? 1u : 0u) | fr.bl;
      op.ra = fr.cat == 3 ? n3 : (fr.cat == 4 ? n4 : 0u);
      nfid = fr.next;
    } else {
      if (fr.ptn == 3 && row == t.jmark) {
        // this frame is a jmark frame: column 0 is forbidden in it and ld gets bit 0.
        // Both happen when the frame is created: fold into the parent's LA.
        if (d == 0) { root->avail &= ~1u; root->ld |= 1u; if (root->avail == 0) return -1; }
        else ops[d - 1].la |= 1u;
        nfid = fr.next;
      }
      op.fc = (fr.av == 1 && row + 1 < t.endmark) ? 1u : 0u;
    }
    ops[d] = op;
    fid = nfid;
    row += (int)op.s;
  }
}

// True when the op packs into a compact word without overlapping fields.
NQ_HD bool compact_fits(const Op& o, int N) {
  if (o.s < 1 || o.s > 3 || o.tall || o.la >= (1u << o.s)) return false;
  const uint64_t ra = (uint64_t)o.ra << o.s;
  return (ra & ~(uint64_t)compact_ra_mask(N)) == 0;
}
NQ_HD uint32_t pack_compact(const Op& o) {
  return o.s | (o.ra << o.s) | (o.fc ? C_FC : 0u) | (o.s ? (o.la << (32 - o.s)) : 0u);
}
// The op of a compact word (split kernel and host checks); `term`: the word's depth is T.
NQ_HD Op unpack_compact(uint32_t w, int N, bool term) {
  Op o;
  o.s = w & C_S;
  o.la = w >> (32 - o.s);
  o.ra = (w & compact_ra_mask(N)) >> o.s;
  o.fc = (w & C_FC) ? 1u : 0u;
  o.term = term ? 1u : 0u;
  o.tall = 0;
  return o;
}
// True when the op packs into a wide word: LA in the top s bits clear of the flags (s <= 24).
NQ_HD bool wide_fits(const Op& o) { return o.s <= 24 && (uint64_t)o.la < (1ull << o.s); }
NQ_HD uint32_t pack_wide_x(const Op& o) {
  return o.s | (o.fc ? W_FC : 0u) | (o.term ? W_TERM : 0u) | (o.tall ? W_TALL : 0u) |
         (o.s ? (o.la << (32 - o.s)) : 0u);
}

}  // namespace nq
