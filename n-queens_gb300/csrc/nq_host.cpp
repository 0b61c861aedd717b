// nq_host.cpp -- host-side task builders of the native library.
//
// 1. gen_constellations: start constellations with their x2/x4/x8 classes and
//    their preset-queen expansion (14Bit_codon_GPU/356Py_savesp_narrow.py:
//    2714-2926).  The start-constellation set is built sequentially (the
//    rotation check depends on insertion order, 356Py:2850-2880); the preset
//    expansion of each start constellation is independent (its subconst
//    cache and signature set are cleared per constellation, 356Py:2886-2889)
//    and runs on all host threads.  Output order: ascending packed ijkl, then
//    the reference's expansion order within a constellation.
// 2. build_completion_tasks: DFS tasks for boards with pre-placed queens (no
//    reference counterpart: the reference only counts whole boards).  Rows
//    holding a pre-placed queen are skipped with a multi-row step, and the
//    queens' diagonals are carried in ld/rd from the root or injected when
//    they enter the bitboard, as the reference does for its corner queens
//    (blockK/blockL, 356Py:2586-2589).  The first free rows are expanded on
//    the host until there are enough tasks to fill the GPU.
#include <algorithm>
#include <atomic>
#include <cstring>
#include <thread>
#include <vector>

#include "nq_common.cuh"
#include "nq_host.h"

namespace nq {

// ---------------------------------------------------------------------------
// generator
// ---------------------------------------------------------------------------
namespace {

inline int to_ijkl(int i, int j, int k, int l) { return (i << 15) + (j << 10) + (k << 5) + l; }
inline int rot90h(int x, int N) { return ((N - 1 - getk(x)) << 15) + ((N - 1 - getl(x)) << 10) + (getj(x) << 5) + geti(x); }
inline int canon(int x, int N) {   // jasmin, 356Py:2739-2756
  auto dist = [N](int v) { return std::min(v, N - 1 - v); };
  int arg = 0, mn = dist(getj(x));
  if (dist(geti(x)) < mn) { arg = 2; mn = dist(geti(x)); }
  if (dist(getk(x)) < mn) { arg = 3; mn = dist(getk(x)); }
  if (dist(getl(x)) < mn) { arg = 1; mn = dist(getl(x)); }
  for (int a = 0; a < arg; a++) x = rot90h(x, N);
  if (getj(x) < N - 1 - getj(x)) x = to_ijkl(N - 1 - geti(x), N - 1 - getj(x), getl(x), getk(x));
  return x;
}

inline uint64_t hmix(uint64_t x) {
  x ^= x >> 31; x *= 0x7fb5d329728ea185ULL; x ^= x >> 27; x *= 0x81dadef4bc2dd44dULL; x ^= x >> 33;
  return x;
}

// Open-addressing set of fixed-width keys with O(1) clear (generation stamps).
template <int W>
struct KeySet {
  std::vector<uint64_t> keys;
  std::vector<uint32_t> stamp;
  uint32_t gen = 1;
  size_t count = 0, mask = 0;
  KeySet() { resize(1 << 12); }
  void resize(size_t cap) {
    std::vector<uint64_t> ok;
    std::vector<uint32_t> os;
    ok.swap(keys); os.swap(stamp);
    keys.assign(cap * W, 0); stamp.assign(cap, 0); mask = cap - 1; count = 0;
    for (size_t s = 0; s < os.size(); s++)
      if (os[s] == gen) insert(&ok[s * W]);
  }
  void clear() { gen++; count = 0; if (gen == 0) { std::fill(stamp.begin(), stamp.end(), 0); gen = 1; } }
  // true when the key was absent (and is now present)
  bool insert(const uint64_t* k) {
    if ((count + 1) * 2 > stamp.size()) resize(stamp.size() * 2);
    uint64_t h = 0x243f6a8885a308d3ULL;
    for (int w = 0; w < W; w++) h = hmix(h ^ k[w]);
    size_t p = h & mask;
    while (stamp[p] == gen) {
      if (std::memcmp(&keys[p * W], k, W * sizeof(uint64_t)) == 0) return false;
      p = (p + 1) & mask;
    }
    std::memcpy(&keys[p * W], k, W * sizeof(uint64_t));
    stamp[p] = gen; count++;
    return true;
  }
};

struct Expander {
  int N, preset, k, l;
  uint64_t board_mask;
  KeySet<6> cache;     // (ld, rd, col, LD, RD, row | queens<<8)
  KeySet<4> sigs;      // (ld, rd, col, row)
  std::vector<GenRecord>* out;
  uint32_t base;
  int err = 0;

  void cached(uint64_t ld, uint64_t rd, uint64_t col, int row, int queens, uint64_t LD, uint64_t RD) {
    if (err) return;
    if (preset < 7) {   // set_pre_queens_cached bypasses its cache for preset >= 7 (356Py:2773-2784)
      const uint64_t key[6] = {ld, rd, col, LD, RD, (uint64_t)row | ((uint64_t)queens << 8)};
      if (!cache.insert(key)) return;
    }
    expand(ld, rd, col, row, queens, LD, RD);
  }
  void expand(uint64_t ld, uint64_t rd, uint64_t col, int row, int queens, uint64_t LD, uint64_t RD) {
    if (row == k || row == l) { cached(ld << 1, rd >> 1, col, row + 1, queens, LD, RD); return; }
    if (queens == preset) {
      if (preset <= 5) {  // signature prune only up to preset 5 (356Py:2820-2824)
        const uint64_t s[4] = {ld, rd, col, (uint64_t)row};
        if (!sigs.insert(s)) return;
      }
      out->push_back(GenRecord{ld, rd, col, ((uint32_t)row << 20) | base});
      return;
    }
    const int sh = N - 1 - row;
    if (sh < 0) { err = 1; return; }   // the reference raises on a negative shift here
    uint64_t fr = ~(ld | rd | col | (LD >> sh) | (RD << sh)) & board_mask;
    while (fr) {
      const uint64_t bit = fr & (0 - fr);
      fr &= fr - 1;
      cached((ld | bit) << 1, (rd | bit) >> 1, col | bit, row + 1, queens + 1, LD, RD);
      if (err) return;
    }
  }
};

bool rotated_present(const std::vector<uint8_t>& S, int i, int j, int k, int l, int N) {
  const int r1 = ((N - 1 - k) << 15) + ((N - 1 - l) << 10) + (j << 5) + i;
  const int r2 = ((N - 1 - j) << 15) + ((N - 1 - i) << 10) + ((N - 1 - l) << 5) + (N - 1 - k);
  const int r3 = (l << 15) + (k << 10) + ((N - 1 - i) << 5) + (N - 1 - j);
  return S[r1] || S[r2] || S[r3];
}

}  // namespace

int start_constellations(int N, std::vector<int>& starts) {
  starts.clear();
  if (N < 5 || N > kMaxN) return -1;
  const int halfN = (N + 1) / 2, N1 = N - 1, N2 = N - 2;
  // S: the set of start constellations (random access for the rotation check),
  // with its members also listed so nothing scans all 2^20 packed ijkl values.
  std::vector<uint8_t> S(1u << 20, 0);
  std::vector<int> members;
  auto add = [&](int x) { if (!S[x]) { S[x] = 1; members.push_back(x); } };
  if (N % 2 == 1) {   // centre column of odd boards (356Py:2857-2867)
    const int c = N / 2;
    for (int l = c + 1; l < N1; l++)
      for (int i = c + 1; i < N1; i++) {
        if (i == N1 - l) continue;
        for (int j = N - c - 2; j > 0; j--)
          if (j != i && j != l && !rotated_present(S, i, j, c, l, N)) add(to_ijkl(i, j, c, l));
      }
  }
  for (int k = 1; k < halfN; k++)   // no queen in a corner (356Py:2869-2878)
    for (int l = k + 1; l < N1; l++)
      for (int i = k + 1; i < N1; i++) {
        if (i == N1 - l) continue;
        for (int j = N - k - 2; j > 0; j--)
          if (j != i && j != l && !rotated_present(S, i, j, k, l, N)) add(to_ijkl(i, j, k, l));
      }
  for (int j = 1; j < N2; j++)      // queen in a corner (356Py:2880)
    for (int l = j + 1; l < N1; l++) add(to_ijkl(0, j, 0, l));
  // canonical forms (jasmin), distinct, in ascending packed order
  starts.reserve(members.size());
  for (int x : members) starts.push_back(canon(x, N));
  std::sort(starts.begin(), starts.end());
  starts.erase(std::unique(starts.begin(), starts.end()), starts.end());
  return 0;
}

int expand_starts(int N, int preset, const std::vector<int>& starts, size_t s0, size_t s1,
                  std::vector<GenRecord>& out, int threads) {
  if (N < 5 || N > kMaxN || preset < 1) return -1;
  if (preset < 4) return -2;   // the start constellations already hold 3-4 queens; the reference presets are 4..8
  const int N1 = N - 1;
  s1 = std::min(s1, starts.size());
  if (s0 >= s1) return 0;
  const size_t ns = s1 - s0;
  std::vector<std::vector<GenRecord>> parts(ns);
  std::atomic<size_t> next{0};
  std::atomic<int> err{0};
  auto worker = [&]() {
    Expander e;
    e.N = N; e.preset = preset; e.board_mask = (1ull << N) - 1;
    for (;;) {
      const size_t q = next.fetch_add(1);
      if (q >= ns) break;
      const int sc = starts[s0 + q];
      const int i = geti(sc), j = getj(sc), k = getk(sc), l = getl(sc);
      if (l < 1) { err = 1; break; }
      const uint64_t L = 1ull << N1, Lj = L >> j, Li = L >> i, Ll = L >> l;
      const uint64_t ld = ((i > 0) ? (L >> (i - 1)) : 0) | (1ull << (N - k));
      const uint64_t rd = (L >> (i + 1)) | (1ull << (l - 1));
      const uint64_t col = 1 | L | Li | Lj;
      e.cache.clear(); e.sigs.clear();
      e.k = k; e.l = l; e.out = &parts[q]; e.base = (uint32_t)to_ijkl(i, j, k, l);
      e.cached(ld, rd, col, 1, (j == N1) ? 3 : 4, Lj | Ll, Lj | (1ull << k));
      if (e.err) { err = 1; break; }
    }
  };
  if (threads <= 0) threads = (int)std::max(1u, std::thread::hardware_concurrency());
  threads = (int)std::min<size_t>((size_t)threads, std::max<size_t>(1, ns / 8));
  if (threads <= 1) worker();
  else {
    std::vector<std::thread> th;
    for (int t = 0; t < threads; t++) th.emplace_back(worker);
    for (auto& t : th) t.join();
  }
  if (err) return -2;
  size_t total = out.size();
  for (auto& p : parts) total += p.size();
  out.reserve(total);
  for (auto& p : parts) out.insert(out.end(), p.begin(), p.end());
  return 0;
}

int gen_constellations(int N, int preset, std::vector<GenRecord>& out, int threads) {
  out.clear();
  if (N < 5 || N > kMaxN || preset < 1) return -1;
  if (preset < 4) return -2;
  std::vector<int> starts;
  if (int s = start_constellations(N, starts)) return s;
  return expand_starts(N, preset, starts, 0, starts.size(), out, threads);
}

// ---------------------------------------------------------------------------
// completion queries
// ---------------------------------------------------------------------------
int build_completion_tasks(int N, int k, const int* rows, const int* cols, int min_tasks, uint32_t job,
                           std::vector<HostTask>& out, int* max_T) {
  if (N < 1 || N > kMaxN || k < 0 || k > N) return -1;
  int fixed_col[32];
  for (int r = 0; r < N; r++) fixed_col[r] = -1;
  for (int q = 0; q < k; q++) {
    if (rows[q] < 0 || rows[q] >= N || cols[q] < 0 || cols[q] >= N) return -1;
    if (fixed_col[rows[q]] >= 0) return (fixed_col[rows[q]] == cols[q]) ? -1 : 1;
    fixed_col[rows[q]] = cols[q];
  }
  for (int a = 0; a < k; a++)       // attacking pre-placed queens: no completion
    for (int b = a + 1; b < k; b++) {
      const int dr = rows[a] - rows[b], dc = cols[a] - cols[b];
      if (cols[a] == cols[b] || dr == dc || dr == -dc) return 1;
    }
  int F[32], n = 0;
  for (int r = 0; r < N; r++)
    if (fixed_col[r] < 0) F[n++] = r;
  if (n == 0) return 2;   // every row holds a pre-placed queen and none attack: exactly one placement
  const uint32_t bm = (N >= 32) ? 0xFFFFFFFFu : ((1u << N) - 1u);
  // root frame at row F[0]
  uint32_t ld = 0, rd = 0, col = 0;
  Op ops[kMaxDepth + 1];
  if (n > kMaxDepth) return -1;
  for (int d = 0; d < n; d++) ops[d] = Op{1, 0, 0, 0, 0, 0};
  for (int q = 0; q < k; q++) {
    const int r = rows[q], c = cols[q];
    col |= 1u << c;
    // diagonal c - r + x (ld, moves up one bit per row)
    const int lpos = c - r + F[0];
    if (lpos >= 0) { if (lpos < 32) ld |= 1u << lpos; }
    else {
      const int enter = r - c;   // row where the diagonal reaches bit 0
      for (int d = 0; d + 1 < n; d++)
        if (F[d] < enter && enter <= F[d + 1]) { ops[d].la |= 1u << (F[d + 1] - enter); break; }
    }
    // anti-diagonal c + r - x (rd, moves down one bit per row)
    const int rpos = c + r - F[0];
    if (rpos >= 0 && rpos < 32) rd |= 1u << rpos;
    else if (rpos >= 32) {
      for (int d = 0; d + 1 < n; d++) {
        const int p = c + r - F[d + 1];
        if (p < 32) { if (p >= 0) ops[d].ra |= 1u << p; break; }
      }
    }
  }
  for (int d = 0; d + 1 < n; d++) ops[d].s = (uint32_t)(F[d + 1] - F[d]);
  ops[n - 1].term = 1; ops[n - 1].tall = 1;
  const int T = n - 1;
  extend_lookahead(ops, T);
  for (int d = 0; d < n; d++)
    if (!wide_fits(ops[d])) return -1;

  // Expand the first levels breadth-first until there are enough tasks.
  struct F4 { uint32_t ld, rd, col, avail; };
  std::vector<F4> cur{F4{ld, rd, col, bm & ~(ld | rd | col)}}, nxt;
  int depth = 0;
  while (depth < T && (int)cur.size() < min_tasks) {
    nxt.clear();
    const Op& o = ops[depth];
    for (const F4& f : cur) {
      uint32_t av = f.avail;
      while (av) {
        const uint32_t bit = av & (0u - av);
        av ^= bit;
        const uint32_t nl = ((f.ld | bit) << o.s) | o.la, nr = ((f.rd | bit) >> o.s) | o.ra, nc = f.col | bit;
        const uint32_t nf = bm & ~(nl | nr | nc);
        if (nf) nxt.push_back(F4{nl, nr, nc, nf});
      }
    }
    cur.swap(nxt);
    depth++;
    if (cur.empty()) break;
  }
  const int Tt = T - depth;
  if (max_T && Tt > *max_T) *max_T = Tt;
  for (const F4& f : cur) {
    if (f.avail == 0) continue;
    HostTask h;
    h.root[0] = f.ld; h.root[1] = f.rd; h.root[2] = f.col; h.root[3] = f.avail;
    h.info = info_pack((uint32_t)Tt, 0, 0, (uint32_t)N, TS_OK);
    h.job = job;
    h.T = Tt;
    for (int d = 0; d <= Tt; d++) { h.sched[2 * d] = pack_wide_x(ops[depth + d]); h.sched[2 * d + 1] = ops[depth + d].ra; }
    out.push_back(h);
  }
  return 0;
}

int64_t start_row_min(const uint32_t* startijkl, int64_t m, int stride_words) {
  int64_t mn = 64;
  for (int64_t i = 0; i < m; i++) {
    const int64_t s = (int64_t)(startijkl[i * stride_words] >> 20);
    if (s < mn) mn = s;
  }
  return mn;
}

}  // namespace nq
