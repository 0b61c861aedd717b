/*
 * nq_oracle.c -- CPU restatement of the reference N-Queens constellation solver.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker: it is compiled into
 * oracle/_build/libnqoracle.so and may be loaded only by tests/, by
 * __graft_entry__.smoke() and by bench.py's cpu_baseline / --impl reference
 * legs.  The product library (n-queens_gb300/csrc) never links or calls it.
 *
 * Every function restates one reference function of suzukiiichiro/N-Queens
 * (paths relative to that project):
 *
 *   ijkl algebra, symmetry ...... 14Bit_codon_GPU/356Py_savesp_narrow.py:2714-2727
 *   jasmin ...................... 356Py_savesp_narrow.py:2739-2756
 *   set_pre_queens(_cached) ..... 356Py_savesp_narrow.py:2758-2835
 *   gen_constellations .......... 356Py_savesp_narrow.py:2837-2926
 *   select_dynamic_preset_queens  356Py_savesp_narrow.py:5744-5753
 *   build_soa_for_range ......... 356Py_savesp_narrow.py:1971-2169
 *   func_meta / blockK / blockL . 356Py_savesp_narrow.py:2236-2289,2586-2589
 *   dfs_iter .................... 356Py_savesp_narrow.py:1837-1967 (plus a node counter)
 *   exec_solutions (CPU branch) . 356Py_savesp_narrow.py:2579-2610
 *   _bit_total .................. 356Py_savesp_narrow.py:5755-5767
 *   unique (symmetry method) .... 11Bit_Python/07Py_bit_symmetry.py:65-200
 *
 * Parity is pinned: the generator reproduces 13Bit_codon/Archive/bin/
 * constellations_N{6..21}_5.bin and the solver reproduces
 * solutions_N{6..19}_5_v2.bin record for record (tests/golden holds digests
 * of those files plus vectors produced by running the reference's own Python
 * host functions under CPython; see tests/golden/make_golden.py).
 *
 * A "node" is one candidate-queen extraction `bit = avail & -avail` of
 * dfs_iter; orc_exec_solutions can report nodes per task.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <pthread.h>

#define ORC_OK 0
#define ORC_EINVAL (-1)
#define ORC_ENOMEM (-5)

/* ------------------------------------------------------------------ */
/* ijkl algebra: 356Py:2714-2727                                       */
/* ------------------------------------------------------------------ */
static inline int to_ijkl(int i, int j, int k, int l) { return (i << 15) + (j << 10) + (k << 5) + l; }
static inline int geti(int x) { return (x >> 15) & 0x1F; }
static inline int getj(int x) { return (x >> 10) & 0x1F; }
static inline int getk(int x) { return (x >> 5) & 0x1F; }
static inline int getl(int x) { return x & 0x1F; }
static inline int ffmin(int a, int b) { return a < b ? a : b; }
static inline int rot90(int x, int N) {
  return ((N - 1 - getk(x)) << 15) + ((N - 1 - getl(x)) << 10) + (getj(x) << 5) + geti(x);
}
static inline int mirvert(int x, int N) { return to_ijkl(N - 1 - geti(x), N - 1 - getj(x), getl(x), getk(x)); }
static inline int symmetry90(int x, int N) { return x == rot90(x, N); }
/* symmetry(): weight 2 / 4 / 8 (356Py:2723) */
int orc_symmetry(int x, int N) {
  if (symmetry90(x, N)) return 2;
  if (geti(x) == N - 1 - getj(x) && getk(x) == N - 1 - getl(x)) return 4;
  return 8;
}

/* jasmin(): canonical orientation (356Py:2739-2756) */
int orc_jasmin(int x, int N) {
  int arg = 0;
  int mn = ffmin(getj(x), N - 1 - getj(x));
  if (ffmin(geti(x), N - 1 - geti(x)) < mn) { arg = 2; mn = ffmin(geti(x), N - 1 - geti(x)); }
  if (ffmin(getk(x), N - 1 - getk(x)) < mn) { arg = 3; mn = ffmin(getk(x), N - 1 - getk(x)); }
  if (ffmin(getl(x), N - 1 - getl(x)) < mn) { arg = 1; mn = ffmin(getl(x), N - 1 - getl(x)); }
  for (int a = 0; a < arg; a++) x = rot90(x, N);
  if (getj(x) < N - 1 - getj(x)) x = mirvert(x, N);
  return x;
}

/* select_dynamic_preset_queens (356Py:5744-5753) */
int orc_preset_for(int N, int fallback) {
  if (N >= 5 && N <= 17) return 5;
  if (N >= 18 && N <= 21) return 6;
  if (N >= 22 && N <= 24) return 7;
  if (N >= 25 && N <= 27) return 8;
  return fallback;
}

/* ------------------------------------------------------------------ */
/* Generator: 356Py:2758-2926                                          */
/* ------------------------------------------------------------------ */
typedef struct { uint64_t ld, rd, col, LD, RD; int row, queens; } ckey_t;   /* k,l,N,preset fixed per sc */
typedef struct { uint64_t ld, rd, col; int row; } skey_t;

typedef struct {
  uint64_t *ld, *rd, *col; uint32_t *sijkl;
  int64_t n, cap;
} recvec_t;

typedef struct {
  /* subconst_cache: open addressing with generation stamps (cleared per sc) */
  ckey_t *ck; uint32_t *cstamp; uint64_t ccap, ccount;
  skey_t *sk; uint32_t *sstamp; uint64_t scap, scount;
  uint32_t gen;
  int N, preset, k, l;
  int64_t counter;
  int err;
  recvec_t out;
} gen_t;

static inline uint64_t mix64(uint64_t x) {
  x ^= x >> 33; x *= 0xff51afd7ed558ccdULL; x ^= x >> 33; x *= 0xc4ceb9fe1a85ec53ULL; x ^= x >> 33;
  return x;
}
static uint64_t ckey_hash(const ckey_t *k) {
  uint64_t h = mix64(k->ld + 0x9e3779b97f4a7c15ULL);
  h = mix64(h ^ k->rd); h = mix64(h ^ k->col); h = mix64(h ^ k->LD); h = mix64(h ^ k->RD);
  h = mix64(h ^ ((uint64_t)k->row << 8 | (uint64_t)k->queens));
  return h;
}
static uint64_t skey_hash(const skey_t *k) {
  uint64_t h = mix64(k->ld + 0x51ed270b27ULL);
  h = mix64(h ^ k->rd); h = mix64(h ^ k->col); h = mix64(h ^ (uint64_t)k->row);
  return h;
}

static int cache_grow(gen_t *g) {
  uint64_t ncap = g->ccap ? g->ccap * 2 : 4096;
  ckey_t *nk = (ckey_t *)malloc(ncap * sizeof(ckey_t));
  uint32_t *ns = (uint32_t *)calloc(ncap, sizeof(uint32_t));
  if (!nk || !ns) { free(nk); free(ns); return ORC_ENOMEM; }
  for (uint64_t s = 0; s < g->ccap; s++) {
    if (g->cstamp[s] != g->gen) continue;
    uint64_t p = ckey_hash(&g->ck[s]) & (ncap - 1);
    while (ns[p] == g->gen) p = (p + 1) & (ncap - 1);
    nk[p] = g->ck[s]; ns[p] = g->gen;
  }
  free(g->ck); free(g->cstamp);
  g->ck = nk; g->cstamp = ns; g->ccap = ncap;
  return ORC_OK;
}
/* returns 1 if inserted (was absent), 0 if present */
static int cache_add(gen_t *g, const ckey_t *k) {
  if ((g->ccount + 1) * 2 > g->ccap) { if (cache_grow(g)) { g->err = ORC_ENOMEM; return 0; } }
  uint64_t p = ckey_hash(k) & (g->ccap - 1);
  while (g->cstamp[p] == g->gen) {
    if (memcmp(&g->ck[p], k, sizeof(ckey_t)) == 0) return 0;
    p = (p + 1) & (g->ccap - 1);
  }
  g->ck[p] = *k; g->cstamp[p] = g->gen; g->ccount++;
  return 1;
}
static int sig_grow(gen_t *g) {
  uint64_t ncap = g->scap ? g->scap * 2 : 4096;
  skey_t *nk = (skey_t *)malloc(ncap * sizeof(skey_t));
  uint32_t *ns = (uint32_t *)calloc(ncap, sizeof(uint32_t));
  if (!nk || !ns) { free(nk); free(ns); return ORC_ENOMEM; }
  for (uint64_t s = 0; s < g->scap; s++) {
    if (g->sstamp[s] != g->gen) continue;
    uint64_t p = skey_hash(&g->sk[s]) & (ncap - 1);
    while (ns[p] == g->gen) p = (p + 1) & (ncap - 1);
    nk[p] = g->sk[s]; ns[p] = g->gen;
  }
  free(g->sk); free(g->sstamp);
  g->sk = nk; g->sstamp = ns; g->scap = ncap;
  return ORC_OK;
}
static int sig_add(gen_t *g, const skey_t *k) {
  if ((g->scount + 1) * 2 > g->scap) { if (sig_grow(g)) { g->err = ORC_ENOMEM; return 0; } }
  uint64_t p = skey_hash(k) & (g->scap - 1);
  while (g->sstamp[p] == g->gen) {
    if (memcmp(&g->sk[p], k, sizeof(skey_t)) == 0) return 0;
    p = (p + 1) & (g->scap - 1);
  }
  g->sk[p] = *k; g->sstamp[p] = g->gen; g->scount++;
  return 1;
}
static void rec_push(gen_t *g, uint64_t ld, uint64_t rd, uint64_t col, uint32_t sijkl) {
  recvec_t *v = &g->out;
  if (v->n == v->cap) {
    int64_t nc = v->cap ? v->cap * 2 : 1024;
    uint64_t *a = (uint64_t *)realloc(v->ld, nc * 8), *b, *c; uint32_t *d;
    if (!a) { g->err = ORC_ENOMEM; return; } v->ld = a;
    b = (uint64_t *)realloc(v->rd, nc * 8); if (!b) { g->err = ORC_ENOMEM; return; } v->rd = b;
    c = (uint64_t *)realloc(v->col, nc * 8); if (!c) { g->err = ORC_ENOMEM; return; } v->col = c;
    d = (uint32_t *)realloc(v->sijkl, nc * 4); if (!d) { g->err = ORC_ENOMEM; return; } v->sijkl = d;
    v->cap = nc;
  }
  v->ld[v->n] = ld; v->rd[v->n] = rd; v->col[v->n] = col; v->sijkl[v->n] = sijkl; v->n++;
}

static void set_pre_queens(gen_t *g, uint64_t ld, uint64_t rd, uint64_t col, int row, int queens, uint64_t LD, uint64_t RD);

/* set_pre_queens_cached (356Py:2758-2805): cache bypass when preset >= 7 */
static void set_pre_queens_cached(gen_t *g, uint64_t ld, uint64_t rd, uint64_t col, int row, int queens,
                                  uint64_t LD, uint64_t RD) {
  if (g->err) return;
  if (g->preset >= 7) { set_pre_queens(g, ld, rd, col, row, queens, LD, RD); return; }
  ckey_t k; memset(&k, 0, sizeof k);
  k.ld = ld; k.rd = rd; k.col = col; k.LD = LD; k.RD = RD; k.row = row; k.queens = queens;
  if (!cache_add(g, &k)) return;
  set_pre_queens(g, ld, rd, col, row, queens, LD, RD);
}

/* set_pre_queens (356Py:2808-2835).  use_visited_prune is False in the reference. */
static void set_pre_queens(gen_t *g, uint64_t ld, uint64_t rd, uint64_t col, int row, int queens, uint64_t LD, uint64_t RD) {
  const int N = g->N;
  const uint64_t board_mask = (N >= 64) ? ~0ULL : ((1ULL << N) - 1);
  if (g->err) return;
  if (row == g->k || row == g->l) {
    set_pre_queens_cached(g, ld << 1, rd >> 1, col, row + 1, queens, LD, RD);
    return;
  }
  if (queens == g->preset) {
    if (g->preset <= 5) {       /* DISABLE_CONSTELLATION_SIGNATURE_PRUNE is False */
      skey_t s; memset(&s, 0, sizeof s);
      s.ld = ld; s.rd = rd; s.col = col; s.row = row;
      if (!sig_add(g, &s)) return;
    }
    rec_push(g, ld, rd, col, (uint32_t)row << 20);
    g->counter++;
    return;
  }
  int sh = N - 1 - row;
  if (sh < 0) { g->err = ORC_EINVAL; return; }   /* Python raises on a negative shift */
  uint64_t fr = ~(ld | rd | col | (LD >> sh) | (RD << sh)) & board_mask;
  while (fr) {
    uint64_t bit = fr & (0 - fr);
    fr &= fr - 1;
    set_pre_queens_cached(g, (ld | bit) << 1, (rd | bit) >> 1, col | bit, row + 1, queens + 1, LD, RD);
    if (g->err) return;
  }
}

static int check_rotations(const uint8_t *S, int i, int j, int k, int l, int N) {
  int r1 = ((N - 1 - k) << 15) + ((N - 1 - l) << 10) + (j << 5) + i;
  int r2 = ((N - 1 - j) << 15) + ((N - 1 - i) << 10) + ((N - 1 - l) << 5) + (N - 1 - k);
  int r3 = (l << 15) + (k << 10) + ((N - 1 - i) << 5) + (N - 1 - j);
  return S[r1] || S[r2] || S[r3];
}

/*
 * gen_constellations (356Py:2837-2926).  Fills the output arrays with the
 * generated records {ld, rd, col, startijkl} (full-width ld/rd/col, as the
 * reference's Python ints).  Returns the record count, or a negative error.
 * When `cap` is smaller than the count nothing is copied: call again with a
 * large enough buffer.  Start constellations are visited in ascending packed
 * ijkl order (the reference visits a Python set; order is not part of the
 * result, which is compared as a multiset keyed by (startijkl, ld, rd, col)).
 */
int64_t orc_gen_constellations(int N, int preset, uint64_t *ld_out, uint64_t *rd_out, uint64_t *col_out,
                               uint32_t *sijkl_out, int64_t cap) {
  if (N < 5 || N > 31 || preset < 1) return ORC_EINVAL;
  const int halfN = (N + 1) / 2, N1 = N - 1, N2 = N - 2;
  uint8_t *S = (uint8_t *)calloc(1 << 20, 1);
  uint8_t *J = (uint8_t *)calloc(1 << 20, 1);
  if (!S || !J) { free(S); free(J); return ORC_ENOMEM; }
  if (N % 2 == 1) {
    int center = N / 2;
    for (int l = center + 1; l < N1; l++)
      for (int i = center + 1; i < N1; i++) {
        if (i == N1 - l) continue;
        for (int j = N - center - 2; j > 0; j--) {
          if (j == i || j == l) continue;
          if (!check_rotations(S, i, j, center, l, N)) S[to_ijkl(i, j, center, l)] = 1;
        }
      }
  }
  for (int k = 1; k < halfN; k++)
    for (int l = k + 1; l < N1; l++)
      for (int i = k + 1; i < N1; i++) {
        if (i == N1 - l) continue;
        for (int j = N - k - 2; j > 0; j--) {
          if (j == i || j == l) continue;
          if (!check_rotations(S, i, j, k, l, N)) S[to_ijkl(i, j, k, l)] = 1;
        }
      }
  for (int j = 1; j < N2; j++)
    for (int l = j + 1; l < N1; l++) S[to_ijkl(0, j, 0, l)] = 1;
  for (int x = 0; x < (1 << 20); x++) if (S[x]) J[orc_jasmin(x, N)] = 1;
  free(S);

  gen_t g; memset(&g, 0, sizeof g);
  g.N = N; g.preset = preset;
  const uint64_t L = 1ULL << N1;
  for (int sc = 0; sc < (1 << 20) && !g.err; sc++) {
    if (!J[sc]) continue;
    g.gen++; g.ccount = 0; g.scount = 0;          /* subconst_cache.clear(); signatures = set() */
    int i = geti(sc), j = getj(sc), k = getk(sc), l = getl(sc);
    if (l < 1 || k > N) { g.err = ORC_EINVAL; break; }
    uint64_t Lj = L >> j, Li = L >> i, Ll = L >> l;
    uint64_t ld = ((i > 0) ? (L >> (i - 1)) : 0) | (1ULL << (N - k));
    uint64_t rd = (L >> (i + 1)) | (1ULL << (l - 1));
    uint64_t col = 1 | L | Li | Lj;
    uint64_t LD = Lj | Ll, RD = Lj | (1ULL << k);
    g.k = k; g.l = l; g.counter = 0;
    int64_t first = g.out.n;
    set_pre_queens_cached(&g, ld, rd, col, 1, (j == N1) ? 3 : 4, LD, RD);
    for (int64_t a = first; a < g.out.n; a++) g.out.sijkl[a] |= (uint32_t)to_ijkl(i, j, k, l);
  }
  free(J);
  int64_t n = g.out.n;
  int64_t ret = g.err ? g.err : n;
  if (!g.err && cap >= n && n > 0) {
    memcpy(ld_out, g.out.ld, n * 8); memcpy(rd_out, g.out.rd, n * 8);
    memcpy(col_out, g.out.col, n * 8); memcpy(sijkl_out, g.out.sijkl, n * 4);
  }
  free(g.ck); free(g.cstamp); free(g.sk); free(g.sstamp);
  free(g.out.ld); free(g.out.rd); free(g.out.col); free(g.out.sijkl);
  return ret;
}

/* ------------------------------------------------------------------ */
/* Task builder: build_soa_for_range (356Py:1971-2169)                 */
/* ------------------------------------------------------------------ */
typedef struct {
  uint32_t ld, rd, col, free_;
  int32_t fid, start, jmark, endmark, mark1, mark2, ijkl, w;
} orc_task;

int orc_build_task(int N, uint64_t rld, uint64_t rrd, uint64_t rcol, uint32_t sijkl, orc_task *t) {
  const uint64_t board_mask = (1ULL << N) - 1;
  const uint64_t small_mask = (N - 2 > 0) ? ((1ULL << (N - 2)) - 1) : 0;
  const int N1 = N - 1, N2 = N - 2;
  int jmark = 0, mark1 = 0, mark2 = 0, endmark = 0, target = 0;
  int start = (int)(sijkl >> 20);
  int ijkl = (int)(sijkl & ((1u << 20) - 1));
  int j = getj(ijkl), k = getk(ijkl), l = getl(ijkl);
  uint64_t ld = rld >> 1, rd = rrd >> 1;
  uint64_t col = ((rcol >> 1) | ~small_mask) & board_mask;
  uint64_t LD = (1ULL << (N1 - j)) | (1ULL << (N1 - l));
  if (N - start < 0) return ORC_EINVAL;
  ld |= LD >> (N - start);
  if (start > k) {
    int sh = N1 - (start - k + 1);
    if (sh < 0) return ORC_EINVAL;
    rd |= 1ULL << sh;
  }
  if (j >= 2 * N - 33 - start) {
    if (N2 - start < 0) return ORC_EINVAL;
    rd |= (1ULL << (N1 - j)) << (N2 - start);
  }
  uint64_t fr = board_mask & ~(ld | rd | col);
  int j_lt_N3 = j < N - 3, j_eq_N3 = j == N - 3, j_eq_N2 = j == N - 2;
  int k_lt_l = k < l, start_lt_k = start < k, start_lt_l = start < l;
  int l_eq_kp1 = l == k + 1, k_eq_lp1 = k == l + 1;
  int j_gate = j > 2 * N - 34 - start;
  if (j_lt_N3) {
    jmark = j + 1; endmark = N2;
    if (j_gate) {
      if (k_lt_l) {
        mark1 = k - 1; mark2 = l - 1;
        if (start_lt_l) target = start_lt_k ? (!l_eq_kp1 ? 0 : 4) : 1;
        else target = 2;
      } else {
        mark1 = l - 1; mark2 = k - 1;
        if (start_lt_k) target = start_lt_l ? (!k_eq_lp1 ? 5 : 7) : 6;
        else target = 2;
      }
    } else {
      if (k_lt_l) { mark1 = k - 1; mark2 = l - 1; target = !l_eq_kp1 ? 8 : 9; }
      else { mark1 = l - 1; mark2 = k - 1; target = !k_eq_lp1 ? 10 : 11; }
    }
  } else if (j_eq_N3) {
    endmark = N2;
    if (k_lt_l) {
      mark1 = k - 1; mark2 = l - 1;
      if (start_lt_l) {
        if (start_lt_k) target = !l_eq_kp1 ? 12 : 15;
        else { mark2 = l - 1; target = 13; }
      } else target = 14;
    } else {
      mark1 = l - 1; mark2 = k - 1;
      if (start_lt_k) {
        if (start_lt_l) target = !k_eq_lp1 ? 16 : 18;
        else { mark2 = k - 1; target = 17; }
      } else target = 14;
    }
  } else if (j_eq_N2) {
    if (k_lt_l) {
      endmark = N2;
      if (start_lt_l) {
        if (start_lt_k) {
          mark1 = k - 1;
          if (!l_eq_kp1) { mark2 = l - 1; target = 19; } else target = 22;
        } else { mark2 = l - 1; target = 20; }
      } else target = 21;
    } else {
      if (start_lt_k) {
        if (start_lt_l) {
          if (k < N2) {
            mark1 = l - 1; endmark = N2;
            if (!k_eq_lp1) { mark2 = k - 1; target = 23; } else target = 24;
          } else {
            if (l != N - 3) { mark2 = l - 1; endmark = N - 3; target = 20; }
            else { endmark = N - 4; target = 21; }
          }
        } else {
          if (k != N2) { mark2 = k - 1; endmark = N2; target = 25; }
          else { endmark = N - 3; target = 21; }
        }
      } else { endmark = N2; target = 21; }
    }
  } else {
    endmark = N2;
    if (start > k) target = 26;
    else { mark1 = k - 1; target = 27; }
  }
  t->ld = (uint32_t)ld; t->rd = (uint32_t)rd; t->col = (uint32_t)col; t->free_ = (uint32_t)fr;
  t->fid = target; t->start = start; t->jmark = jmark; t->endmark = endmark;
  t->mark1 = mark1; t->mark2 = mark2; t->ijkl = ijkl; t->w = orc_symmetry(ijkl, N);
  return ORC_OK;
}

/* ------------------------------------------------------------------ */
/* SQ* state machine tables (356Py:2236-2289, 2586-2589)               */
/* ------------------------------------------------------------------ */
/* func_meta: (next_funcid, funcptn, avail_flag) per fid */
static const int META_NEXT[28] = {1, 2, 3, 3, 2, 6, 2, 2, 0, 4, 5, 7, 13, 14, 14, 14, 17, 14, 14, 20, 21, 21, 21, 25, 21, 21, 26, 26};
static const int META_PTN[28]  = {0, 1, 3, 5, 2, 0, 1, 2, 4, 4, 4, 4, 0, 1, 5, 2, 0, 1, 2, 0, 1, 5, 2, 0, 2, 1, 5, 0};
static const int META_AV[28]   = {0, 0, 1, 1, 0, 0, 0, 0, 1, 1, 1, 1, 0, 0, 1, 0, 0, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0};
/* FUNC_CATEGORY -> blockK: 3 => 1<<(N-3), 4 => 1<<(N-4), 0 => 0 */
static const int FUNC_CAT[28]  = {3, 0, 0, 0, 4, 0, 3, 3, 0, 0, 0, 0, 3, 0, 0, 4, 0, 3, 3, 3, 0, 0, 4, 0, 3, 3, 0, 3};
static const int BLOCK_L[28]   = {0, 1, 0, 0, 1, 1, 0, 2, 0, 0, 0, 0, 0, 1, 0, 1, 1, 0, 2, 0, 0, 0, 1, 1, 2, 0, 0, 0};

void orc_tables(int *next, int *ptn, int *av, int *cat, int *bl) {
  for (int f = 0; f < 28; f++) { next[f] = META_NEXT[f]; ptn[f] = META_PTN[f]; av[f] = META_AV[f]; cat[f] = FUNC_CAT[f]; bl[f] = BLOCK_L[f]; }
}

/* ------------------------------------------------------------------ */
/* dfs_iter (356Py:1837-1967), with a node counter                     */
/* ------------------------------------------------------------------ */
typedef struct { int fid; uint64_t ld, rd, col; int row; uint64_t fr; } frame_t;

uint64_t orc_dfs_iter(int N, const orc_task *t, uint64_t *nodes_out) {
  const uint64_t bm = (1ULL << N) - 1;
  const uint64_t n3 = 1ULL << (N - 3 > 0 ? N - 3 : 0), n4 = 1ULL << (N - 4 > 0 ? N - 4 : 0);
  frame_t stack[4096];
  int sp = 0;
  uint64_t total = 0, nodes = 0;
  stack[sp++] = (frame_t){t->fid, t->ld, t->rd, t->col, t->start, t->free_};
  while (sp) {
    frame_t f = stack[--sp];
    if (!f.fr) continue;
    int fid = f.fid, nxt = META_NEXT[fid], ptn = META_PTN[fid], av = META_AV[fid];
    uint64_t avail = f.fr, ld = f.ld, rd = f.rd, col = f.col;
    int row = f.row;
    if (ptn == 5 && row == t->endmark) {
      if (fid == 14) total += (avail >> 1) ? 1 : 0;
      else total += 1;
      continue;
    }
    int step = 1; uint64_t add1 = 0; int row_step = row + 1;
    int use_blocks = 0, use_future = (av == 1), local_next = fid;
    uint64_t bK = 0, bL = 0;
    if (ptn == 0 || ptn == 1 || ptn == 2) {
      int at_mark = (ptn == 0 || ptn == 2) ? (row == t->mark1) : (row == t->mark2);
      if (at_mark && avail) {
        step = (ptn == 0 || ptn == 1) ? 2 : 3;
        add1 = (ptn == 1 && fid == 20) ? 1 : 0;
        row_step = row + step;
        bK = FUNC_CAT[fid] == 3 ? n3 : (FUNC_CAT[fid] == 4 ? n4 : 0);
        bL = (uint64_t)BLOCK_L[fid];
        use_blocks = 1; use_future = 0; local_next = nxt;
      }
    } else if (ptn == 3 && row == t->jmark) {
      avail &= ~1ULL; ld |= 1; local_next = nxt;
      if (!avail) continue;
    } else if (ptn == 4 && row == t->mark1) {
      if (sp >= 4096) return ~0ULL;
      stack[sp++] = (frame_t){nxt, ld, rd, col, row, avail};
      continue;
    }
    if (sp + 64 >= 4096) { if (nodes_out) *nodes_out = nodes; return ~0ULL; }
    /* The reference pushes every child and pops LIFO; the per-frame loops are identical
       except for the step/blocks and the optional look-ahead. */
    int lookahead = !use_blocks && use_future && !(row_step >= t->endmark);
    while (avail) {
      uint64_t bit = avail & (0 - avail);
      avail &= avail - 1;
      nodes++;
      uint64_t nld, nrd, ncol = col | bit;
      if (use_blocks) { nld = ((ld | bit) << step) | add1 | bL; nrd = ((rd | bit) >> step) | bK; }
      else { nld = (ld | bit) << 1; nrd = (rd | bit) >> 1; }
      uint64_t nf = bm & ~(nld | nrd | ncol);
      if (!nf) continue;
      if (lookahead && !(bm & ~((nld << 1) | (nrd >> 1) | ncol))) continue;
      stack[sp++] = (frame_t){local_next, nld, nrd, ncol, row_step, nf};
    }
  }
  if (nodes_out) *nodes_out = nodes;
  return total;
}

/* ------------------------------------------------------------------ */
/* exec_solutions, CPU branch (356Py:2579-2610), multi-threaded        */
/* ------------------------------------------------------------------ */
typedef struct {
  int N; int64_t m;
  const uint64_t *ld, *rd, *col; const uint32_t *sijkl;
  uint64_t *sol, *nodes;
  int64_t next;
  pthread_mutex_t mu;
  int err;
} exec_ctx;

static void *exec_worker(void *arg) {
  exec_ctx *c = (exec_ctx *)arg;
  for (;;) {
    pthread_mutex_lock(&c->mu);
    int64_t a = c->next; c->next += 16;
    pthread_mutex_unlock(&c->mu);
    if (a >= c->m) break;
    int64_t b = a + 16 < c->m ? a + 16 : c->m;
    for (int64_t i = a; i < b; i++) {
      orc_task t;
      if (orc_build_task(c->N, c->ld[i], c->rd[i], c->col[i], c->sijkl[i], &t)) { c->err = ORC_EINVAL; continue; }
      uint64_t nd = 0;
      uint64_t cnt = orc_dfs_iter(c->N, &t, &nd);
      if (cnt == ~0ULL) { c->err = ORC_EINVAL; continue; }
      c->sol[i] = cnt * (uint64_t)t.w;
      if (c->nodes) c->nodes[i] = nd;
    }
  }
  return NULL;
}

/*
 * exec_solutions: per-record weighted counts into sol[] (and dfs_iter nodes
 * into nodes[] when non-NULL).  `threads` <= 1 runs on the calling thread.
 */
int orc_exec_solutions(int N, int64_t m, const uint64_t *ld, const uint64_t *rd, const uint64_t *col,
                       const uint32_t *sijkl, uint64_t *sol, uint64_t *nodes, int threads) {
  exec_ctx c; memset(&c, 0, sizeof c);
  c.N = N; c.m = m; c.ld = ld; c.rd = rd; c.col = col; c.sijkl = sijkl; c.sol = sol; c.nodes = nodes;
  pthread_mutex_init(&c.mu, NULL);
  if (threads <= 1) exec_worker(&c);
  else {
    if (threads > 512) threads = 512;
    pthread_t th[512];
    for (int t = 0; t < threads; t++) pthread_create(&th[t], NULL, exec_worker, &c);
    for (int t = 0; t < threads; t++) pthread_join(th[t], NULL);
  }
  pthread_mutex_destroy(&c.mu);
  return c.err;
}

/* ------------------------------------------------------------------ */
/* Brute force (356Py:5755-5767) and completion counts                 */
/* ------------------------------------------------------------------ */
static uint64_t bt(int N, uint64_t mask, int row, uint64_t left, uint64_t down, uint64_t right, const int *forced) {
  if (row == N) return 1;
  uint64_t total = 0;
  uint64_t bitmap = mask & ~(left | down | right);
  if (forced && forced[row] >= 0) bitmap &= 1ULL << forced[row];
  while (bitmap) {
    uint64_t bit = bitmap & (0 - bitmap);
    bitmap ^= bit;
    total += bt(N, mask, row + 1, (left | bit) << 1, down | bit, (right | bit) >> 1, forced);
  }
  return total;
}
uint64_t orc_bit_total(int N) {
  if (N < 1 || N > 31) return 0;
  return bt(N, (1ULL << N) - 1, 0, 0, 0, 0, NULL);
}
/*
 * Completions of a board with k pre-placed queens (rows[i], cols[i]): the
 * number of full N-queens placements that contain them.  Pre-placed queens
 * break the board symmetry, so no weights apply.  Column c is bit c.
 * Returns 0 when the pre-placed queens attack one another.
 */
uint64_t orc_completions(int N, int k, const int *rows, const int *cols) {
  int forced[64];
  for (int r = 0; r < N; r++) forced[r] = -1;
  for (int q = 0; q < k; q++) {
    if (rows[q] < 0 || rows[q] >= N || cols[q] < 0 || cols[q] >= N) return 0;
    if (forced[rows[q]] >= 0 && forced[rows[q]] != cols[q]) return 0;
    forced[rows[q]] = cols[q];
  }
  return bt(N, (1ULL << N) - 1, 0, 0, 0, 0, forced);
}

/* ------------------------------------------------------------------ */
/* Unique + total, symmetry method (07Py_bit_symmetry.py:65-200)       */
/* ------------------------------------------------------------------ */
typedef struct {
  int size; uint64_t board[64];
  int bound1, bound2; uint64_t topbit, endbit, sidemask, lastmask;
  uint64_t c2, c4, c8;
} sym_t;

static void symmetryops(sym_t *s) {
  const int size = s->size;
  uint64_t *b = s->board;
  int own, you; uint64_t bit, ptn;
  if (b[s->bound2] == 1) {
    own = 1; ptn = 2;
    while (own <= size - 1) {
      bit = 1; you = size - 1;
      while (b[you] != ptn && b[own] >= bit) { bit <<= 1; you--; }
      if (b[own] > bit) return;
      if (b[own] < bit) break;
      own++; ptn <<= 1;
    }
    if (own > size - 1) { s->c2++; return; }
  }
  if (b[size - 1] == s->endbit) {
    own = 1; you = size - 1 - 1;
    while (own <= size - 1) {
      bit = 1; ptn = s->topbit;
      while (b[you] != ptn && b[own] >= bit) { bit <<= 1; ptn >>= 1; }
      if (b[own] > bit) return;
      if (b[own] < bit) break;
      own++; you--;
    }
    if (own > size - 1) { s->c4++; return; }
  }
  if (b[s->bound1] == s->topbit) {
    own = 1; ptn = s->topbit >> 1;
    while (own <= size - 1) {
      bit = 1; you = 0;
      while (b[you] != ptn && b[own] >= bit) { bit <<= 1; you++; }
      if (b[own] > bit) return;
      if (b[own] < bit) break;
      own++; ptn >>= 1;
    }
  }
  s->c8++;
}
static void backtrack2(sym_t *s, int row, uint64_t left, uint64_t down, uint64_t right) {
  const int size = s->size;
  uint64_t mask = (1ULL << size) - 1;
  uint64_t bitmap = mask & ~(left | down | right);
  if (row == size - 1) {
    if (bitmap && (bitmap & s->lastmask) == 0) { s->board[row] = bitmap; symmetryops(s); }
    return;
  }
  if (row < s->bound1) { bitmap |= s->sidemask; bitmap ^= s->sidemask; }
  else if (row == s->bound2) {
    if ((down & s->sidemask) == 0) return;
    if ((down & s->sidemask) != s->sidemask) bitmap &= s->sidemask;
  }
  while (bitmap) {
    uint64_t bit = bitmap & (0 - bitmap);
    bitmap ^= bit;
    s->board[row] = bit;
    backtrack2(s, row + 1, (left | bit) << 1, down | bit, (right | bit) >> 1);
  }
}
static void backtrack1(sym_t *s, int row, uint64_t left, uint64_t down, uint64_t right) {
  const int size = s->size;
  uint64_t mask = (1ULL << size) - 1;
  uint64_t bitmap = mask & ~(left | down | right);
  if (row == size - 1) {
    if (bitmap) { s->board[row] = bitmap; s->c8++; }
    return;
  }
  if (row < s->bound1) { bitmap |= 2; bitmap ^= 2; }
  while (bitmap) {
    uint64_t bit = bitmap & (0 - bitmap);
    bitmap ^= bit;
    s->board[row] = bit;
    backtrack1(s, row + 1, (left | bit) << 1, down | bit, (right | bit) >> 1);
  }
}
/* NQueens() of 07Py_bit_symmetry.py:171-200.  Valid for 4 <= N <= 31. */
int orc_unique_symmetry(int N, uint64_t *unique, uint64_t *total, uint64_t *c2, uint64_t *c4, uint64_t *c8) {
  if (N < 4 || N > 31) return ORC_EINVAL;
  sym_t s; memset(&s, 0, sizeof s);
  s.size = N;
  s.topbit = 1ULL << (N - 1);
  s.bound1 = 2; s.bound2 = 0;
  s.board[0] = 1;
  while (s.bound1 > 1 && s.bound1 < N - 1) {
    uint64_t bit = 1ULL << s.bound1;
    s.board[1] = bit;
    backtrack1(&s, 2, (2 | bit) << 1, 1 | bit, (2 | bit) >> 1);
    s.bound1++;
  }
  s.topbit = 1ULL << (N - 1);
  s.endbit = s.topbit >> 1;
  s.sidemask = s.lastmask = s.topbit | 1;
  s.bound1 = 1; s.bound2 = N - 2;
  while (s.bound1 > 0 && s.bound2 < N - 1 && s.bound1 < s.bound2) {
    uint64_t bit = 1ULL << s.bound1;
    s.board[0] = bit;
    backtrack2(&s, 1, bit << 1, bit, bit >> 1);
    s.bound1++; s.bound2--;
    s.endbit >>= 1;
    s.lastmask = (s.lastmask << 1) | s.lastmask | (s.lastmask >> 1);
  }
  *unique = s.c2 + s.c4 + s.c8;
  *total = s.c2 * 2 + s.c4 * 4 + s.c8 * 8;
  if (c2) *c2 = s.c2;
  if (c4) *c4 = s.c4;
  if (c8) *c8 = s.c8;
  return ORC_OK;
}
