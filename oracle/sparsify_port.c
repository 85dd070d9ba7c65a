/*
 * ORACLE — test infrastructure, not product code.
 *
 * Plain-C restatement of LightNE's sparsifier: the counter-based generator,
 * the per-edge path sampler, the concurrent pair-count table, the trunc-log
 * map and the CSR build.  Only tests/, __graft_entry__.smoke() and the CPU
 * leg of bench.py load this library, and only as a checker or as the timed
 * CPU baseline.  It is pinned against the reference itself (the program
 * built from oracle/ref_sparsify_harness.cc) by tests/test_oracle_pin.py and
 * by the committed fixtures in tests/golden/.
 *
 * Reference correspondence (paths inside the reference project):
 *   hash64_2                 pbbslib/utilities.h:154-159
 *   pbbs::random rand/next/fork   pbbslib/random.h:38-51
 *   map_uint64_t             LightNE/PathEmbed.h:25-30
 *   random_walk, path_sample LightNE/PathEmbed.h:37-58
 *   sampling parameters      LightNE/PathEmbed.h:89-117
 *   table sizing             LightNE/PathEmbed.h:99-102, LightNE/par_table.h:60-70
 *   per-edge sampler g_map_f LightNE/PathEmbed.h:128-171
 *   insert_add               LightNE/par_table.h:86-109
 *   M_exact, factor          LightNE/PathEmbed.h:175-200
 *   trunc-log map            LightNE/PathEmbed.h:203-218
 *   CSR build                LightNE/PathEmbed.h:224-311
 *
 * The table claims a slot with an 8-byte compare-and-swap of the key and then
 * adds the weight with a separate atomic add, instead of the reference's
 * 16-byte (key, value) CAS.  The final multiset of (key, summed weight) is the
 * same; with -sample 0 every weight is 1.0 and the sums are exact integers, so
 * the result is independent of thread interleaving, as in the reference.
 * The output CSR is canonical: each row sorted by column (the reference's
 * within-row order is nondeterministic, PathEmbed.h:300-311).
 *
 * Built with -ffp-contract=off so that no multiply-add is fused: every
 * floating-point expression rounds exactly as written in the reference.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#include <omp.h>

#define LNE_EMPTY_KEY UINT64_MAX

/* Status codes shared with the product's C ABI. */
#define PORT_OK 0
#define PORT_ERR_ALLOC 2
#define PORT_ERR_TABLE_FULL 3

static inline uint64_t h64(uint64_t x) {
  x = (x ^ (x >> 30)) * UINT64_C(0xbf58476d1ce4e5b9);
  x = (x ^ (x >> 27)) * UINT64_C(0x94d049bb133111eb);
  return x ^ (x >> 31);
}
/* pbbs::random: rand() = h(state); next() = h(h(state)); fork(i) = h(h(i+state)) */
static inline uint64_t rng_rand(uint64_t s) { return h64(s); }
static inline uint64_t rng_next(uint64_t s) { return h64(h64(s)); }
static inline uint64_t rng_fork(uint64_t s, uint64_t i) { return h64(h64(i + s)); }
static inline double map_u64(uint64_t u) { return (double)u / 18446744073709551616.0; }

uint64_t lne_port_hash64_2(uint64_t x) { return h64(x); }
double lne_port_map_uint64(uint64_t x) { return map_u64(x); }

/* Sampling parameters, in the reference's evaluation order.
 * out[0]=logn out[1]=M out[2]=1/lambda out[3]=exp_rv_rounded out[4]=frac
 * out[5]=table_size out[6]=capacity */
void lne_port_params(int64_t n, int64_t m_dir, int64_t walk_len, int64_t tablesz,
                     float sample_ratio, float mem_ratio, double* out) {
  double logn = log((double)(size_t)n);
  size_t ts = (size_t)((double)((size_t)walk_len * (size_t)n) * logn * (double)mem_ratio);
  if ((size_t)tablesz > ts) ts = (size_t)tablesz;
  size_t want = 2 * ts, b = want - 1, bits = 0;
  while (b > 0) { b >>= 1; bits++; }
  double M = (double)((size_t)walk_len * (size_t)n) * logn * (double)sample_ratio;
  double inv_lambda = M / (double)(size_t)m_dir;
  size_t exp_rv = (size_t)inv_lambda;
  double frac = inv_lambda - (double)exp_rv;
  out[0] = logn; out[1] = M; out[2] = inv_lambda; out[3] = (double)exp_rv;
  out[4] = frac; out[5] = (double)ts; out[6] = (double)((size_t)1 << bits);
}

typedef struct { uint64_t key; double val; } slot_t;

typedef struct {
  slot_t* slots;
  uint64_t mask;
  int full;
} table_t;

static inline void atomic_add_double(double* p, double w) {
  uint64_t* q = (uint64_t*)p;
  uint64_t old = __atomic_load_n(q, __ATOMIC_RELAXED);
  for (;;) {
    double d; memcpy(&d, &old, 8);
    d += w;
    uint64_t nw; memcpy(&nw, &d, 8);
    if (__atomic_compare_exchange_n(q, &old, nw, 0, __ATOMIC_RELAXED, __ATOMIC_RELAXED)) return;
  }
}

static inline void table_insert_add(table_t* t, uint64_t k, double w) {
  uint64_t h = h64(k) & t->mask;
  for (uint64_t ctr = 0; ctr <= t->mask; ++ctr) {
    uint64_t cur = __atomic_load_n(&t->slots[h].key, __ATOMIC_RELAXED);
    if (cur == LNE_EMPTY_KEY) {
      uint64_t expect = LNE_EMPTY_KEY;
      if (__atomic_compare_exchange_n(&t->slots[h].key, &expect, k, 0, __ATOMIC_RELAXED,
                                      __ATOMIC_RELAXED)) {
        atomic_add_double(&t->slots[h].val, w);
        return;
      }
      cur = expect;
    }
    if (cur == k) { atomic_add_double(&t->slots[h].val, w); return; }
    h = (h + 1) & t->mask;
  }
  t->full = 1; /* every slot holds another key: the reference loops until it exits */
}

/* One directed edge's worth of samples: LightNE/PathEmbed.h:128-171. */
static inline uint64_t walk(const int64_t* off, const int32_t* nbr, uint32_t u,
                            uint64_t steps, uint64_t* s) {
  for (uint64_t i = 0; i < steps; ++i) {
    uint64_t deg = (uint64_t)(off[u + 1] - off[u]);
    uint64_t idx = rng_rand(*s) % deg; /* 64-bit modulo, as the reference */
    u = (uint32_t)nbr[off[u] + (int64_t)idx];
    *s = rng_next(*s);
  }
  return u;
}

static inline uint64_t sample_edge(const int64_t* off, const int32_t* nbr, uint64_t seed,
                                   uint32_t u, uint32_t v, uint64_t walk_len, int sample,
                                   uint64_t exp_rv_rounded, double frac, double logn,
                                   table_t* t) {
  uint64_t s = rng_fork(seed, ((uint64_t)u << 32) | (uint64_t)v);
  uint64_t exp_rv = exp_rv_rounded;
  if (frac > 0.0000000001) {
    exp_rv += (map_u64(rng_rand(s)) < frac) ? 1u : 0u;
    s = rng_next(s);
  }
  uint64_t emitted = 0;
  double p = 1.0, ipw = 1.0;
  if (sample) {
    double du = (double)(uint32_t)(off[u + 1] - off[u]);
    double dv = (double)(uint32_t)(off[v + 1] - off[v]);
    p = (1.0 / du + 1.0 / dv) * logn;
    if (p > 1.0) p = 1.0;
    ipw = 1.0 / p;
  }
  for (uint64_t k = 0; k < exp_rv; ++k) {
    if (sample) {
      double eff = map_u64(rng_rand(s));
      s = rng_next(s);
      if (!(eff < p)) continue;
    }
    uint64_t r = (uint64_t)(uint32_t)(rng_rand(s) % walk_len + 1);
    s = rng_next(s);
    uint64_t kk = (uint64_t)(uint32_t)(rng_rand(s) % r + 1);
    s = rng_next(s);
    uint32_t x = (uint32_t)walk(off, nbr, u, kk - 1, &s);
    uint32_t z = (uint32_t)walk(off, nbr, v, r - kk, &s);
    uint32_t lo = x < z ? x : z, hi = x < z ? z : x;
    table_insert_add(t, ((uint64_t)lo << 32) + (uint64_t)hi, sample ? ipw : 1.0);
    emitted++;
  }
  return emitted;
}

static double now_s(void) {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

static int cmp_u64(const void* a, const void* b) {
  uint64_t x = *(const uint64_t*)a, y = *(const uint64_t*)b;
  return x < y ? -1 : (x > y ? 1 : 0);
}

/*
 * A sparsifier run in steps: lne_port_session_create sizes and clears the
 * table, lne_port_session_sample runs the per-edge sampler over the out-edges
 * of the vertices [u_begin, u_end) (any number of calls, in any order: the
 * table's final contents do not depend on it), lne_port_session_finish runs
 * M_exact, the trunc-log map and the CSR build and releases the table.
 */
typedef struct {
  int64_t n;
  const int64_t* off;
  const int32_t* nbr;
  uint64_t seed;
  int64_t walk_len, negative;
  int sample, upper;
  double prm[7];
  table_t t;
  uint64_t emitted;
  double sec_sample;
} port_session_t;

void* lne_port_session_create(int64_t n, const int64_t* off, const int32_t* nbr, uint64_t seed, int64_t walk_len,
                              int64_t tablesz, int64_t negative, int sample, float sample_ratio, float mem_ratio,
                              int upper, int nthreads) {
  if (nthreads > 0) omp_set_num_threads(nthreads);
  port_session_t* ps = (port_session_t*)calloc(1, sizeof(port_session_t));
  if (!ps) return NULL;
  ps->n = n; ps->off = off; ps->nbr = nbr; ps->seed = seed; ps->walk_len = walk_len;
  ps->negative = negative; ps->sample = sample; ps->upper = upper;
  lne_port_params(n, off[n], walk_len, tablesz, sample_ratio, mem_ratio, ps->prm);
  uint64_t cap = (uint64_t)ps->prm[6];
  ps->t.slots = (slot_t*)malloc(cap * sizeof(slot_t));
  if (!ps->t.slots) { free(ps); return NULL; }
  ps->t.mask = cap - 1;
  ps->t.full = 0;
  slot_t* sl = ps->t.slots;
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < (int64_t)cap; ++i) { sl[i].key = LNE_EMPTY_KEY; sl[i].val = 0.0; }
  return ps;
}

int64_t lne_port_session_sample(void* h, int64_t u_begin, int64_t u_end) {
  port_session_t* ps = (port_session_t*)h;
  const int64_t* off = ps->off;
  const int32_t* nbr = ps->nbr;
  double logn = ps->prm[0], frac = ps->prm[4];
  uint64_t exp_rv_rounded = (uint64_t)ps->prm[3];
  double t0 = now_s();
  uint64_t emitted = 0;
#pragma omp parallel for schedule(dynamic, 64) reduction(+ : emitted)
  for (int64_t u = u_begin; u < u_end; ++u) {
    for (int64_t e = off[u]; e < off[u + 1]; ++e) {
      emitted += sample_edge(off, nbr, ps->seed, (uint32_t)u, (uint32_t)nbr[e], (uint64_t)ps->walk_len,
                             ps->sample, exp_rv_rounded, frac, logn, &ps->t);
    }
  }
  ps->sec_sample += now_s() - t0;
  ps->emitted += emitted;
  return ps->t.full ? -PORT_ERR_TABLE_FULL : (int64_t)emitted;
}

void lne_port_session_free(void* h) {
  port_session_t* ps = (port_session_t*)h;
  if (!ps) return;
  free(ps->t.slots);
  free(ps);
}

/*
 * Trunc-log and CSR of a session; frees the session.  stats (double[16]):
 *  0 logn, 1 M, 2 1/lambda, 3 exp_rv_rounded, 4 frac, 5 table_size, 6 capacity,
 *  7 samples emitted, 8 M_exact, 9 factor, 10 nnz_upper (kept slots),
 *  11 nnz, 12 seconds (sampling+insert), 13 seconds (trunc-log + CSR),
 *  14 threads used, 15 distinct keys before trunc-log.
 * On success *out_col / *out_val are malloc'd (free with lne_port_free);
 * row_ptr is caller-allocated int64[n+1].
 */
int lne_port_session_finish(void* h, int64_t* row_ptr, int32_t** out_col, float** out_val, double* stats) {
  port_session_t* ps = (port_session_t*)h;
  const int64_t n = ps->n;
  const int64_t* off = ps->off;
  const int64_t m_dir = off[n];
  const int upper = ps->upper;
  table_t t = ps->t;
  uint64_t cap = (uint64_t)ps->prm[6];
  for (int i = 0; i < 7; ++i) stats[i] = ps->prm[i];
  stats[7] = (double)ps->emitted;
  stats[12] = ps->sec_sample;
  if (t.full) { lne_port_session_free(ps); return PORT_ERR_TABLE_FULL; }
  double t1 = now_s();

  /* M_exact: sum of weights in slot order. */
  double M_exact = 0.0;
  uint64_t distinct = 0;
  for (uint64_t i = 0; i < cap; ++i)
    if (t.slots[i].key != LNE_EMPTY_KEY) { M_exact += t.slots[i].val; distinct++; }
  stats[8] = M_exact;
  stats[15] = (double)distinct;
  double vol = (double)(size_t)m_dir;
  double factor = vol * (double)(size_t)m_dir / M_exact / 2 / (double)(size_t)ps->negative;
  stats[9] = factor;

  /* Trunc-log map (PathEmbed.h:203-218), then row counts. */
  int64_t* cnt = (int64_t*)calloc((size_t)n + 1, sizeof(int64_t));
  if (!cnt) { lne_port_session_free(ps); return PORT_ERR_ALLOC; }
  uint64_t kept = 0;
#pragma omp parallel for schedule(static) reduction(+ : kept)
  for (int64_t i = 0; i < (int64_t)cap; ++i) {
    uint64_t key = t.slots[i].key;
    if (key == LNE_EMPTY_KEY) continue;
    uint32_t u = (uint32_t)(key >> 32), v = (uint32_t)key;
    uint32_t du = (uint32_t)(off[u + 1] - off[u]), dv = (uint32_t)(off[v + 1] - off[v]);
    double w = (u != v) ? t.slots[i].val : t.slots[i].val * 2;
    double adj = w * factor / du / dv;
    double L = log(adj);
    if (L > 0.0) {
      t.slots[i].val = L;
      kept++;
      __atomic_fetch_add(&cnt[u], 1, __ATOMIC_RELAXED);
      if (!upper && u != v) __atomic_fetch_add(&cnt[v], 1, __ATOMIC_RELAXED);
    } else {
      t.slots[i].key = LNE_EMPTY_KEY;
    }
  }
  stats[10] = (double)kept;
  row_ptr[0] = 0;
  for (int64_t i = 0; i < n; ++i) row_ptr[i + 1] = row_ptr[i] + cnt[i];
  int64_t nnz = row_ptr[n];
  stats[11] = (double)nnz;
  uint64_t* packed = (uint64_t*)malloc((size_t)(nnz > 0 ? nnz : 1) * sizeof(uint64_t));
  if (!packed) { free(cnt); lne_port_session_free(ps); return PORT_ERR_ALLOC; }
  memset(cnt, 0, (size_t)(n + 1) * sizeof(int64_t));
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < (int64_t)cap; ++i) {
    uint64_t key = t.slots[i].key;
    if (key == LNE_EMPTY_KEY) continue;
    uint32_t u = (uint32_t)(key >> 32), v = (uint32_t)key;
    float fv = (float)t.slots[i].val;
    uint32_t bits; memcpy(&bits, &fv, 4);
    int64_t p = __atomic_fetch_add(&cnt[u], 1, __ATOMIC_RELAXED);
    packed[row_ptr[u] + p] = ((uint64_t)v << 32) | bits;
    if (!upper && u != v) {
      p = __atomic_fetch_add(&cnt[v], 1, __ATOMIC_RELAXED);
      packed[row_ptr[v] + p] = ((uint64_t)u << 32) | bits;
    }
  }
#pragma omp parallel for schedule(dynamic, 16)
  for (int64_t i = 0; i < n; ++i)
    qsort(packed + row_ptr[i], (size_t)(row_ptr[i + 1] - row_ptr[i]), sizeof(uint64_t), cmp_u64);
  int32_t* col = (int32_t*)malloc((size_t)(nnz > 0 ? nnz : 1) * sizeof(int32_t));
  float* val = (float*)malloc((size_t)(nnz > 0 ? nnz : 1) * sizeof(float));
  if (!col || !val) {
    free(col); free(val); free(packed); free(cnt); lne_port_session_free(ps);
    return PORT_ERR_ALLOC;
  }
#pragma omp parallel for schedule(static)
  for (int64_t j = 0; j < nnz; ++j) {
    col[j] = (int32_t)(packed[j] >> 32);
    uint32_t bits = (uint32_t)packed[j];
    memcpy(&val[j], &bits, 4);
  }
  double t2 = now_s();
  stats[13] = t2 - t1;
  stats[14] = (double)omp_get_max_threads();
  free(packed);
  free(cnt);
  lne_port_session_free(ps);
  *out_col = col;
  *out_val = val;
  return PORT_OK;
}

/* Full sparsifier in one call: a session over all vertices (stats and
 * outputs as lne_port_session_finish). */
int lne_port_sparsify(int64_t n, const int64_t* off, const int32_t* nbr, uint64_t seed,
                      int64_t walk_len, int64_t tablesz, int64_t negative, int sample,
                      float sample_ratio, float mem_ratio, int upper, int nthreads,
                      int64_t* row_ptr, int32_t** out_col, float** out_val, double* stats) {
  void* ps = lne_port_session_create(n, off, nbr, seed, walk_len, tablesz, negative, sample, sample_ratio,
                                     mem_ratio, upper, nthreads);
  if (!ps) return PORT_ERR_ALLOC;
  lne_port_session_sample(ps, 0, n);
  return lne_port_session_finish(ps, row_ptr, out_col, out_val, stats);
}

/*
 * Sampling + insert only, over the directed edges [e_begin, e_end) of the
 * CSR (edge index order): the bounded CPU baseline of the sampler stage.
 * Returns the number of samples emitted; *seconds gets the wall time.
 * The table has the capacity the full run would use.
 */
int64_t lne_port_sample_range(int64_t n, const int64_t* off, const int32_t* nbr, uint64_t seed,
                              int64_t walk_len, int64_t tablesz, int sample, float sample_ratio,
                              float mem_ratio, int64_t e_begin, int64_t e_end, int nthreads,
                              double* seconds) {
  if (nthreads > 0) omp_set_num_threads(nthreads);
  double prm[7];
  lne_port_params(n, off[n], walk_len, tablesz, sample_ratio, mem_ratio, prm);
  uint64_t cap = (uint64_t)prm[6];
  table_t t;
  t.slots = (slot_t*)malloc(cap * sizeof(slot_t));
  if (!t.slots) return -1;
  t.mask = cap - 1;
  t.full = 0;
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < (int64_t)cap; ++i) { t.slots[i].key = LNE_EMPTY_KEY; t.slots[i].val = 0.0; }
  /* source vertex of each edge in range: binary search in off[] */
  double t0 = now_s();
  uint64_t emitted = 0;
#pragma omp parallel for schedule(dynamic, 256) reduction(+ : emitted)
  for (int64_t e = e_begin; e < e_end; ++e) {
    int64_t lo = 0, hi = n; /* largest u with off[u] <= e */
    while (hi - lo > 1) { int64_t mid = (lo + hi) / 2; if (off[mid] <= e) lo = mid; else hi = mid; }
    emitted += sample_edge(off, nbr, seed, (uint32_t)lo, (uint32_t)nbr[e], (uint64_t)walk_len,
                           sample, (uint64_t)prm[3], prm[4], prm[0], &t);
  }
  *seconds = now_s() - t0;
  free(t.slots);
  return t.full ? -2 : (int64_t)emitted;
}

void lne_port_free(void* p) { free(p); }
