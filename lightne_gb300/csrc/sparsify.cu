// NetSMF sparsifier on the device: path sampler, pair-count table,
// trunc-log map and canonical CSR build.
//
// Reference: path_embed::generate_trunc_log_matrix_v2 (LightNE/PathEmbed.h:81-369)
// with par_table (LightNE/par_table.h).
//
// Layout in HBM during one call:
//   table   Slot[capacity]       16 B per slot: u64 key, u64 count (or f64 weight)
//   rowcnt  i64[n]               kept entries per row, then the scatter cursor
//   row_ptr i64[n+1]             exclusive scan of rowcnt (the output row_ptr)
//   packed  u64[nnz]             (col << 32 | float bits) per entry; rows sorted in place
//   col/val i32[nnz], f32[nnz]   output CSR
#include <cuda_runtime.h>
#include <math.h>
#include <stdio.h>

#include <algorithm>
#include <string>

#include "lne_internal.h"
#include "lne_math.cuh"

namespace lne {

struct __align__(16) Slot {
  unsigned long long key;
  unsigned long long val;
};
static constexpr unsigned long long kEmptyKey = ~0ULL;
// Probe limit of one insert.  The reference gives up after 10^7 probes
// (LightNE/par_table.h:104-107); under its sizing rule (capacity >= 2x the
// requested size) a linear-probe run this long only occurs in a table that
// is essentially full, so the status is the same and the wait is bounded.
static constexpr uint32_t kMaxProbes = 1u << 16;
static constexpr unsigned kFullMask = 0xffffffffu;

struct SampleArgs {
  uint64_t seed;
  uint64_t walk_len;      // T (< 2^31)
  uint64_t walk_magic;    // Granlund-Montgomery multiplier of T
  uint64_t exp_rv;
  double frac;
  double logn;
  uint64_t mask;
  int use_frac;
};

__device__ __forceinline__ bool table_full(const int* flags) {
  return __ldcg(flags + kFlagTableFull) != 0;
}

__global__ void k_table_init(Slot* __restrict__ T, uint64_t cap) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < cap; i += (uint64_t)gridDim.x * blockDim.x)
    T[i] = Slot{kEmptyKey, 0ULL};
}

// Linear-probe insert-or-add (par_table::insert_add, LightNE/par_table.h:86-109).
// Keys never change once written, so a stale read of a key is still a valid
// key; a stale EMPTY is resolved by the compare-and-swap.
template <bool WEIGHTED>
__device__ __forceinline__ bool table_insert_add(Slot* __restrict__ T, uint64_t mask, uint64_t key,
                                                 double w, int* flags, unsigned long long cnt = 1ULL) {
  uint64_t h = hash64_2(key) & mask;
  for (uint32_t p = 0; p < kMaxProbes; ++p) {
    unsigned long long k = __ldcg(&T[h].key);
    if (k == kEmptyKey) k = atomicCAS(&T[h].key, kEmptyKey, (unsigned long long)key);
    if (k == kEmptyKey || k == key) {
      if (WEIGHTED)
        atomicAdd(reinterpret_cast<double*>(&T[h].val), w);
      else
        atomicAdd(&T[h].val, cnt);
      return true;
    }
    h = (h + 1) & mask;
    if ((p & 1023u) == 1023u && table_full(flags)) return false;
  }
  atomicExch(flags + kFlagTableFull, 1);
  return false;
}

// Path sampler, one thread per directed CSR entry (u, v), over the entries
// [e0, e1): LightNE/PathEmbed.h:128-171.  The per-edge generator state is a
// chain (every draw advances it), so the samples of one edge are sequential.
// Every loop iteration makes exactly one draw (rand + next) and reduces it
// modulo the divisor of the current phase with that divisor's
// Granlund-Montgomery multiplier:
//   [eff test (-sample 1)] -> r = rand % T + 1 -> k = rand % r + 1 ->
//   k-1 steps from u, then r-k steps from v (rand % degree each)
// so the lanes of a warp execute the same instructions whatever phase each
// lane is in.  Emitted pair keys (and weights with -sample 1) are staged per
// warp in shared memory and written to the sample buffer 32 at a time, so
// the walk never waits on the pair table; k_insert adds them to the table.
static constexpr int kWalkThreads = 256;
static constexpr int kQueue = 64;    // staged keys per warp
static constexpr int kMaxRMagic = 64;  // multipliers of r = 1..64 kept in shared memory

enum WalkPhase : int { kPhEff = 0, kPhR = 1, kPhK = 2, kPhW1 = 3, kPhW2 = 4 };

template <bool SAMPLE>
__global__ void __launch_bounds__(kWalkThreads, 6) k_walk(const Vertex* __restrict__ vd, const uint32_t* __restrict__ nbrs,
                                                      const uint32_t* __restrict__ src, int64_t e0, int64_t e1,
                                                      SampleArgs a, unsigned long long* __restrict__ out_keys,
                                                      double* __restrict__ out_w,
                                                      unsigned long long* __restrict__ out_count, uint64_t out_cap,
                                                      int* flags) {
  __shared__ unsigned long long qk[kWalkThreads / 32][kQueue];
  __shared__ double qw[SAMPLE ? kWalkThreads / 32 : 1][SAMPLE ? kQueue : 1];
  __shared__ unsigned long long rmag[kMaxRMagic + 1];
  for (int i = threadIdx.x; i <= kMaxRMagic; i += blockDim.x) rmag[i] = gm_magic(i > 0 ? (uint32_t)i : 1u);
  __syncthreads();
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int64_t e = e0 + (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  bool active = e < e1;
  uint32_t u = 0, v = 0, cur = 0, x = 0, left1 = 0, left2 = 0, r = 0;
  uint32_t cur_off = 0, div = 1;
  uint64_t mag = 1;
  uint4 vu = make_uint4(0, 1, 1, 0), vv = make_uint4(0, 1, 1, 0);
  uint64_t s = 0, todo = 0;
  double p = 1.0, ipw = 1.0;
  int phase = SAMPLE ? kPhEff : kPhR;
  if (active) {
    u = __ldg(src + e);
    v = __ldg(nbrs + e);
    vu = __ldg(reinterpret_cast<const uint4*>(vd + u));
    vv = __ldg(reinterpret_cast<const uint4*>(vd + v));
    s = rng_fork(a.seed, ((uint64_t)u << 32) | (uint64_t)v);
    todo = a.exp_rv;
    if (a.use_frac) todo += (map_uint64(rng_draw(s)) < a.frac) ? 1u : 0u;
    if (SAMPLE) {
      p = __dmul_rn(__dadd_rn(__ddiv_rn(1.0, (double)vu.y), __ddiv_rn(1.0, (double)vv.y)), a.logn);
      p = p < 1.0 ? p : 1.0;
      ipw = __ddiv_rn(1.0, p);
    }
    active = todo > 0;
    div = (uint32_t)a.walk_len;
    mag = a.walk_magic;
  }
  int qlen = 0;  // warp-uniform
  while (__any_sync(kFullMask, active)) {
    bool emit = false;
    unsigned long long key = 0;
    if (active) {
      const uint64_t rnd = rng_draw(s);
      bool sample_done = false;
      if (SAMPLE && phase == kPhEff) {
        if (map_uint64(rnd) < p) {
          phase = kPhR;
          div = (uint32_t)a.walk_len;
          mag = a.walk_magic;
        } else {
          sample_done = true;
        }
      } else {
        const uint32_t m = gm_mod(rnd, div, mag);
        if (phase == kPhR) {
          r = m + 1;
          phase = kPhK;
          div = r;
          mag = r <= kMaxRMagic ? rmag[r] : gm_magic(r);
        } else {
          uint32_t nxt = 0;
          bool to_v = false, end_walk = false;
          if (phase == kPhK) {
            const uint32_t k = m + 1;
            left1 = k - 1;
            left2 = r - k;
            if (left1 > 0) {
              phase = kPhW1;
              cur = u;
              cur_off = vu.x;
              div = vu.y;
              mag = ((uint64_t)vu.w << 32) | vu.z;
            } else {
              x = u;
              to_v = true;
            }
          } else {
            nxt = __ldg(nbrs + cur_off + m);
            cur = nxt;
            if (phase == kPhW1) {
              if (--left1 == 0) {
                x = cur;
                to_v = true;
              }
            } else if (--left2 == 0) {
              end_walk = true;
            }
            if (!to_v && !end_walk) {
              const uint4 rw = __ldg(reinterpret_cast<const uint4*>(vd + cur));
              cur_off = rw.x;
              div = rw.y;
              mag = ((uint64_t)rw.w << 32) | rw.z;
              if (div == 0) active = false;  // unreachable for a validated (symmetric) graph
            }
          }
          if (to_v) {
            cur = v;
            if (left2 > 0) {
              phase = kPhW2;
              cur_off = vv.x;
              div = vv.y;
              mag = ((uint64_t)vv.w << 32) | vv.z;
            } else {
              end_walk = true;
            }
          }
          if (end_walk) {
            const uint32_t lo = x < cur ? x : cur, hi = x < cur ? cur : x;
            key = ((uint64_t)lo << 32) + (uint64_t)hi;
            emit = true;
            sample_done = true;
          }
        }
      }
      if (sample_done) {
        if (--todo == 0) {
          active = false;
        } else {
          phase = SAMPLE ? kPhEff : kPhR;
          div = (uint32_t)a.walk_len;
          mag = a.walk_magic;
        }
      }
    }
    // stage this iteration's keys in the warp queue
    const unsigned em = __ballot_sync(kFullMask, emit);
    if (emit) {
      const int pos = qlen + __popc(em & ((1u << lane) - 1));
      qk[wid][pos] = key;
      if (SAMPLE) qw[wid][pos] = ipw;
    }
    qlen += __popc(em);
    __syncwarp();
    if (qlen >= 32) {
      unsigned long long base = 0;
      if (lane == 0) base = atomicAdd(out_count, 32ULL);
      base = __shfl_sync(kFullMask, base, 0);
      if (base + 32 <= out_cap) {
        out_keys[base + lane] = qk[wid][lane];
        if (SAMPLE) out_w[base + lane] = qw[wid][lane];
      } else if (lane == 0) {
        atomicExch(flags + kFlagSortOverflow, 1);
      }
      __syncwarp();
      if (lane < qlen - 32) {
        qk[wid][lane] = qk[wid][32 + lane];
        if (SAMPLE) qw[wid][lane] = qw[wid][32 + lane];
      }
      qlen -= 32;
      __syncwarp();
    }
  }
  if (qlen > 0) {
    unsigned long long base = 0;
    if (lane == 0) base = atomicAdd(out_count, (unsigned long long)qlen);
    base = __shfl_sync(kFullMask, base, 0);
    if (lane < qlen) {
      if (base + lane < out_cap) {
        out_keys[base + lane] = qk[wid][lane];
        if (SAMPLE) out_w[base + lane] = qw[wid][lane];
      } else {
        atomicExch(flags + kFlagSortOverflow, 1);
      }
    }
  }
}

// Adds every staged key to the pair table (par_table::insert_add).  For
// counts, the lanes of a warp that hold the same key are merged first
// (match.any) and one of them adds their number: hub pairs recur often.
template <bool WEIGHTED>
__global__ void k_insert(const unsigned long long* __restrict__ keys, const double* __restrict__ w, uint64_t count,
                         Slot* __restrict__ table, uint64_t mask, int* flags) {
  const int lane = threadIdx.x & 31;
  const uint64_t nwarp = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  for (uint64_t wb = (((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5) * 32; wb < count; wb += nwarp * 32) {
    const uint64_t i = wb + lane;
    const bool have = i < count;
    const unsigned long long key = have ? keys[i] : kEmptyKey;
    if (WEIGHTED) {
      if (have && !table_insert_add<true>(table, mask, key, w[i], flags)) return;
    } else {
      const unsigned same = __match_any_sync(kFullMask, key);
      const bool leader = have && (__ffs(same) - 1) == lane;
      if (leader && !table_insert_add<false>(table, mask, key, 1.0, flags, (unsigned long long)__popc(same))) return;
    }
  }
}

// Sum of weights and number of occupied slots (PathEmbed.h:175-188).  Counts
// are integers and summed exactly; weights (sample mode) are summed per block
// and then in block order, so the result depends only on the table layout.
template <bool WEIGHTED>
__global__ void k_table_sum(const Slot* __restrict__ T, uint64_t cap, unsigned long long* __restrict__ cnt,
                            unsigned long long* __restrict__ distinct, double* __restrict__ block_w) {
  unsigned long long c = 0, dcount = 0;
  double w = 0.0;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < cap; i += (uint64_t)gridDim.x * blockDim.x) {
    const Slot s = T[i];
    if (s.key != kEmptyKey) {
      ++dcount;
      if (WEIGHTED)
        w += __longlong_as_double((long long)s.val);
      else
        c += s.val;
    }
  }
  __shared__ double sw[32];
  __shared__ unsigned long long sc[32], sd[32];
  for (int o = 16; o > 0; o >>= 1) {
    c += __shfl_down_sync(0xffffffffu, c, o);
    dcount += __shfl_down_sync(0xffffffffu, dcount, o);
    w += __shfl_down_sync(0xffffffffu, w, o);
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) { sc[wid] = c; sd[wid] = dcount; sw[wid] = w; }
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long tc = 0, td = 0;
    double tw = 0.0;
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) { tc += sc[i]; td += sd[i]; tw += sw[i]; }
    if (tc) atomicAdd(cnt, tc);
    if (td) atomicAdd(distinct, td);
    block_w[blockIdx.x] = tw;
  }
}

__global__ void k_sum_blocks(const double* __restrict__ block_w, int nb, double* out) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    double s = 0.0;
    for (int i = 0; i < nb; ++i) s += block_w[i];
    *out = s;
  }
}

// log(adj) as the reference's double result: CUDA's log (within 1 ulp) where
// that cannot change the float the value is narrowed to, otherwise the
// correctly rounded double from the double-double evaluation.
__device__ __forceinline__ double trunc_log_value(double adj) {
  double L = log(adj);
  if (float_rounding_is_close(L)) {
    const dd r = log_dd(adj);
    L = __dadd_rn(r.hi, r.lo);
  }
  return L;
}

__global__ void k_trunc_log_values(const double* __restrict__ x, int64_t n, double* __restrict__ out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = trunc_log_value(x[i]);
}

// Trunc-log map (PathEmbed.h:203-218) fused with the per-row counts of the
// CSR build (PathEmbed.h:226-288).  Kept slots get the float bits of the
// log value in `val`; dropped slots become empty.
//
// Counts (-sample 0): adj = ((w * factor) / d_u) / d_v is reproduced
// exactly by integer arithmetic (the reference's three double roundings),
// adj > 1 decides the keep test exactly, and log(adj) is evaluated in
// double-float; only values whose narrowing to float the double-float
// result cannot decide go through FP64 (trunc_log_value).  Weights
// (-sample 1) take the FP64 path throughout.
template <bool WEIGHTED>
__global__ void __launch_bounds__(256) k_trunclog(Slot* __restrict__ T, uint64_t cap, const Vertex* __restrict__ vd,
                                                  double factor, int upper, const LogTable* __restrict__ ltab,
                                                  unsigned long long* __restrict__ rowcnt,
                                                  unsigned long long* __restrict__ kept_total) {
  __shared__ LogTable tab;
  for (int i = threadIdx.x; i < 128; i += blockDim.x) {
    tab.log_hi[i] = ltab->log_hi[i];
    tab.log_lo[i] = ltab->log_lo[i];
    tab.inv_hi[i] = ltab->inv_hi[i];
    tab.inv_lo[i] = ltab->inv_lo[i];
  }
  __syncthreads();
  const XDouble xf = xd_from_double(factor);
  unsigned long long kept = 0;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < cap; i += (uint64_t)gridDim.x * blockDim.x) {
    const unsigned long long key = T[i].key;
    if (key == kEmptyKey) continue;
    const uint32_t u = (uint32_t)(key >> 32), v = (uint32_t)key;
    const uint4 ru = __ldg(reinterpret_cast<const uint4*>(vd + u));
    const uint4 rv = __ldg(reinterpret_cast<const uint4*>(vd + v));
    const unsigned long long raw = T[i].val;
    float f = 0.0f;
    bool keep;
    if (WEIGHTED) {
      double w = __longlong_as_double((long long)raw);
      if (u == v) w = __dmul_rn(w, 2.0);
      const double adj = __ddiv_rn(__ddiv_rn(__dmul_rn(w, factor), (double)ru.y), (double)rv.y);
      const double L = trunc_log_value(adj);
      keep = L > 0.0;
      if (keep) f = __double2float_rn(L);
    } else {
      const XDouble adj = trunc_log_adj(raw, u == v, xf, ru.y, ((uint64_t)ru.w << 32) | ru.z, rv.y,
                                        ((uint64_t)rv.w << 32) | rv.z);
      keep = adj.e > -52 || (adj.e == -52 && adj.m > (1ull << 52));  // adj > 1  <=>  log(adj) > 0
      if (keep && !float_of_log_fast(log_df(adj, tab), &f)) f = __double2float_rn(trunc_log_value(xd_to_double(adj)));
    }
    if (keep) {
      T[i].val = (unsigned long long)__float_as_uint(f);
      atomicAdd(&rowcnt[u], 1ULL);
      if (!upper && u != v) atomicAdd(&rowcnt[v], 1ULL);
      ++kept;
    } else {
      T[i].key = kEmptyKey;
    }
  }
  for (int o = 16; o > 0; o >>= 1) kept += __shfl_down_sync(0xffffffffu, kept, o);
  if ((threadIdx.x & 31) == 0 && kept) atomicAdd(kept_total, kept);
}

// Scatter each kept entry into its row (and the mirrored row unless -upper),
// PathEmbed.h:300-311.  rowcnt serves as a decrementing cursor.
__global__ void k_scatter(const Slot* __restrict__ T, uint64_t cap, const int64_t* __restrict__ row_ptr,
                          unsigned long long* __restrict__ cursor, int upper, uint64_t* __restrict__ packed) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < cap; i += (uint64_t)gridDim.x * blockDim.x) {
    const unsigned long long key = T[i].key;
    if (key == kEmptyKey) continue;
    const uint32_t u = (uint32_t)(key >> 32), v = (uint32_t)key;
    const uint64_t fb = (uint32_t)T[i].val;
    unsigned long long p = atomicAdd(&cursor[u], ~0ULL) - 1ULL;  // decrement
    packed[row_ptr[u] + (int64_t)p] = ((uint64_t)v << 32) | fb;
    if (!upper && u != v) {
      p = atomicAdd(&cursor[v], ~0ULL) - 1ULL;
      packed[row_ptr[v] + (int64_t)p] = ((uint64_t)u << 32) | fb;
    }
  }
}

// ---------------------------------------------------------------------------
// Per-row sort of the packed entries (ascending column), by row length class.
// All classes use the ascending bitonic network in which the first
// comparator of each merge stage pairs i with i ^ (k-1) and the following
// ones pair i with i ^ j.  Every comparator keeps the minimum at the lower
// index, so a row of length L sorts in place as if padded with +inf up to
// the next power of two: comparators that touch an index >= L never swap.
// Rows longer than kCapXL are cut into kCapXL-entry segments sorted the same
// way, then merged pairwise in global memory (merge path).
// ---------------------------------------------------------------------------
enum RowClass { kClsWarp = 0, kClsS = 1, kClsM = 2, kClsL = 3, kClsXL = 4, kClsHuge = 5, kNumCls = 6 };
static constexpr int kCapS = 256, kCapM = 1024, kCapL = 4096, kCapXL = 16384;

struct Segment {  // a run of packed entries to sort in shared memory
  int64_t start;
  int32_t len;
  int32_t final_;  // 1: a whole row, write col/val; 0: a chunk of a long row
};

__device__ __forceinline__ void unpack_store(uint64_t x, int32_t* col, float* val, int64_t j) {
  col[j] = (int32_t)(x >> 32);
  val[j] = __uint_as_float((uint32_t)x);
}

// cls_cnt: [kNumCls] counts, [kNumCls] = total entries of huge rows,
// [kNumCls + 1] = longest huge row.
__global__ void k_classify_rows(const int64_t* __restrict__ row_ptr, int64_t n, const uint64_t* __restrict__ packed,
                                int32_t* __restrict__ col, float* __restrict__ val, unsigned long long* __restrict__ cls_cnt,
                                uint32_t* __restrict__ cls_rows, int64_t list_stride, Segment* __restrict__ segs) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int64_t a = row_ptr[i], L = row_ptr[i + 1] - a;
  if (L == 0) return;
  if (L == 1) {
    unpack_store(packed[a], col, val, a);
    return;
  }
  if (L <= kCapL) {
    const int c = L <= 32 ? kClsWarp : L <= kCapS ? kClsS : L <= kCapM ? kClsM : kClsL;
    const unsigned long long slot = atomicAdd(&cls_cnt[c], 1ULL);
    cls_rows[(int64_t)c * list_stride + (int64_t)slot] = (uint32_t)i;
    return;
  }
  if (L <= kCapXL) {
    const unsigned long long slot = atomicAdd(&cls_cnt[kClsXL], 1ULL);
    segs[slot] = Segment{a, (int32_t)L, 1};
    return;
  }
  const int64_t nseg = (L + kCapXL - 1) / kCapXL;
  const unsigned long long s0 = atomicAdd(&cls_cnt[kClsXL], (unsigned long long)nseg);
  for (int64_t c = 0; c < nseg; ++c) {
    const int64_t b = c * kCapXL;
    const int64_t len = (L - b) < kCapXL ? (L - b) : kCapXL;
    segs[s0 + c] = Segment{a + b, (int32_t)len, 0};
  }
  const unsigned long long h = atomicAdd(&cls_cnt[kClsHuge], 1ULL);
  cls_rows[(int64_t)kClsHuge * list_stride + (int64_t)h] = (uint32_t)i;
  atomicAdd(&cls_cnt[kNumCls], (unsigned long long)L);
  atomicMax(&cls_cnt[kNumCls + 1], (unsigned long long)L);
}

__global__ void k_sort_warp_rows(const int64_t* __restrict__ row_ptr, const unsigned long long* __restrict__ cls_cnt,
                                 const uint32_t* __restrict__ rows, const uint64_t* __restrict__ packed,
                                 int32_t* __restrict__ col, float* __restrict__ val) {
  const int lane = threadIdx.x & 31;
  const int64_t nrows = (int64_t)cls_cnt[kClsWarp];
  for (int64_t w = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; w < nrows;
       w += ((int64_t)gridDim.x * blockDim.x) >> 5) {
    const uint32_t r = rows[w];
    const int64_t a = row_ptr[r];
    const int L = (int)(row_ptr[r + 1] - a);
    uint64_t x = lane < L ? packed[a + lane] : ~0ULL;
#pragma unroll
    for (int k = 2; k <= 32; k <<= 1) {
#pragma unroll
      for (int j = k >> 1; j > 0; j >>= 1) {
        const int partner = (j == (k >> 1)) ? (lane ^ (k - 1)) : (lane ^ j);
        const uint64_t y = __shfl_sync(0xffffffffu, x, partner);
        const bool low = lane < partner;
        x = low ? (x < y ? x : y) : (x < y ? y : x);
      }
    }
    if (lane < L) unpack_store(x, col, val, a + lane);
  }
}

__device__ __forceinline__ void bitonic_smem(uint64_t* s, int L) {
  int N = 1;
  while (N < L) N <<= 1;
  const int half = N >> 1;
  for (int k = 2; k <= N; k <<= 1) {
    for (int j = k >> 1; j > 0; j >>= 1) {
      for (int c = threadIdx.x; c < half; c += blockDim.x) {
        int i, l;
        if (j == (k >> 1)) {
          const int blk = c / j, pos = c % j;
          i = blk * k + pos;
          l = blk * k + k - 1 - pos;
        } else {
          i = (c / j) * 2 * j + (c % j);
          l = i + j;
        }
        if (l < L) {
          const uint64_t x = s[i], y = s[l];
          if (x > y) { s[i] = y; s[l] = x; }
        }
      }
      __syncthreads();
    }
  }
}

template <int CLS>
__global__ void k_sort_block_rows(const int64_t* __restrict__ row_ptr, const unsigned long long* __restrict__ cls_cnt,
                                  const uint32_t* __restrict__ rows, const uint64_t* __restrict__ packed,
                                  int32_t* __restrict__ col, float* __restrict__ val) {
  extern __shared__ uint64_t sbuf[];
  const int64_t nrows = (int64_t)cls_cnt[CLS];
  for (int64_t w = blockIdx.x; w < nrows; w += gridDim.x) {
    const uint32_t r = rows[w];
    const int64_t a = row_ptr[r];
    const int L = (int)(row_ptr[r + 1] - a);
    for (int i = threadIdx.x; i < L; i += blockDim.x) sbuf[i] = packed[a + i];
    __syncthreads();
    bitonic_smem(sbuf, L);
    for (int i = threadIdx.x; i < L; i += blockDim.x) unpack_store(sbuf[i], col, val, a + i);
    __syncthreads();
  }
}

// Segments of up to kCapXL entries: whole rows write col/val, chunks of
// long rows are written back sorted in place for the merge passes.
__global__ void k_sort_segments(const unsigned long long* __restrict__ cls_cnt, const Segment* __restrict__ segs,
                                uint64_t* __restrict__ packed, int32_t* __restrict__ col, float* __restrict__ val) {
  extern __shared__ uint64_t sbuf[];
  const int64_t nseg = (int64_t)cls_cnt[kClsXL];
  for (int64_t w = blockIdx.x; w < nseg; w += gridDim.x) {
    const Segment sg = segs[w];
    for (int i = threadIdx.x; i < sg.len; i += blockDim.x) sbuf[i] = packed[sg.start + i];
    __syncthreads();
    bitonic_smem(sbuf, sg.len);
    if (sg.final_) {
      for (int i = threadIdx.x; i < sg.len; i += blockDim.x) unpack_store(sbuf[i], col, val, sg.start + i);
    } else {
      for (int i = threadIdx.x; i < sg.len; i += blockDim.x) packed[sg.start + i] = sbuf[i];
    }
    __syncthreads();
  }
}

// One merge pass over the long rows: runs of `run` sorted entries are merged
// pairwise from `src` into `dst` (same offsets).  One block per (row, pair);
// each thread finds its split of the merged output by binary search along
// the merge-path diagonal and merges its share sequentially.  The last pass
// writes col/val instead of dst.
__global__ void k_merge_pass(const int64_t* __restrict__ row_ptr, const unsigned long long* __restrict__ cls_cnt,
                             const uint32_t* __restrict__ rows, const uint64_t* __restrict__ src,
                             uint64_t* __restrict__ dst, int64_t run, int last, int32_t* __restrict__ col,
                             float* __restrict__ val) {
  const int64_t nrows = (int64_t)cls_cnt[kClsHuge];
  for (int64_t w = blockIdx.x; w < nrows; w += gridDim.x) {
    const uint32_t r = rows[w];
    const int64_t base = row_ptr[r];
    const int64_t L = row_ptr[r + 1] - base;
    for (int64_t p0 = 0; p0 < L; p0 += 2 * run) {
      const int64_t na = (L - p0) < run ? (L - p0) : run;
      const int64_t rest = L - p0 - na;
      const int64_t nb = rest < run ? rest : run;
      const uint64_t* A = src + base + p0;
      const uint64_t* B = A + na;
      const int64_t tot = na + nb;
      const int64_t per = (tot + blockDim.x - 1) / blockDim.x;
      const int64_t d0 = (int64_t)threadIdx.x * per;
      if (d0 < tot) {
        const int64_t d1 = (d0 + per) < tot ? (d0 + per) : tot;
        // largest i in [max(0, d0-nb), min(d0, na)] with A[i-1] <= B[d0-i]
        int64_t lo = d0 - nb > 0 ? d0 - nb : 0, hi = d0 < na ? d0 : na;
        while (lo < hi) {
          const int64_t mid = (lo + hi + 1) >> 1;
          if (A[mid - 1] <= B[d0 - mid]) lo = mid; else hi = mid - 1;
        }
        int64_t i = lo, j = d0 - lo;
        for (int64_t o = d0; o < d1; ++o) {
          uint64_t x;
          if (j >= nb || (i < na && A[i] <= B[j])) x = A[i++]; else x = B[j++];
          if (last) unpack_store(x, col, val, base + p0 + o); else dst[base + p0 + o] = x;
        }
      }
    }
  }
}

static unsigned grid_for(int64_t items, int threads, int64_t cap_blocks) {
  int64_t b = (items + threads - 1) / threads;
  if (b < 1) b = 1;
  if (b > cap_blocks) b = cap_blocks;
  return (unsigned)b;
}

}  // namespace lne

using namespace lne;

namespace {

struct Scratch {
  lne_ctx* ctx;
  void* p[12] = {};
  int k = 0;
  explicit Scratch(lne_ctx* c) : ctx(c) {}
  int get(void** out, size_t bytes, const char* what) {
    int rc = dalloc(ctx, out, bytes, what);
    if (rc == LNE_OK) p[k++] = *out;
    return rc;
  }
  void release(void* q) {
    for (int i = 0; i < k; ++i)
      if (p[i] == q) { dfree(ctx, q); p[i] = nullptr; }
  }
  ~Scratch() {
    for (int i = 0; i < k; ++i) dfree(ctx, p[i]);
  }
};

struct Events {
  cudaEvent_t e[5] = {};
  Events() { for (auto& x : e) cudaEventCreate(&x); }
  ~Events() { for (auto& x : e) cudaEventDestroy(x); }
};

}  // namespace

extern "C" int lne_sparsify(lne_ctx* ctx, const lne_graph* g, const lne_sparsify_params* p, lne_csr** out,
                            lne_sparsify_stats* stats) {
  LNE_CHECK_ARG(ctx && g && p && out, "lne_sparsify: NULL argument");
  *out = nullptr;
  LNE_CHECK_ARG(p->walk_len >= 1 && p->walk_len < (int64_t)1 << 31, "lne_sparsify: walk_len must be in [1, 2^31)");
  LNE_CHECK_ARG(p->negative >= 1, "lne_sparsify: negative must be >= 1");
  LNE_CHECK_ARG(p->table_size >= 0, "lne_sparsify: table_size must be >= 0");
  LNE_CHECK_ARG(g->m_dir >= 1, "lne_sparsify: the graph has no edges");
  LNE_CUDA_TRY(cudaSetDevice(ctx->device));
  cudaStream_t st = ctx->stream;
  const int64_t n = g->n, m_dir = g->m_dir;

  // Sampling parameters in the reference's evaluation order (PathEmbed.h:89-117).
  const double logn = log((double)(size_t)n);
  size_t table_size = (size_t)((double)((size_t)p->walk_len * (size_t)n) * logn * (double)p->mem_ratio);
  if ((size_t)p->table_size > table_size) table_size = (size_t)p->table_size;
  size_t bits = 0;
  for (size_t b = 2 * table_size - 1; b > 0; b >>= 1) ++bits;  // pbbslib::log2_up(2 * table_size)
  if (bits > 40) { set_error("lne_sparsify: table capacity above 2^40 slots"); return LNE_ERR_UNSUPPORTED; }
  const uint64_t cap = (uint64_t)1 << bits;
  const double M = (double)((size_t)p->walk_len * (size_t)n) * logn * (double)p->sample_ratio;
  const double inv_lambda = M / (double)(size_t)m_dir;
  const size_t exp_rv = (size_t)inv_lambda;
  const double frac = inv_lambda - (double)exp_rv;

  Scratch S(ctx);
  Events ev;
  Slot* table = nullptr;
  unsigned long long* counters = nullptr;  // [0] emitted [1] count sum [2] distinct [3] kept
  double* wsum = nullptr;
  int rc;
  if ((rc = S.get((void**)&table, sizeof(Slot) * cap, "pair table"))) return rc;
  const int sum_blocks = 1024;
  if ((rc = S.get((void**)&counters, 64 + sizeof(double) * (sum_blocks + 1), "counters"))) return rc;
  wsum = (double*)((char*)counters + 64);
  k_table_init<<<grid_for((int64_t)cap, 256, (int64_t)ctx->num_sms * 32), 256, 0, st>>>(table, cap);
  LNE_CUDA_TRY(cudaMemsetAsync(counters, 0, 64, st));
  LNE_CUDA_TRY(cudaMemsetAsync(ctx->d_flags, 0, sizeof(int) * kFlagWords, st));

  SampleArgs a;
  a.seed = p->seed;
  a.walk_len = (uint64_t)p->walk_len;
  a.walk_magic = gm_magic((uint32_t)p->walk_len);
  a.exp_rv = (uint64_t)exp_rv;
  a.frac = frac;
  a.logn = logn;
  a.mask = cap - 1;
  a.use_frac = frac > 0.0000000001 ? 1 : 0;

  cudaEventRecord(ev.e[0], st);
  // Sample buffer: at most exp_rv + 1 samples per directed entry; the edge
  // range is processed in batches that fit the buffer.
  const uint64_t per_edge = (uint64_t)exp_rv + 1;
  const uint64_t want_keys = per_edge * (uint64_t)m_dir;
  const uint64_t max_keys = (uint64_t)1 << 30;  // 8 GiB of keys per batch
  const uint64_t buf_keys = want_keys < max_keys ? want_keys : max_keys;
  const int64_t edges_per_batch = (int64_t)std::max<uint64_t>(1, buf_keys / per_edge);
  unsigned long long* keys = nullptr;
  double* wts = nullptr;
  if ((rc = S.get((void**)&keys, sizeof(unsigned long long) * buf_keys, "sample buffer"))) return rc;
  if (p->sample && (rc = S.get((void**)&wts, sizeof(double) * buf_keys, "sample weights"))) return rc;
  int launches_sample = 0;
  unsigned long long emitted_total = 0;
  for (int64_t eb = 0; eb < m_dir; eb += edges_per_batch) {
    const int64_t ee = std::min<int64_t>(m_dir, eb + edges_per_batch);
    LNE_CUDA_TRY(cudaMemsetAsync(counters, 0, 8, st));
    const unsigned wblocks = (unsigned)((ee - eb + kWalkThreads - 1) / kWalkThreads);
    if (p->sample)
      k_walk<true><<<wblocks, kWalkThreads, 0, st>>>(g->vdata, g->nbrs, g->src, eb, ee, a, keys, wts, counters,
                                                     buf_keys, ctx->d_flags);
    else
      k_walk<false><<<wblocks, kWalkThreads, 0, st>>>(g->vdata, g->nbrs, g->src, eb, ee, a, keys, wts, counters,
                                                      buf_keys, ctx->d_flags);
    unsigned long long got = 0;
    LNE_CUDA_TRY(cudaMemcpyAsync(&got, counters, 8, cudaMemcpyDeviceToHost, st));
    LNE_CUDA_TRY(cudaStreamSynchronize(st));
    if (got > buf_keys) got = buf_keys;  // overflow is flagged and reported below
    const unsigned iblocks = grid_for((int64_t)got, 256, (int64_t)ctx->num_sms * 32);
    if (p->sample)
      k_insert<true><<<iblocks, 256, 0, st>>>(keys, wts, got, table, cap - 1, ctx->d_flags);
    else
      k_insert<false><<<iblocks, 256, 0, st>>>(keys, wts, got, table, cap - 1, ctx->d_flags);
    emitted_total += got;
    launches_sample += 2;
  }
  LNE_CUDA_TRY(cudaGetLastError());
  S.release(keys);
  if (wts) S.release(wts);
  cudaEventRecord(ev.e[1], st);

  const unsigned tgrid = grid_for((int64_t)cap, 256, (int64_t)ctx->num_sms * 16);
  const int sgrid = sum_blocks;
  if (p->sample)
    k_table_sum<true><<<sgrid, 256, 0, st>>>(table, cap, counters + 1, counters + 2, wsum);
  else
    k_table_sum<false><<<sgrid, 256, 0, st>>>(table, cap, counters + 1, counters + 2, wsum);
  k_sum_blocks<<<1, 32, 0, st>>>(wsum, sgrid, wsum + sum_blocks);
  unsigned long long h_cnt[3] = {0, 0, 0};
  LNE_CUDA_TRY(cudaMemsetAsync(counters, 0, 8, st));
  double h_w = 0.0;
  int h_flags[kFlagWords];
  LNE_CUDA_TRY(cudaMemcpyAsync(h_cnt, counters, sizeof(h_cnt), cudaMemcpyDeviceToHost, st));
  LNE_CUDA_TRY(cudaMemcpyAsync(&h_w, wsum + sum_blocks, sizeof(double), cudaMemcpyDeviceToHost, st));
  LNE_CUDA_TRY(cudaMemcpyAsync(h_flags, ctx->d_flags, sizeof(h_flags), cudaMemcpyDeviceToHost, st));
  LNE_CUDA_TRY(cudaStreamSynchronize(st));
  LNE_CUDA_TRY(cudaGetLastError());
  h_cnt[0] = emitted_total;
  if (h_flags[kFlagSortOverflow]) {
    set_error("lne_sparsify: sample buffer overflow (internal sizing error)");
    return LNE_ERR_UNSUPPORTED;
  }
  if (h_flags[kFlagTableFull]) {
    char buf[256];
    snprintf(buf, sizeof(buf),
             "lne_sparsify: pair table full (capacity %llu slots); raise -tablesz "
             "(the reference prints \"looping forever\" and exits)",
             (unsigned long long)cap);
    set_error(buf);
    return LNE_ERR_TABLE_FULL;
  }
  const double M_exact = p->sample ? h_w : (double)h_cnt[1];
  // factor = vol * m / M_exact / 2 / negative, left to right (PathEmbed.h:199-200)
  const double vol = (double)(size_t)m_dir;
  const double factor = vol * (double)(size_t)m_dir / M_exact / 2 / (double)(size_t)p->negative;

  unsigned long long* rowcnt = nullptr;
  int64_t* row_ptr = nullptr;
  void* scan_tmp = nullptr;
  if ((rc = S.get((void**)&rowcnt, sizeof(unsigned long long) * n, "row counts"))) return rc;
  if ((rc = dalloc(ctx, (void**)&row_ptr, sizeof(int64_t) * (n + 1), "row_ptr"))) return rc;
  if ((rc = S.get(&scan_tmp, scan_tmp_bytes(n), "scan scratch"))) { dfree(ctx, row_ptr); return rc; }
  LNE_CUDA_TRY(cudaMemsetAsync(rowcnt, 0, sizeof(unsigned long long) * n, st));
  if (p->sample)
    k_trunclog<true><<<tgrid, 256, 0, st>>>(table, cap, g->vdata, factor, p->upper,
                                            (const LogTable*)ctx->log_table, rowcnt, counters + 3);
  else
    k_trunclog<false><<<tgrid, 256, 0, st>>>(table, cap, g->vdata, factor, p->upper,
                                             (const LogTable*)ctx->log_table, rowcnt, counters + 3);
  cudaEventRecord(ev.e[2], st);
  scan_exclusive_i64((const int64_t*)rowcnt, row_ptr, n, scan_tmp, st);
  int64_t nnz = 0;
  unsigned long long kept = 0;
  LNE_CUDA_TRY(cudaMemcpyAsync(&nnz, row_ptr + n, 8, cudaMemcpyDeviceToHost, st));
  LNE_CUDA_TRY(cudaMemcpyAsync(&kept, counters + 3, 8, cudaMemcpyDeviceToHost, st));
  LNE_CUDA_TRY(cudaStreamSynchronize(st));
  LNE_CUDA_TRY(cudaGetLastError());

  uint64_t* packed = nullptr;
  if ((rc = S.get((void**)&packed, sizeof(uint64_t) * (nnz > 0 ? nnz : 1), "packed entries"))) {
    dfree(ctx, row_ptr);
    return rc;
  }
  k_scatter<<<tgrid, 256, 0, st>>>(table, cap, row_ptr, rowcnt, p->upper, packed);
  S.release(table);
  S.release(rowcnt);

  int32_t* col = nullptr;
  float* val = nullptr;
  unsigned long long* cls_cnt = nullptr;
  uint32_t* cls_rows = nullptr;
  Segment* segs = nullptr;
  const int64_t max_segs = n + nnz / kCapXL + 8;
  if ((rc = dalloc(ctx, (void**)&col, sizeof(int32_t) * (nnz > 0 ? nnz : 1), "csr col")) ||
      (rc = dalloc(ctx, (void**)&val, sizeof(float) * (nnz > 0 ? nnz : 1), "csr val")) ||
      (rc = S.get((void**)&cls_cnt, sizeof(unsigned long long) * 16, "row classes")) ||
      (rc = S.get((void**)&cls_rows, sizeof(uint32_t) * kNumCls * n, "row class lists")) ||
      (rc = S.get((void**)&segs, sizeof(Segment) * max_segs, "sort segments"))) {
    dfree(ctx, row_ptr);
    dfree(ctx, col);
    dfree(ctx, val);
    return rc;
  }
  LNE_CUDA_TRY(cudaMemsetAsync(cls_cnt, 0, sizeof(unsigned long long) * 16, st));
  int launches = 13 + launches_sample;  // 7 + walk/insert before this point, 6 sort launches below
  k_classify_rows<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(row_ptr, n, packed, col, val, cls_cnt, cls_rows, n,
                                                               segs);
  const int64_t sms = ctx->num_sms;
  k_sort_warp_rows<<<(unsigned)(sms * 16), 256, 0, st>>>(row_ptr, cls_cnt, cls_rows + (int64_t)kClsWarp * n, packed,
                                                          col, val);
  k_sort_block_rows<kClsS><<<(unsigned)(sms * 16), 128, kCapS * 8, st>>>(row_ptr, cls_cnt, cls_rows + (int64_t)kClsS * n,
                                                                         packed, col, val);
  k_sort_block_rows<kClsM><<<(unsigned)(sms * 8), 256, kCapM * 8, st>>>(row_ptr, cls_cnt, cls_rows + (int64_t)kClsM * n,
                                                                        packed, col, val);
  k_sort_block_rows<kClsL><<<(unsigned)(sms * 4), 512, kCapL * 8, st>>>(row_ptr, cls_cnt, cls_rows + (int64_t)kClsL * n,
                                                                        packed, col, val);
  cudaFuncSetAttribute(k_sort_segments, cudaFuncAttributeMaxDynamicSharedMemorySize, kCapXL * 8);
  k_sort_segments<<<(unsigned)sms, 1024, kCapXL * 8, st>>>(cls_cnt, segs, packed, col, val);
  unsigned long long h_cls[16];
  LNE_CUDA_TRY(cudaMemcpyAsync(h_cls, cls_cnt, sizeof(h_cls), cudaMemcpyDeviceToHost, st));
  LNE_CUDA_TRY(cudaStreamSynchronize(st));
  if (h_cls[kClsHuge] > 0) {
    uint64_t* other = nullptr;
    if ((rc = S.get((void**)&other, sizeof(uint64_t) * (nnz > 0 ? nnz : 1), "merge buffer"))) {
      dfree(ctx, row_ptr);
      dfree(ctx, col);
      dfree(ctx, val);
      return rc;
    }
    const int64_t maxL = (int64_t)h_cls[kNumCls + 1];
    uint64_t* src = packed;
    uint64_t* dst = other;
    const unsigned mgrid = (unsigned)std::min<int64_t>((int64_t)h_cls[kClsHuge], sms * 8);
    for (int64_t run = kCapXL; run < maxL; run *= 2) {
      const int last = (2 * run >= maxL) ? 1 : 0;
      k_merge_pass<<<mgrid, 512, 0, st>>>(row_ptr, cls_cnt, cls_rows + (int64_t)kClsHuge * n, src, dst, run, last,
                                          col, val);
      ++launches;
      uint64_t* t = src;
      src = dst;
      dst = t;
    }
  }
  cudaEventRecord(ev.e[3], st);
  cudaError_t le = cudaGetLastError();
  if (le != cudaSuccess) {
    dfree(ctx, row_ptr);
    dfree(ctx, col);
    dfree(ctx, val);
    set_error(std::string("lne_sparsify: kernel launch failed: ") + cudaGetErrorString(le));
    return LNE_ERR_CUDA;
  }
  if (stats) {
    LNE_CUDA_TRY(cudaEventSynchronize(ev.e[3]));
    stats->logn = logn;
    stats->total_samples = M;
    stats->inv_lambda = inv_lambda;
    stats->frac = frac;
    stats->factor = factor;
    stats->m_exact = M_exact;
    stats->exp_rv_rounded = (int64_t)exp_rv;
    stats->table_size = (int64_t)table_size;
    stats->capacity = (int64_t)cap;
    stats->samples_emitted = (int64_t)h_cnt[0];
    stats->distinct = (int64_t)h_cnt[2];
    stats->nnz_upper = (int64_t)kept;
    stats->nnz = nnz;
    cudaEventElapsedTime(&stats->ms_sample, ev.e[0], ev.e[1]);
    cudaEventElapsedTime(&stats->ms_trunclog, ev.e[1], ev.e[2]);
    cudaEventElapsedTime(&stats->ms_csr, ev.e[2], ev.e[3]);
    // init, sample, table sum, block sum, trunc-log, 3 scan, scatter,
    // classify, 5 row-sort classes, merge passes
    stats->kernel_launches = launches;
  }
  lne_csr* c = new lne_csr();
  c->n = n;
  c->nnz = nnz;
  c->row_ptr = row_ptr;
  c->col = col;
  c->val = val;
  c->owned = true;
  c->stream = st;
  *out = c;
  return LNE_OK;
}

extern "C" int lne_trunc_log_values(lne_ctx* ctx, const double* x, int64_t n, double* out) {
  LNE_CHECK_ARG(ctx && x && out && n >= 0, "lne_trunc_log_values: bad argument");
  if (n == 0) return LNE_OK;
  LNE_CUDA_TRY(cudaSetDevice(ctx->device));
  double* d = nullptr;
  int rc = dalloc(ctx, (void**)&d, sizeof(double) * 2 * n, "trunc-log values");
  if (rc) return rc;
  LNE_CUDA_TRY(cudaMemcpyAsync(d, x, sizeof(double) * n, cudaMemcpyHostToDevice, ctx->stream));
  k_trunc_log_values<<<(unsigned)((n + 255) / 256), 256, 0, ctx->stream>>>(d, n, d + n);
  LNE_CUDA_TRY(cudaMemcpyAsync(out, d + n, sizeof(double) * n, cudaMemcpyDeviceToHost, ctx->stream));
  dfree(ctx, d);
  LNE_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  LNE_CUDA_TRY(cudaGetLastError());
  return LNE_OK;
}
