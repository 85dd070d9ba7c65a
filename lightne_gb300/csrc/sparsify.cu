// NetSMF sparsifier on the device: path sampler, pair-count table,
// trunc-log map and canonical CSR build.
//
// Reference: path_embed::generate_trunc_log_matrix_v2 (LightNE/PathEmbed.h:81-369)
// with par_table (LightNE/par_table.h).
//
// Layout in HBM during one call:
//   keys    u64[samples] x 2     the walk's samples (hashed keys on the sliced
//                                path) and their radix-partitioned copy
//   uniq    Slot[distinct]       sliced path: the distinct pairs with counts
//   table   Slot[capacity]       pair table (weights, several batches, or the
//                                sliced path's fallback): 16 B per slot,
//                                u64 key, u64 count (or f64 weight)
//   rowcnt  i64[n]               kept entries per row
//   row_ptr i64[n+1]             exclusive scan of rowcnt (the output row_ptr)
//   items   u64[nnz] + u32[nnz]  (row << cbits | col, float bits) per CSR entry,
//                                twice (ping-pong buffers of the radix sort)
//   col/val i32[nnz], f32[nnz]   output CSR (every row sorted by column)
#include <cuda_runtime.h>
#include <math.h>
#include <stdio.h>

#include <algorithm>
#include <string>

#include "lne_internal.h"
#include "lne_math.cuh"
#include "radix.h"

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
  // hash-range rounds (the counts path above one batch): keep only the
  // samples whose hashed key has these top qbits (0: keep every sample),
  // and store the key rotated left by qbits
  int qbits;
  uint32_t qsel;
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
// so the lanes of a warp draw in step whatever phase each lane is in.
// Emitted pair keys (and weights with -sample 1) are staged per warp in
// shared memory and written to the sample buffer 32 at a time, so the walk
// never waits on the aggregation.  k_walk (below) is the -sample 1 form, with
// one branch per phase; k_walk_counts is the -sample 0 form with selects.
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

// The sampler for counts (-sample 0), the same draws and walks as k_walk
// with the per-draw state update written as selects rather than branches:
// the lanes of a warp sit in different phases (r, k, walk on u's side, walk
// on v's side), and branches per phase ran each phase's code in turn at
// about half the lanes.  Here every lane runs the same instructions; only
// the neighbour load (walk phases) and the vertex-record load (a walk that
// goes on) are predicated.  HASHED writes hash64_2(key) instead of the key.
// The grid is persistent: a lane whose edge has drawn all its samples takes
// the next unstarted edge of [e0, e1) from edge_ctr (one atomic per warp
// and refill), so the lanes of a warp stay busy until the range runs out
// instead of waiting for the warp's longest edge.  Which lane samples which
// edge does not change any sample: every edge's draws come from its own
// generator, fork((u << 32) | v).
template <bool HASHED>
__global__ void __launch_bounds__(kWalkThreads, 6) k_walk_counts(
    const Vertex* __restrict__ vd, const uint32_t* __restrict__ nbrs, const uint32_t* __restrict__ src, int64_t e0,
    int64_t e1, SampleArgs a, unsigned long long* __restrict__ out_keys, unsigned long long* __restrict__ out_count,
    uint64_t out_cap, int* flags, unsigned long long* __restrict__ edge_ctr) {
  __shared__ unsigned long long qk[kWalkThreads / 32][kQueue];
  __shared__ unsigned long long rmag[kMaxRMagic + 1];
  for (int i = threadIdx.x; i <= kMaxRMagic; i += blockDim.x) rmag[i] = gm_magic(i > 0 ? (uint32_t)i : 1u);
  __syncthreads();
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  bool active = false, exhausted = false;
  uint32_t u = 0, v = 0, x = 0, left1 = 0, left2 = 0, r = 1;
  uint32_t cur_off = 0, div = 1;
  uint64_t mag = 1;
  uint4 vu = make_uint4(0, 1, 1, 0), vv = make_uint4(0, 1, 1, 0);
  uint64_t s = 0, todo = 0;
  int phase = kPhR;
  const uint32_t T = (uint32_t)a.walk_len;
  int qlen = 0;  // warp-uniform
  for (;;) {
    // refill: the lanes without an edge take the next ones
    const unsigned need = __ballot_sync(kFullMask, !active && !exhausted);
    if (need) {
      const int leader = __ffs(need) - 1;
      unsigned long long base = 0;
      if (lane == leader) base = atomicAdd(edge_ctr, (unsigned long long)__popc(need));
      base = __shfl_sync(kFullMask, base, leader);
      if (!active && !exhausted) {
        const int64_t e = e0 + (int64_t)base + __popc(need & ((1u << lane) - 1));
        if (e >= e1) {
          exhausted = true;
        } else {
          u = __ldg(src + e);
          v = __ldg(nbrs + e);
          vu = __ldg(reinterpret_cast<const uint4*>(vd + u));
          vv = __ldg(reinterpret_cast<const uint4*>(vd + v));
          s = rng_fork(a.seed, ((uint64_t)u << 32) | (uint64_t)v);
          todo = a.exp_rv;
          if (a.use_frac) todo += (map_uint64(rng_draw(s)) < a.frac) ? 1u : 0u;
          active = todo > 0;
          phase = kPhR;
          div = T;
          mag = a.walk_magic;
        }
      }
    }
    if (!__any_sync(kFullMask, active)) {
      if (__all_sync(kFullMask, exhausted)) break;
      continue;  // lanes whose new edge has no samples take another
    }
    const uint64_t rnd = rng_draw(s);
    const uint32_t m = gm_mod(rnd, div, mag);
    const bool isR = phase == kPhR, isK = phase == kPhK, isW1 = phase == kPhW1;
    const bool isW = phase >= kPhW1;
    uint32_t nxt = 0;
    if (active && isW) nxt = __ldg(nbrs + cur_off + m);
    // position reached by this draw (k: the walk on u's side starts at u)
    // and the steps left on each side
    const uint32_t pos = isW ? nxt : u;
    const uint32_t l1 = isK ? m : (isW1 ? left1 - 1u : left1);
    const uint32_t l2 = isK ? r - m - 1u : (isW1 || isR ? left2 : left2 - 1u);
    const bool side_u = isK || isW1;
    const bool go_u = side_u && l1 > 0;             // walk on from pos, u's side
    const bool to_v = side_u && l1 == 0 && l2 > 0;  // u's side done: walk from v
    const bool go_v = !side_u && !isR && l2 > 0;    // walk on from pos, v's side
    const bool end = !isR && !go_u && !to_v && !go_v;
    const uint32_t xn = (side_u && l1 == 0) ? pos : x;
    const uint32_t eb = side_u ? v : pos;
    uint4 rec = to_v ? vv : vu;
    if (active && isW && (go_u || go_v)) rec = __ldg(reinterpret_cast<const uint4*>(vd + pos));
    const uint32_t rn = m + 1u;  // r from the first draw of a sample
    const bool fin = active && end;  // a sample completes
    bool emit = fin;
    unsigned long long key = 0;
    if (fin) {
      const uint32_t lo = xn < eb ? xn : eb, hi = xn < eb ? eb : xn;
      key = ((uint64_t)lo << 32) + (uint64_t)hi;
      if (HASHED) {
        key = hash64_2(key);
        if (a.qbits) {
          emit = (uint32_t)(key >> (64 - a.qbits)) == a.qsel;
          key = (key << a.qbits) | (key >> (64 - a.qbits));
        }
      }
    }
    // next state
    const uint64_t rmg = rmag[rn <= (uint32_t)kMaxRMagic ? rn : 0u];
    x = xn;
    left1 = l1;
    left2 = l2;
    r = isR ? rn : r;
    if (isR) {
      phase = kPhK;
      div = rn;
      mag = rn <= (uint32_t)kMaxRMagic ? rmg : gm_magic(rn);
    } else if (end) {
      phase = kPhR;
      div = T;
      mag = a.walk_magic;
    } else {
      phase = go_u ? kPhW1 : kPhW2;
      cur_off = rec.x;
      div = rec.y;
      mag = ((uint64_t)rec.w << 32) | rec.z;
      if (div == 0) active = false;  // unreachable for a validated (symmetric) graph
    }
    if (fin && --todo == 0) active = false;
    // stage this iteration's keys in the warp queue
    const unsigned em = __ballot_sync(kFullMask, emit);
    if (emit) qk[wid][qlen + __popc(em & ((1u << lane) - 1))] = key;
    qlen += __popc(em);
    __syncwarp();
    if (qlen >= 32) {
      unsigned long long base = 0;
      if (lane == 0) base = atomicAdd(out_count, 32ULL);
      base = __shfl_sync(kFullMask, base, 0);
      if (base + 32 <= out_cap)
        out_keys[base + lane] = qk[wid][lane];
      else if (lane == 0)
        atomicExch(flags + kFlagSortOverflow, 1);
      __syncwarp();
      if (lane < qlen - 32) qk[wid][lane] = qk[wid][32 + lane];
      qlen -= 32;
      __syncwarp();
    }
  }
  if (qlen > 0) {
    unsigned long long base = 0;
    if (lane == 0) base = atomicAdd(out_count, (unsigned long long)qlen);
    base = __shfl_sync(kFullMask, base, 0);
    if (lane < qlen) {
      if (base + lane < out_cap)
        out_keys[base + lane] = qk[wid][lane];
      else
        atomicExch(flags + kFlagSortOverflow, 1);
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

// ---------------------------------------------------------------------------
// Sliced aggregation (counts, one batch of samples).  The insert-add of
// par_table only has to produce the multiset of (pair, count); where the
// slot of a pair lies does not show in the output, which is sorted.  So the
// sampler writes every key as h = hash64_2(key) (a bijection), the batch is
// sorted by the top `sbits` bits of h (a few radix passes), and each slice
// of 2^-sbits of the hash space -- a few thousand samples -- is counted by
// one CTA in a shared-memory open-addressing table (linear probing on the
// low bits of h, the same insert-or-add as par_table).  The occupied slots
// are appended, with the key recovered by hash64_2_inv, as a dense
// Slot[distinct] array that the trunc-log reads in place of the table.
// No pair table is written or read in HBM.  If a slice has more distinct
// pairs than its shared table holds, the slice kernel raises
// kFlagSliceOverflow and the host reruns the batch through the pair table.
// The all-ones word marks an empty shared slot: its hash preimage is a pair
// with a vertex id above 2^31, which int32 vertex ids rule out.
// ---------------------------------------------------------------------------
static constexpr int kSliceThreads = 512;
static constexpr int kSliceSlotsMax = 8192;  // 96 KB of shared memory: two CTAs per SM
static constexpr int kSliceBitsMax = 16;        // one batch: two radix passes
static constexpr int kRoundSliceBitsMax = 24;   // a hash-range round: up to three

__device__ __forceinline__ int64_t slice_of(unsigned long long h, int sbits) {
  return sbits == 0 ? 0 : (int64_t)(h >> (64 - sbits));
}

// start[s] = first index of slice s in the sorted hashed keys, s = 0..nslices
// (start[nslices] = count).
__global__ void k_slice_bounds(const unsigned long long* __restrict__ hk, int64_t count, int sbits, int64_t nslices,
                               int64_t* __restrict__ start) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i <= count;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t s_cur = i < count ? slice_of(hk[i], sbits) : nslices;
    const int64_t s_prev = i > 0 ? slice_of(hk[i - 1], sbits) : -1;
    for (int64_t s = s_prev + 1; s <= s_cur; ++s) start[s] = i;
  }
}

// One CTA per slice at a time (slices round-robin over the grid, two CTAs
// per SM so that one counts while the other waits); adds the slices'
// distinct pairs to *n_distinct and the samples counted to *n_samples.  A
// slice's keys are loaded into registers (kSliceRegs per thread, in chunks
// for larger slices) before the table is cleared, so the global loads
// overlap the clearing; every lane inserts its own key (equal keys meet in
// the table: the CAS admits one, the others add).  The occupied slots are
// found in 32-slot chunks (one per warp in turn, conflict-free) whose
// occupancy masks stay in registers between the count and the write.
static constexpr int kSliceRegs = 12;
static constexpr int kSliceMaskRegs = kSliceSlotsMax / 32 / (kSliceThreads / 32);  // 16

__global__ void __launch_bounds__(kSliceThreads, 2) k_slice_count(const unsigned long long* __restrict__ hk,
                                                                  const int64_t* __restrict__ start, int64_t nslices,
                                                                  int slots_max, Slot* __restrict__ uniq,
                                                                  unsigned long long* __restrict__ n_distinct,
                                                                  unsigned long long* __restrict__ n_samples,
                                                                  int* __restrict__ flags, int qbits) {
  extern __shared__ __align__(16) unsigned char slice_smem[];
  unsigned long long* sk = reinterpret_cast<unsigned long long*>(slice_smem);
  unsigned* sc = reinterpret_cast<unsigned*>(slice_smem + sizeof(unsigned long long) * slots_max);
  __shared__ unsigned warp_tot[kSliceThreads / 32];
  __shared__ unsigned long long blk_base;
  __shared__ int blk_ovf;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int nthr = blockDim.x, nwarps = nthr >> 5;
  const unsigned lt = (1u << lane) - 1u;
  unsigned long long my_samples = 0;
  int64_t s = blockIdx.x;
  int64_t b = s < nslices ? start[s] : 0, e = s < nslices ? start[s + 1] : 0;
  for (; s < nslices; s += gridDim.x) {
    // bounds of this CTA's next slice, loaded while this one is counted
    const int64_t sn = s + gridDim.x;
    const int64_t bn = sn < nslices ? start[sn] : 0, en = sn < nslices ? start[sn + 1] : 0;
    if (e > b) {  // the same for every thread of the CTA
      int slots = 64;
      while (slots < slots_max && (int64_t)slots < (e - b) + (e - b) / 2) slots <<= 1;
      const unsigned smask = (unsigned)slots - 1u;
      unsigned long long reg[kSliceRegs];
      int64_t c0 = b;
      {
        const int64_t i0 = c0 + (threadIdx.x & ~31) + lane;
#pragma unroll
        for (int k = 0; k < kSliceRegs; ++k) {
          const int64_t i = i0 + (int64_t)k * nthr;
          reg[k] = i < e ? hk[i] : kEmptyKey;
        }
      }
      for (int i = threadIdx.x; i < slots; i += nthr) {
        sk[i] = kEmptyKey;
        sc[i] = 0u;
      }
      if (threadIdx.x == 0) blk_ovf = 0;
      __syncthreads();
      // insert-or-add; lanes holding the same pair are merged first
      for (;;) {
#pragma unroll
        for (int k = 0; k < kSliceRegs; ++k) {
          const unsigned long long h = reg[k];
          if (h != kEmptyKey) {
            const unsigned add = 1u;
            unsigned pos = (unsigned)h & smask;
            bool placed = false;
            for (int p = 0; p < slots; ++p) {
              unsigned long long kk = *reinterpret_cast<volatile unsigned long long*>(&sk[pos]);
              if (kk == kEmptyKey) kk = atomicCAS(&sk[pos], kEmptyKey, h);
              if (kk == kEmptyKey || kk == h) {
                atomicAdd(&sc[pos], add);
                placed = true;
                break;
              }
              pos = (pos + 1u) & smask;
            }
            if (placed)
              my_samples += add;
            else
              blk_ovf = 1;
          }
        }
        c0 += (int64_t)kSliceRegs * nthr;
        if (c0 >= e) break;  // the same for every thread
        const int64_t i0 = c0 + (threadIdx.x & ~31) + lane;
#pragma unroll
        for (int k = 0; k < kSliceRegs; ++k) {
          const int64_t i = i0 + (int64_t)k * nthr;
          reg[k] = i < e ? hk[i] : kEmptyKey;
        }
      }
      __syncthreads();
      // occupied slots: 32-slot chunks, chunk c by warp c % nwarps
      const int nchunk = slots >> 5;
      unsigned mask[kSliceMaskRegs];
      unsigned occ = 0;
#pragma unroll
      for (int q = 0; q < kSliceMaskRegs; ++q) {
        const int c = wid + q * nwarps;
        const bool in = c < nchunk;
        mask[q] = __ballot_sync(kFullMask, in && sk[(in ? c : 0) * 32 + lane] != kEmptyKey);
        occ += __popc(mask[q]);
      }
      if (lane == 0) warp_tot[wid] = occ;
      __syncthreads();
      unsigned before = 0, total = 0;
      for (int w = 0; w < nwarps; ++w) {
        const unsigned t = warp_tot[w];
        if (w < wid) before += t;
        total += t;
      }
      if (threadIdx.x == 0) {
        blk_base = atomicAdd(n_distinct, (unsigned long long)total);
        if (blk_ovf) atomicExch(flags + kFlagSliceOverflow, 1);
      }
      __syncthreads();
      uint64_t pos = blk_base + before;
#pragma unroll
      for (int q = 0; q < kSliceMaskRegs; ++q) {
        const int j = (wid + q * nwarps) * 32 + lane;
        if ((mask[q] >> lane) & 1u) {
          const unsigned long long h = qbits ? (sk[j] >> qbits) | (sk[j] << (64 - qbits)) : sk[j];
          uniq[pos + __popc(mask[q] & lt)] = Slot{hash64_2_inv(h), (unsigned long long)sc[j]};
        }
        pos += __popc(mask[q]);
      }
      __syncthreads();  // the table is cleared for the next slice
    }
    b = bn;
    e = en;
  }
  for (int o = 16; o > 0; o >>= 1) my_samples += __shfl_down_sync(kFullMask, my_samples, o);
  if (lane == 0 && my_samples) atomicAdd(n_samples, my_samples);
}

// Hashed keys back to pair keys, in place (the pair-table fallback).
__global__ void k_unhash(unsigned long long* __restrict__ k, int64_t count) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += (int64_t)gridDim.x * blockDim.x)
    k[i] = hash64_2_inv(k[i]);
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
// CSR build (PathEmbed.h:226-288).  Every kept pair (u, v), u <= v, is
// appended to the item list once, as key u << cbits | v with the float bits
// of its log value; its entry (v, u) of the lower triangle (PathEmbed.h:
// 300-311, unless -upper or u == v) is not written but counted: rowcnt[u]
// counts row u's upper entries (diagonal included), lowcnt[v] row v's lower
// ones, diag[u] marks a kept diagonal entry.  The append order depends on
// scheduling; the keys are distinct, so the radix sort by key that follows
// (and, for the lower triangle, the sort of its transpose) makes the CSR
// independent of it.
//
// Counts (-sample 0): adj = ((w * factor) / d_u) / d_v is reproduced
// exactly by integer arithmetic (the reference's three double roundings),
// adj > 1 decides the keep test exactly, and log(adj) is evaluated in
// double-float; only values whose narrowing to float the double-float
// result cannot decide go through FP64 (trunc_log_value).  Weights
// (-sample 1) take the FP64 path throughout.
//
// The slots of a warp's stretch of the table are compacted into a per-warp
// queue first (about a third of the slots are occupied), so that the
// log evaluation runs with all 32 lanes busy.  On the dense distinct pairs
// each thread evaluates kTruncLogPer pairs per round.
static constexpr int kTruncLogPer = 4;

template <bool WEIGHTED>
struct TruncLogOut {
  unsigned nitem;  // 0, 1 or 2 CSR entries
  uint32_t u, v;
  float f;
};

template <bool WEIGHTED>
__device__ __forceinline__ TruncLogOut<WEIGHTED> trunclog_entry(unsigned long long key, unsigned long long raw,
                                                                const Vertex* __restrict__ vd, double factor,
                                                                const XDouble& xf, int upper, const LogTable& tab) {
  TruncLogOut<WEIGHTED> o;
  o.nitem = 0;
  o.f = 0.0f;
  o.u = (uint32_t)(key >> 32);
  o.v = (uint32_t)key;
  const uint4 ru = __ldg(reinterpret_cast<const uint4*>(vd + o.u));
  const uint4 rv = __ldg(reinterpret_cast<const uint4*>(vd + o.v));
  bool keep;
  if (WEIGHTED) {
    double w = __longlong_as_double((long long)raw);
    if (o.u == o.v) w = __dmul_rn(w, 2.0);
    const double adj = __ddiv_rn(__ddiv_rn(__dmul_rn(w, factor), (double)ru.y), (double)rv.y);
    const double L = trunc_log_value(adj);
    keep = L > 0.0;
    if (keep) o.f = __double2float_rn(L);
  } else {
    const XDouble adj = trunc_log_adj(raw, o.u == o.v, xf, ru.y, ((uint64_t)ru.w << 32) | ru.z, rv.y,
                                      ((uint64_t)rv.w << 32) | rv.z);
    keep = adj.e > -52 || (adj.e == -52 && adj.m > (1ull << 52));  // adj > 1  <=>  log(adj) > 0
    if (keep && !float_of_log_fast(log_df(adj, tab), &o.f))
      o.f = __double2float_rn(trunc_log_value(xd_to_double(adj)));
  }
  if (keep) o.nitem = (upper || o.u == o.v) ? 1u : 2u;
  return o;
}

template <bool WEIGHTED, bool DENSE>
__global__ void __launch_bounds__(256) k_trunclog(const Slot* __restrict__ T, uint64_t cap,
                                                  const Vertex* __restrict__ vd, double factor, int upper,
                                                  const LogTable* __restrict__ ltab,
                                                  unsigned long long* __restrict__ rowcnt,
                                                  unsigned long long* __restrict__ lowcnt,
                                                  uint8_t* __restrict__ diag,
                                                  unsigned long long* __restrict__ kept_total,
                                                  unsigned long long* __restrict__ n_items, int cbits,
                                                  uint64_t max_items, unsigned long long* __restrict__ okeys,
                                                  uint32_t* __restrict__ ovals, int* __restrict__ flags) {
  __shared__ LogTable tab;
  __shared__ unsigned long long qkey[8][64], qraw[8][64];  // per-warp queue of occupied slots
  for (int i = threadIdx.x; i < 128; i += blockDim.x) {
    tab.log_hi[i] = ltab->log_hi[i];
    tab.log_lo[i] = ltab->log_lo[i];
    tab.inv_hi[i] = ltab->inv_hi[i];
    tab.inv_lo[i] = ltab->inv_lo[i];
  }
  __syncthreads();
  const XDouble xf = xd_from_double(factor);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const unsigned lt = (1u << lane) - 1u;
  unsigned long long* qk = qkey[wid];
  unsigned long long* qr = qraw[wid];
  unsigned long long kept = 0;
  int qn = 0;  // queued entries (warp-uniform), < 32 between flushes

  // Evaluates one entry per lane (lanes with have set) and appends their
  // CSR entries.
  auto emit = [&](bool have, unsigned long long key, unsigned long long raw) {
    TruncLogOut<WEIGHTED> o;
    o.nitem = 0;
    if (have) o = trunclog_entry<WEIGHTED>(key, raw, vd, factor, xf, upper, tab);
    if (o.nitem) {
      atomicAdd(&rowcnt[o.u], 1ULL);
      if (o.nitem == 2) atomicAdd(&lowcnt[o.v], 1ULL);
      if (o.u == o.v) diag[o.u] = 1;
      ++kept;
    }
    const unsigned one = o.nitem ? 1u : 0u;
    unsigned incl = one;
#pragma unroll
    for (int s = 1; s < 32; s <<= 1) {
      const unsigned t = __shfl_up_sync(kFullMask, incl, s);
      if (lane >= s) incl += t;
    }
    const unsigned wtot = __shfl_sync(kFullMask, incl, 31);
    unsigned long long base = 0;
    if (lane == 31 && wtot) base = atomicAdd(n_items, (unsigned long long)wtot);
    base = __shfl_sync(kFullMask, base, 31);
    if (one) {
      const uint64_t pos = base + incl - 1;
      if (pos < max_items) {
        okeys[pos] = ((unsigned long long)o.u << cbits) | o.v;
        ovals[pos] = __float_as_uint(o.f);
      } else {
        atomicOr(&flags[kFlagSortOverflow], 1);
      }
    }
  };

  // Evaluates the first min(qn, 32) queued entries (one per lane).
  auto flush = [&](int take) {
    const bool have = lane < take;
    const unsigned long long key = have ? qk[lane] : 0ULL, raw = have ? qr[lane] : 0ULL;
    __syncwarp();
    emit(have, key, raw);
  };

  // warp-uniform loop: the lanes of a warp read 32 consecutive slots
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  if (DENSE) {
    // every slot occupied (the distinct pairs of the sliced aggregation):
    // block-uniform rounds of kTruncLogPer x 256 consecutive pairs, each
    // thread evaluating kTruncLogPer of them (their vertex-record gathers in
    // flight together), whose items are placed with one atomic on the item
    // count per round (per warp, the atomics on that one counter serialise
    // in L2)
    __shared__ unsigned wsum[8];
    __shared__ unsigned long long bbase;
    constexpr int kPer = kTruncLogPer;
    const uint64_t span = (uint64_t)blockDim.x * kPer;
    for (uint64_t b0 = (uint64_t)blockIdx.x * span; b0 < cap; b0 += (uint64_t)gridDim.x * span) {
      TruncLogOut<WEIGHTED> o[kPer];
      unsigned mine = 0;
#pragma unroll
      for (int q = 0; q < kPer; ++q) {
        const uint64_t i = b0 + (uint64_t)q * blockDim.x + threadIdx.x;
        o[q].nitem = 0;
        if (i < cap) {
          const Slot sl = T[i];
          o[q] = trunclog_entry<WEIGHTED>(sl.key, sl.val, vd, factor, xf, upper, tab);
        }
      }
#pragma unroll
      for (int q = 0; q < kPer; ++q) {
        if (o[q].nitem) {
          atomicAdd(&rowcnt[o[q].u], 1ULL);
          if (o[q].nitem == 2) atomicAdd(&lowcnt[o[q].v], 1ULL);
          if (o[q].u == o[q].v) diag[o[q].u] = 1;
          ++kept;
          ++mine;
        }
      }
      unsigned incl = mine;
#pragma unroll
      for (int sh = 1; sh < 32; sh <<= 1) {
        const unsigned t = __shfl_up_sync(kFullMask, incl, sh);
        if (lane >= sh) incl += t;
      }
      if (lane == 31) wsum[wid] = incl;
      __syncthreads();
      if (threadIdx.x == 0) {
        unsigned tot = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) tot += wsum[w];
        bbase = tot ? atomicAdd(n_items, (unsigned long long)tot) : 0ULL;
      }
      __syncthreads();
      unsigned before = 0;
      for (int w = 0; w < wid; ++w) before += wsum[w];
      uint64_t pos = bbase + before + incl - mine;
#pragma unroll
      for (int q = 0; q < kPer; ++q) {
        if (o[q].nitem) {
          if (pos < max_items) {
            okeys[pos] = ((unsigned long long)o[q].u << cbits) | o[q].v;
            ovals[pos] = __float_as_uint(o[q].f);
          } else {
            atomicOr(&flags[kFlagSortOverflow], 1);
          }
          ++pos;
        }
      }
      __syncthreads();  // wsum and bbase are rewritten in the next round
    }
  }
  for (uint64_t b = (uint64_t)blockIdx.x * blockDim.x + (threadIdx.x & ~31u); !DENSE && b < cap; b += stride) {
    const uint64_t i = b + lane;
    const unsigned long long key = i < cap ? T[i].key : kEmptyKey;
    const bool occ = key != kEmptyKey;
    const unsigned occm = __ballot_sync(kFullMask, occ);
    if (occ) {
      const int at = qn + __popc(occm & lt);
      qk[at] = key;
      qr[at] = T[i].val;
    }
    qn += __popc(occm);
    __syncwarp();
    if (qn >= 32) {
      flush(32);
      // move the entries past the first 32 to the front of the queue
      const unsigned long long k2 = lane < qn - 32 ? qk[32 + lane] : 0ULL;
      const unsigned long long r2 = lane < qn - 32 ? qr[32 + lane] : 0ULL;
      __syncwarp();
      if (lane < qn - 32) {
        qk[lane] = k2;
        qr[lane] = r2;
      }
      qn -= 32;
      __syncwarp();
    }
  }
  if (qn > 0) flush(qn);
  for (int o = 16; o > 0; o >>= 1) kept += __shfl_down_sync(kFullMask, kept, o);
  if (lane == 0 && kept) atomicAdd(kept_total, kept);
}

// Counts of the symmetric CSR from the trunc-log's counts: full[r] = row r's
// entries (upper, diagonal included, plus lower); tcnt[r] = entries of row r
// in the transposed upper triangle (the lower ones plus the diagonal).
__global__ void k_sym_counts(const unsigned long long* __restrict__ up, const unsigned long long* __restrict__ lo,
                             const uint8_t* __restrict__ diag, int64_t n, int64_t* __restrict__ full,
                             int64_t* __restrict__ tcnt) {
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
    full[r] = (int64_t)(up[r] + lo[r]);
    tcnt[r] = (int64_t)lo[r] + diag[r];
  }
}

// Final CSR position of an entry = offset of its row + its position in the
// sorted (upper or transposed) item array: row r's lower entries come first
// (columns < r), then its diagonal and upper entries.
__global__ void k_sym_offsets(const int64_t* __restrict__ row_ptr, const unsigned long long* __restrict__ lo,
                              const int64_t* __restrict__ upstart, const int64_t* __restrict__ tstart, int64_t n,
                              int64_t* __restrict__ upoff, int64_t* __restrict__ looff) {
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
    upoff[r] = row_ptr[r] + (int64_t)lo[r] - upstart[r];
    looff[r] = row_ptr[r] - tstart[r];
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
  void* p[16] = {};
  int k = 0;
  explicit Scratch(lne_ctx* c) : ctx(c) {}
  int get(void** out, size_t bytes, const char* what) {
    if (k == 16) {
      set_error("lne_sparsify: scratch list full (internal)");
      return LNE_ERR_UNSUPPORTED;
    }
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

// ---------------------------------------------------------------------------
// Hash-range rounds: the counts path (-sample 0) above one batch of samples
// when the reference's pair table does not fit in device memory (or when
// lne_ctx_set_sparsify_rounds forces it).  The sampler is a function of
// the seed and the edge alone, so it can be replayed: round q replays all
// edges and keeps the samples whose hash64_2(key) has top bits q, which
// then fit one batch of the sliced aggregation; the rounds' distinct pairs
// are disjoint (a pair's samples all fall in one round), so every pair is
// counted whole in one round.  A first sweep over the rounds applies the
// trunc-log and counts each row's kept entries (row_ptr); a second sweep
// replays the rounds and writes each kept entry into its row at an atomic
// cursor; a last pass sorts every row by column.  Peak memory is the CSR
// plus one round's buffers, where the pair table path needs the table and
// twice the CSR's items.
// ---------------------------------------------------------------------------
// Total samples (M_exact for counts): per directed entry exp_rv, plus one
// when the entry's first draw falls below frac (as the sampler starts).
__global__ void k_count_samples(const uint32_t* __restrict__ nbrs, const uint32_t* __restrict__ src, int64_t m_dir,
                                SampleArgs a, unsigned long long* __restrict__ total) {
  unsigned long long c = 0;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < m_dir; e += (int64_t)gridDim.x * blockDim.x) {
    const uint32_t u = __ldg(src + e), v = __ldg(nbrs + e);
    uint64_t s = rng_fork(a.seed, ((uint64_t)u << 32) | (uint64_t)v);
    uint64_t todo = a.exp_rv;
    if (a.use_frac) todo += (map_uint64(rng_draw(s)) < a.frac) ? 1u : 0u;
    c += todo;
  }
  for (int o = 16; o > 0; o >>= 1) c += __shfl_down_sync(kFullMask, c, o);
  if ((threadIdx.x & 31) == 0 && c) atomicAdd(total, c);
}

// Trunc-log of a round's distinct pairs: SCATTER = false counts the kept
// entries per row (rowcnt) and the kept pairs; SCATTER = true writes each
// kept entry at row_ptr[row] + an atomic cursor (rowcnt, zeroed first).
template <bool SCATTER>
__global__ void __launch_bounds__(256) k_trunclog_rows(const Slot* __restrict__ T, uint64_t count,
                                                       const Vertex* __restrict__ vd, double factor, int upper,
                                                       const LogTable* __restrict__ ltab,
                                                       unsigned long long* __restrict__ rowcnt,
                                                       unsigned long long* __restrict__ kept_total,
                                                       const int64_t* __restrict__ row_ptr, int32_t* __restrict__ col,
                                                       float* __restrict__ val, int* __restrict__ flags) {
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
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count;
       i += (uint64_t)gridDim.x * blockDim.x) {
    const Slot sl = T[i];
    const TruncLogOut<false> o = trunclog_entry<false>(sl.key, sl.val, vd, factor, xf, upper, tab);
    if (!o.nitem) continue;
    ++kept;
    if (!SCATTER) {
      atomicAdd(&rowcnt[o.u], 1ULL);
      if (o.nitem == 2) atomicAdd(&rowcnt[o.v], 1ULL);
    } else {
      // the first sweep counted exactly these entries; a cursor past its
      // row is reported instead of written
      const int64_t cu = (int64_t)atomicAdd(&rowcnt[o.u], 1ULL);
      if (cu < row_ptr[o.u + 1] - row_ptr[o.u]) {
        col[row_ptr[o.u] + cu] = (int32_t)o.v;
        val[row_ptr[o.u] + cu] = o.f;
      } else {
        atomicOr(&flags[kFlagSortOverflow], 1);
      }
      if (o.nitem == 2) {
        const int64_t cv = (int64_t)atomicAdd(&rowcnt[o.v], 1ULL);
        if (cv < row_ptr[o.v + 1] - row_ptr[o.v]) {
          col[row_ptr[o.v] + cv] = (int32_t)o.u;
          val[row_ptr[o.v] + cv] = o.f;
        } else {
          atomicOr(&flags[kFlagSortOverflow], 1);
        }
      }
    }
  }
  for (int o = 16; o > 0; o >>= 1) kept += __shfl_down_sync(kFullMask, kept, o);
  if ((threadIdx.x & 31) == 0 && kept) atomicAdd(kept_total, kept);
}

// The rounds path (see above).  Fills *out and stats like lne_sparsify.
static int sparsify_rounds(lne_ctx* ctx, const lne_graph* g, const lne_sparsify_params* p, SampleArgs a,
                           uint64_t cap, uint64_t buf_keys, double logn, double M, double inv_lambda, double frac,
                           size_t exp_rv, size_t table_size, lne_csr** out, lne_sparsify_stats* stats) {
  cudaStream_t st = ctx->stream;
  const int64_t n = g->n, m_dir = g->m_dir;
  const int slots_max = std::min(ctx->sparsify_slice_slots, kSliceSlotsMax);
  const size_t slice_smem = (size_t)slots_max * (sizeof(unsigned long long) + sizeof(unsigned));
  Scratch S(ctx);
  Events ev;
  int rc, launches = 0;
  unsigned long long* cnt = nullptr;  // [0] samples [1] round emitted [2] round distinct [3] round counted
                                      // [4] kept pairs [5] big rows [6] next edge of the sampler
  if ((rc = S.get((void**)&cnt, 64, "round counters"))) return rc;
  LNE_CUDA_TRY(cudaMemsetAsync(cnt, 0, 64, st));
  LNE_CUDA_TRY(cudaMemsetAsync(ctx->d_flags, 0, sizeof(int) * kFlagWords, st));
  cudaEventRecord(ev.e[0], st);
  k_count_samples<<<grid_for(m_dir, 256, (int64_t)ctx->num_sms * 16), 256, 0, st>>>(g->nbrs, g->src, m_dir, a, cnt);
  ++launches;
  unsigned long long total = 0;
  LNE_CUDA_TRY(cudaMemcpyAsync(&total, cnt, 8, cudaMemcpyDeviceToHost, st));
  LNE_CUDA_TRY(cudaStreamSynchronize(st));
  const double M_exact = (double)total;
  const double factor = (double)(size_t)m_dir * (double)(size_t)m_dir / M_exact / 2 / (double)(size_t)p->negative;
  // rounds of at most ~60% of a batch each, in expectation
  int qbits = 0;
  while (qbits < 16 && (total >> qbits) > buf_keys * 6 / 10) ++qbits;
  const uint32_t Q = 1u << qbits;
  unsigned long long *keys = nullptr, *keys2 = nullptr, *rowcnt = nullptr;
  Slot* uniq = nullptr;
  int64_t* starts = nullptr;
  void* scan_tmp = nullptr;
  if ((rc = S.get((void**)&keys, sizeof(unsigned long long) * buf_keys, "sample buffer")) ||
      (rc = S.get((void**)&keys2, sizeof(unsigned long long) * buf_keys, "partitioned samples")) ||
      (rc = S.get((void**)&uniq, sizeof(Slot) * buf_keys, "distinct pairs")) ||
      (rc = S.get((void**)&starts, sizeof(int64_t) * (((int64_t)1 << kRoundSliceBitsMax) + 1), "slice starts")) ||
      (rc = S.get((void**)&rowcnt, sizeof(unsigned long long) * n, "row counts")) ||
      (rc = S.get(&scan_tmp, scan_tmp_bytes(n), "scan scratch")))
    return rc;
  LNE_CUDA_TRY(cudaMemsetAsync(rowcnt, 0, sizeof(unsigned long long) * n, st));
  LNE_CUDA_TRY(cudaFuncSetAttribute(k_slice_count, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)slice_smem));
  const unsigned wblocks = (unsigned)std::min<int64_t>((m_dir + kWalkThreads - 1) / kWalkThreads,
                                                       (int64_t)ctx->num_sms * 6);
  const unsigned tgrid_cap = (unsigned)ctx->num_sms * 16;
  int64_t* row_ptr = nullptr;
  int32_t* col = nullptr;
  float* val = nullptr;
  auto fail = [&](int code) {
    dfree(ctx, row_ptr);
    dfree(ctx, col);
    dfree(ctx, val);
    return code;
  };
  unsigned long long distinct = 0, counted = 0;
  int64_t nnz = 0;
  for (int sweep = 0; sweep < 2; ++sweep) {
    if (sweep == 1) {
      if (distinct >= cap) {
        char buf[256];
        snprintf(buf, sizeof(buf),
                 "lne_sparsify: %llu distinct pairs do not fit the pair table's %llu slots; raise -tablesz (the "
                 "reference prints \"looping forever\" and exits)",
                 distinct, (unsigned long long)cap);
        set_error(buf);
        return LNE_ERR_TABLE_FULL;
      }
      if (counted != total) {
        set_error("lne_sparsify: the rounds counted a different number of samples (internal error)");
        return LNE_ERR_UNSUPPORTED;
      }
      if ((rc = dalloc(ctx, (void**)&row_ptr, sizeof(int64_t) * (n + 1), "row_ptr"))) return rc;
      scan_exclusive_i64((const int64_t*)rowcnt, row_ptr, n, scan_tmp, st);
      launches += 3;
      LNE_CUDA_TRY(cudaMemcpyAsync(&nnz, row_ptr + n, 8, cudaMemcpyDeviceToHost, st));
      LNE_CUDA_TRY(cudaStreamSynchronize(st));
      if ((rc = dalloc(ctx, (void**)&col, sizeof(int32_t) * (nnz > 0 ? nnz : 1), "csr col")) ||
          (rc = dalloc(ctx, (void**)&val, sizeof(float) * (nnz > 0 ? nnz : 1), "csr val")))
        return fail(rc);
      LNE_CUDA_TRY(cudaMemsetAsync(rowcnt, 0, sizeof(unsigned long long) * n, st));
      cudaEventRecord(ev.e[1], st);
    }
    for (uint32_t q = 0; q < Q; ++q) {
      a.qbits = qbits;
      a.qsel = q;
      LNE_CUDA_TRY(cudaMemsetAsync(cnt + 1, 0, 24, st));
      LNE_CUDA_TRY(cudaMemsetAsync(cnt + 6, 0, 8, st));
      k_walk_counts<true><<<wblocks, kWalkThreads, 0, st>>>(g->vdata, g->nbrs, g->src, 0, m_dir, a, keys, cnt + 1,
                                                            buf_keys, ctx->d_flags, cnt + 6);
      ++launches;
      unsigned long long got = 0;
      int fl[kFlagWords];
      LNE_CUDA_TRY(cudaMemcpyAsync(&got, cnt + 1, 8, cudaMemcpyDeviceToHost, st));
      LNE_CUDA_TRY(cudaMemcpyAsync(fl, ctx->d_flags, sizeof(fl), cudaMemcpyDeviceToHost, st));
      LNE_CUDA_TRY(cudaStreamSynchronize(st));
      if (got > buf_keys || fl[kFlagSortOverflow]) {
        set_error("lne_sparsify: a hash-range round exceeded the sample buffer; raise the batch "
                  "(lne_ctx_set_sparsify_batch)");
        return fail(LNE_ERR_UNSUPPORTED);
      }
      if (got == 0) continue;
      int sbits = 0;
      while (sbits < kRoundSliceBitsMax && (got >> sbits) > (uint64_t)slots_max / 4) ++sbits;
      if ((got >> sbits) > (uint64_t)slots_max * 5 / 8) {
        set_error("lne_sparsify: a hash-range round has more samples than its slices hold; lower the batch");
        return fail(LNE_ERR_UNSUPPORTED);
      }
      unsigned long long* hk = keys;
      if ((rc = partition_by_top_bits(ctx, keys, keys2, (int64_t)got, sbits, &hk, &launches))) return fail(rc);
      const int64_t nslices = (int64_t)1 << sbits;
      k_slice_bounds<<<grid_for((int64_t)got + 1, 256, (int64_t)ctx->num_sms * 16), 256, 0, st>>>(hk, (int64_t)got,
                                                                                                  sbits, nslices,
                                                                                                  starts);
      const unsigned sgrid = (unsigned)std::min<int64_t>(nslices, 2 * (int64_t)ctx->num_sms);
      k_slice_count<<<sgrid, kSliceThreads, slice_smem, st>>>(hk, starts, nslices, slots_max, uniq, cnt + 2, cnt + 3,
                                                              ctx->d_flags, qbits);
      launches += 2;
      unsigned long long sc[2] = {0, 0};  // distinct, counted
      LNE_CUDA_TRY(cudaMemcpyAsync(sc, cnt + 2, sizeof(sc), cudaMemcpyDeviceToHost, st));
      LNE_CUDA_TRY(cudaMemcpyAsync(fl, ctx->d_flags, sizeof(fl), cudaMemcpyDeviceToHost, st));
      LNE_CUDA_TRY(cudaStreamSynchronize(st));
      if (fl[kFlagSliceOverflow]) {
        set_error("lne_sparsify: a slice of a hash-range round overflowed its shared table; lower the batch");
        return fail(LNE_ERR_UNSUPPORTED);
      }
      if (sweep == 0) {
        distinct += sc[0];
        counted += sc[1];
      }
      const unsigned tg = (unsigned)std::min<int64_t>(((int64_t)sc[0] + 255) / 256, (int64_t)tgrid_cap);
      if (sc[0] > 0) {
        if (sweep == 0)
          k_trunclog_rows<false><<<tg, 256, 0, st>>>(uniq, sc[0], g->vdata, factor, p->upper,
                                                     (const LogTable*)ctx->log_table, rowcnt, cnt + 4, nullptr,
                                                     nullptr, nullptr, ctx->d_flags);
        else
          k_trunclog_rows<true><<<tg, 256, 0, st>>>(uniq, sc[0], g->vdata, factor, p->upper,
                                                    (const LogTable*)ctx->log_table, rowcnt, cnt + 5, row_ptr, col,
                                                    val, ctx->d_flags);
        ++launches;
      }
    }
  }
  cudaEventRecord(ev.e[2], st);
  unsigned long long kept = 0;
  LNE_CUDA_TRY(cudaMemcpyAsync(&kept, cnt + 4, 8, cudaMemcpyDeviceToHost, st));
  {
    int fl[kFlagWords];
    LNE_CUDA_TRY(cudaMemcpyAsync(fl, ctx->d_flags, sizeof(fl), cudaMemcpyDeviceToHost, st));
    LNE_CUDA_TRY(cudaStreamSynchronize(st));
    if (fl[kFlagSortOverflow]) {
      set_error("lne_sparsify: the rounds' second sweep kept other entries than the first (internal error)");
      return fail(LNE_ERR_UNSUPPORTED);
    }
  }
  // sort every row by column, in place
  if ((rc = sort_csr_rows(ctx, row_ptr, n, n, col, val, col, val, &launches))) return fail(rc);
  cudaEventRecord(ev.e[3], st);
  LNE_CUDA_TRY(cudaEventSynchronize(ev.e[3]));
  cudaError_t le = cudaGetLastError();
  if (le != cudaSuccess) {
    set_error(std::string("lne_sparsify: kernel launch failed: ") + cudaGetErrorString(le));
    return fail(LNE_ERR_CUDA);
  }
  {
    int fl[kFlagWords];
    LNE_CUDA_TRY(cudaMemcpyAsync(fl, ctx->d_flags, sizeof(fl), cudaMemcpyDeviceToHost, st));
    LNE_CUDA_TRY(cudaStreamSynchronize(st));
    if (fl[kFlagSortOverflow]) {
      set_error("lne_sparsify: CSR entries do not match their rows (internal error)");
      return fail(LNE_ERR_UNSUPPORTED);
    }
  }
  if (stats) {
    stats->logn = logn;
    stats->total_samples = M;
    stats->inv_lambda = inv_lambda;
    stats->frac = frac;
    stats->factor = factor;
    stats->m_exact = M_exact;
    stats->exp_rv_rounded = (int64_t)exp_rv;
    stats->table_size = (int64_t)table_size;
    stats->capacity = (int64_t)cap;
    stats->samples_emitted = (int64_t)total;
    stats->distinct = (int64_t)distinct;
    stats->nnz_upper = (int64_t)kept;
    stats->nnz = nnz;
    cudaEventElapsedTime(&stats->ms_sample, ev.e[0], ev.e[1]);
    cudaEventElapsedTime(&stats->ms_trunclog, ev.e[1], ev.e[2]);
    cudaEventElapsedTime(&stats->ms_csr, ev.e[2], ev.e[3]);
    stats->kernel_launches = launches;
    stats->sliced = 2;
  }
  ctx->launch_count += launches;
  lne_csr* c = new lne_csr();
  c->n = n;
  c->nnz = nnz;
  c->row_ptr = row_ptr;
  c->col = col;
  c->val = val;
  c->stream = st;
  *out = c;
  return LNE_OK;
}

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
  Slot* table = nullptr;  // the pair table in HBM (allocated and cleared on first use)
  Slot* uniq = nullptr;   // sliced aggregation: the distinct pairs with their counts
  unsigned long long* counters = nullptr;  // [0] emitted [1] count sum [2] distinct [3] kept [4] items
                                           // [6] next edge of the sampler's persistent grid
  double* wsum = nullptr;
  int rc;
  const int sum_blocks = 1024;
  if ((rc = S.get((void**)&counters, 64 + sizeof(double) * (sum_blocks + 1), "counters"))) return rc;
  wsum = (double*)((char*)counters + 64);
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
  a.qbits = 0;
  a.qsel = 0;

  cudaEventRecord(ev.e[0], st);
  // Sample buffer: at most exp_rv + 1 samples per directed entry; the edge
  // range is processed in batches that fit the buffer.
  const uint64_t per_edge = (uint64_t)exp_rv + 1;
  const uint64_t want_keys = per_edge * (uint64_t)m_dir;
  const uint64_t max_keys = (uint64_t)ctx->sparsify_batch_keys;  // default 2^30: 8 GiB of keys per batch
  const uint64_t buf_keys = want_keys < max_keys ? want_keys : max_keys;
  const int64_t edges_per_batch = (int64_t)std::max<uint64_t>(1, buf_keys / per_edge);
  // Above one batch, counts take the hash-range rounds when the pair table
  // path does not fit in free device memory (or when forced): its peak is
  // the table plus a batch's buffers while sampling, then the CSR build's
  // items twice (radix ping-pong, 12 bytes each) plus the CSR (8 bytes),
  // two items per distinct pair, at most min(samples, capacity) pairs.
  if (!p->sample && want_keys > max_keys && ctx->sparsify_rounds >= 0 && ctx->sparsify_slice_slots > 0) {
    bool rounds = ctx->sparsify_rounds == 1;
    if (!rounds) {
      size_t fr = 0, tot = 0;
      LNE_CUDA_TRY(cudaMemGetInfo(&fr, &tot));
      const double table_peak = (double)cap * sizeof(Slot) + 2.0 * sizeof(unsigned long long) * (double)buf_keys;
      const double pairs = std::min((double)want_keys, (double)cap);
      const double csr_peak = 2.0 * pairs * (2.0 * 12.0 + 8.0);
      rounds = std::max(table_peak, csr_peak) > (double)fr;
    }
    if (rounds) {
      S.release(counters);
      return sparsify_rounds(ctx, g, p, a, cap, buf_keys, logn, M, inv_lambda, frac, exp_rv, table_size, out,
                             stats);
    }
  }
  unsigned long long* keys = nullptr;
  unsigned long long* keys2 = nullptr;  // counts: the batch reordered by slice
  double* wts = nullptr;
  if ((rc = S.get((void**)&keys, sizeof(unsigned long long) * buf_keys, "sample buffer"))) return rc;
  if (p->sample && (rc = S.get((void**)&wts, sizeof(double) * buf_keys, "sample weights"))) return rc;
  if (!p->sample && (rc = S.get((void**)&keys2, sizeof(unsigned long long) * buf_keys, "partitioned samples")))
    return rc;
  int launches_sample = 0;
  auto ensure_table = [&]() -> int {
    if (table) return LNE_OK;
    const int r = S.get((void**)&table, sizeof(Slot) * cap, "pair table");
    if (r) return r;
    k_table_init<<<grid_for((int64_t)cap, 256, (int64_t)ctx->num_sms * 32), 256, 0, st>>>(table, cap);
    ++launches_sample;
    return LNE_OK;
  };
  // Counts commute, so a batch is first grouped by the top 8 bits of its
  // table slot: the inserts then sweep the table one slice (1/256 of it) at
  // a time, and a slice's slots stay in L2 while its atomics land.  A
  // smaller grid keeps the warps within a slice or two.
  auto insert_counts = [&](const unsigned long long* in, unsigned long long* tmp, unsigned long long got) -> int {
    int r = ensure_table();
    if (r) return r;
    if ((r = partition_by_slot(ctx, in, tmp, (int64_t)got, (int)bits, &launches_sample))) return r;
    const unsigned iblocks = grid_for((int64_t)got, 256, (int64_t)ctx->num_sms * 8);
    k_insert<false><<<iblocks, 256, 0, st>>>(tmp, nullptr, got, table, cap - 1, ctx->d_flags);
    ++launches_sample;
    return LNE_OK;
  };

  // Sliced aggregation (see k_slice_count) for counts when the samples fit
  // one batch and the shared-memory table fits the device.
  const int slots_max = std::min(ctx->sparsify_slice_slots, kSliceSlotsMax);
  const size_t slice_smem = (size_t)slots_max * (sizeof(unsigned long long) + sizeof(unsigned));
  const bool sliced_try = !p->sample && slots_max > 0 && want_keys <= max_keys && slice_smem + 1024 <= ctx->smem_optin;
  bool sliced = false;
  unsigned long long emitted_total = 0;
  if (sliced_try) {
    const unsigned wblocks = (unsigned)std::min<int64_t>((m_dir + kWalkThreads - 1) / kWalkThreads,
                                                         (int64_t)ctx->num_sms * 6);
    LNE_CUDA_TRY(cudaMemsetAsync(counters + 6, 0, 8, st));
    k_walk_counts<true><<<wblocks, kWalkThreads, 0, st>>>(g->vdata, g->nbrs, g->src, 0, m_dir, a, keys, counters,
                                                          buf_keys, ctx->d_flags, counters + 6);
    ++launches_sample;
    unsigned long long got = 0;
    LNE_CUDA_TRY(cudaMemcpyAsync(&got, counters, 8, cudaMemcpyDeviceToHost, st));
    LNE_CUDA_TRY(cudaStreamSynchronize(st));
    if (got > buf_keys) got = buf_keys;  // overflow is flagged and reported below
    emitted_total = got;
    // slices of at most a quarter (5/8, with 2^16 slices) of the shared table
    int sbits = ctx->sparsify_slice_bits;
    if (sbits < 0) {
      sbits = 0;
      while (sbits < kSliceBitsMax && (got >> sbits) > (uint64_t)slots_max / 4) ++sbits;
    }
    const bool fits = ctx->sparsify_slice_bits >= 0 || (got >> sbits) <= (uint64_t)slots_max * 5 / 8;
    unsigned long long* hk = keys;
    if (fits) {
      if ((rc = partition_by_top_bits(ctx, keys, keys2, (int64_t)got, sbits, &hk, &launches_sample))) return rc;
      const int64_t nslices = (int64_t)1 << sbits;
      int64_t* starts = nullptr;
      if ((rc = S.get((void**)&starts, sizeof(int64_t) * (nslices + 1), "slice starts"))) return rc;
      if ((rc = S.get((void**)&uniq, sizeof(Slot) * std::max<unsigned long long>(got, 1), "distinct pairs")))
        return rc;
      k_slice_bounds<<<grid_for((int64_t)got + 1, 256, (int64_t)ctx->num_sms * 16), 256, 0, st>>>(hk, (int64_t)got,
                                                                                                  sbits, nslices,
                                                                                                  starts);
      LNE_CUDA_TRY(cudaFuncSetAttribute(k_slice_count, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)slice_smem));
      const unsigned sgrid = (unsigned)std::min<int64_t>(nslices, 2 * (int64_t)ctx->num_sms);
      k_slice_count<<<sgrid, kSliceThreads, slice_smem, st>>>(hk, starts, nslices, slots_max, uniq, counters + 2,
                                                              counters + 1, ctx->d_flags, 0);
      launches_sample += 2;
      unsigned long long sc[2] = {0, 0};  // samples counted, distinct pairs
      int fl[kFlagWords];
      LNE_CUDA_TRY(cudaMemcpyAsync(sc, counters + 1, sizeof(sc), cudaMemcpyDeviceToHost, st));
      LNE_CUDA_TRY(cudaMemcpyAsync(fl, ctx->d_flags, sizeof(fl), cudaMemcpyDeviceToHost, st));
      LNE_CUDA_TRY(cudaStreamSynchronize(st));
      LNE_CUDA_TRY(cudaGetLastError());
      S.release(starts);
      if (!fl[kFlagSliceOverflow] && sc[0] != got) {
        set_error("lne_sparsify: sliced aggregation lost samples (internal error)");
        return LNE_ERR_UNSUPPORTED;
      }
      // Above 90% of the pair table's capacity the table decides whether
      // the reference's table would fill: rerun through it.
      sliced = !fl[kFlagSliceOverflow] && sc[1] * 10 <= (unsigned long long)cap * 9;
      if (!sliced) {
        S.release(uniq);
        uniq = nullptr;
        LNE_CUDA_TRY(cudaMemsetAsync(counters + 1, 0, 16, st));
        LNE_CUDA_TRY(cudaMemsetAsync(ctx->d_flags + kFlagSliceOverflow, 0, sizeof(int), st));
      }
    }
    if (!sliced) {
      k_unhash<<<grid_for((int64_t)got, 256, (int64_t)ctx->num_sms * 16), 256, 0, st>>>(hk, (int64_t)got);
      ++launches_sample;
      if ((rc = insert_counts(hk, hk == keys ? keys2 : keys, got))) return rc;
    }
  } else {
    if ((rc = ensure_table())) return rc;
    for (int64_t eb = 0; eb < m_dir; eb += edges_per_batch) {
      const int64_t ee = std::min<int64_t>(m_dir, eb + edges_per_batch);
      LNE_CUDA_TRY(cudaMemsetAsync(counters, 0, 8, st));
      LNE_CUDA_TRY(cudaMemsetAsync(counters + 6, 0, 8, st));
      const unsigned wblocks = (unsigned)((ee - eb + kWalkThreads - 1) / kWalkThreads);
      if (p->sample)
        k_walk<true><<<wblocks, kWalkThreads, 0, st>>>(g->vdata, g->nbrs, g->src, eb, ee, a, keys, wts,
                                                              counters, buf_keys, ctx->d_flags);
      else
        k_walk_counts<false><<<(unsigned)std::min<int64_t>(wblocks, (int64_t)ctx->num_sms * 6), kWalkThreads, 0,
                               st>>>(g->vdata, g->nbrs, g->src, eb, ee, a, keys, counters, buf_keys, ctx->d_flags,
                                     counters + 6);
      ++launches_sample;
      unsigned long long got = 0;
      LNE_CUDA_TRY(cudaMemcpyAsync(&got, counters, 8, cudaMemcpyDeviceToHost, st));
      LNE_CUDA_TRY(cudaStreamSynchronize(st));
      if (got > buf_keys) got = buf_keys;  // overflow is flagged and reported below
      if (p->sample) {
        const unsigned iblocks = grid_for((int64_t)got, 256, (int64_t)ctx->num_sms * 32);
        k_insert<true><<<iblocks, 256, 0, st>>>(keys, wts, got, table, cap - 1, ctx->d_flags);
        ++launches_sample;
      } else if ((rc = insert_counts(keys, keys2, got))) {
        return rc;
      }
      emitted_total += got;
    }
  }
  LNE_CUDA_TRY(cudaGetLastError());
  S.release(keys);
  if (keys2) S.release(keys2);
  if (wts) S.release(wts);
  cudaEventRecord(ev.e[1], st);

  const int sgrid = sum_blocks;
  if (!sliced) {
    if (p->sample)
      k_table_sum<true><<<sgrid, 256, 0, st>>>(table, cap, counters + 1, counters + 2, wsum);
    else
      k_table_sum<false><<<sgrid, 256, 0, st>>>(table, cap, counters + 1, counters + 2, wsum);
    k_sum_blocks<<<1, 32, 0, st>>>(wsum, sgrid, wsum + sum_blocks);
  }
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

  // Item keys: row << cbits | col with cbits bits per vertex id.
  int cbits = 1;
  while (cbits < 32 && ((int64_t)1 << cbits) < n) ++cbits;
  const uint64_t max_items = (uint64_t)h_cnt[2] + 1;  // one item per kept pair
  unsigned long long* rowcnt = nullptr;
  unsigned long long* lowcnt = nullptr;
  uint8_t* diag = nullptr;
  int64_t* row_ptr = nullptr;
  void* scan_tmp = nullptr;
  unsigned long long* ikeys = nullptr;
  uint32_t* ivals = nullptr;
  if ((rc = S.get((void**)&rowcnt, sizeof(unsigned long long) * n, "row counts"))) return rc;
  if ((rc = S.get((void**)&lowcnt, sizeof(unsigned long long) * n + n, "lower row counts"))) return rc;
  diag = reinterpret_cast<uint8_t*>(lowcnt + n);
  if ((rc = S.get(&scan_tmp, scan_tmp_bytes(n), "scan scratch"))) return rc;
  if ((rc = S.get((void**)&ikeys, sizeof(unsigned long long) * max_items, "csr items"))) return rc;
  if ((rc = S.get((void**)&ivals, sizeof(uint32_t) * max_items, "csr item values"))) return rc;
  if ((rc = dalloc(ctx, (void**)&row_ptr, sizeof(int64_t) * (n + 1), "row_ptr"))) return rc;
  LNE_CUDA_TRY(cudaMemsetAsync(rowcnt, 0, sizeof(unsigned long long) * n, st));
  LNE_CUDA_TRY(cudaMemsetAsync(lowcnt, 0, sizeof(unsigned long long) * n + n, st));
  // the trunc-log reads the pair table, or the dense distinct pairs of the
  // sliced aggregation (every slot occupied)
  const Slot* tsrc = sliced ? uniq : table;
  const uint64_t tcap = sliced ? (uint64_t)h_cnt[2] : cap;
  const unsigned tgrid = grid_for((int64_t)tcap, 256, (int64_t)ctx->num_sms * 16);
  if (p->sample)
    k_trunclog<true, false><<<tgrid, 256, 0, st>>>(tsrc, tcap, g->vdata, factor, p->upper,
                                            (const LogTable*)ctx->log_table, rowcnt, lowcnt, diag, counters + 3, counters + 4,
                                            cbits, max_items, ikeys, ivals, ctx->d_flags);
  else if (sliced)
    k_trunclog<false, true><<<tgrid, 256, 0, st>>>(tsrc, tcap, g->vdata, factor, p->upper,
                                                   (const LogTable*)ctx->log_table, rowcnt, lowcnt, diag, counters + 3,
                                                   counters + 4, cbits, max_items, ikeys, ivals, ctx->d_flags);
  else
    k_trunclog<false, false><<<tgrid, 256, 0, st>>>(tsrc, tcap, g->vdata, factor, p->upper,
                                                    (const LogTable*)ctx->log_table, rowcnt, lowcnt, diag, counters + 3,
                                                    counters + 4, cbits, max_items, ikeys, ivals, ctx->d_flags);
  if (table) S.release(table);
  if (uniq) S.release(uniq);
  cudaEventRecord(ev.e[2], st);
  // Row pointers and, for the full matrix, each row's offsets for the two
  // sorts: [full | tcnt | upstart | tstart | upoff | looff]
  int64_t* offs = nullptr;
  int64_t *upoff = nullptr, *looff = nullptr;
  int extra_launches = 3;  // the row pointer scan
  if (!p->upper) {
    if ((rc = dalloc(ctx, (void**)&offs, sizeof(int64_t) * (6 * (size_t)n + 2), "csr offsets"))) {
      dfree(ctx, row_ptr);
      return rc;
    }
    int64_t* full = offs;
    int64_t* tcnt = offs + n;
    int64_t* upstart = offs + 2 * n;
    int64_t* tstart = offs + 3 * n + 1;
    upoff = offs + 4 * n + 2;
    looff = offs + 5 * n + 2;
    const unsigned og = grid_for(n, 256, (int64_t)ctx->num_sms * 16);
    k_sym_counts<<<og, 256, 0, st>>>(rowcnt, lowcnt, diag, n, full, tcnt);
    scan_exclusive_i64(full, row_ptr, n, scan_tmp, st);
    scan_exclusive_i64((const int64_t*)rowcnt, upstart, n, scan_tmp, st);
    scan_exclusive_i64(tcnt, tstart, n, scan_tmp, st);
    k_sym_offsets<<<og, 256, 0, st>>>(row_ptr, lowcnt, upstart, tstart, n, upoff, looff);
    extra_launches += 2 + 6;
  } else {
    scan_exclusive_i64((const int64_t*)rowcnt, row_ptr, n, scan_tmp, st);
  }
  int64_t nnz = 0;
  unsigned long long tail[2] = {0, 0};  // kept pairs, appended items
  LNE_CUDA_TRY(cudaMemcpyAsync(&nnz, row_ptr + n, 8, cudaMemcpyDeviceToHost, st));
  LNE_CUDA_TRY(cudaMemcpyAsync(tail, counters + 3, sizeof(tail), cudaMemcpyDeviceToHost, st));
  LNE_CUDA_TRY(cudaMemcpyAsync(h_flags, ctx->d_flags, sizeof(h_flags), cudaMemcpyDeviceToHost, st));
  LNE_CUDA_TRY(cudaStreamSynchronize(st));
  LNE_CUDA_TRY(cudaGetLastError());
  const unsigned long long kept = tail[0];
  const int64_t items = (int64_t)tail[1];
  if (h_flags[kFlagSortOverflow] || tail[1] != kept || (p->upper && items != nnz) || items > nnz) {
    dfree(ctx, row_ptr);
    dfree(ctx, offs);
    set_error("lne_sparsify: CSR item count does not match the row counts (internal sizing error)");
    return LNE_ERR_UNSUPPORTED;
  }
  S.release(rowcnt);
  S.release(lowcnt);
  S.release(scan_tmp);

  // Sort the upper-triangle items by (row, col), writing each entry at its
  // final CSR position, and (full matrix) sort their transpose by row to
  // place the lower triangle: ceil(2 cbits / 8) + ceil(cbits / 8) passes over
  // one item per kept pair instead of sorting both orientations.  (Placing the items into
  // their rows at atomic cursors and sorting each row, as the hash-range
  // rounds do, measured slower here: the cursor atomics and scattered 4-byte
  // writes ran at ~29G entries/s, and the per-row sorts cost more than the
  // radix passes they replace.)
  int32_t* col = nullptr;
  float* val = nullptr;
  unsigned long long* tkeys = nullptr;
  uint32_t* tvals = nullptr;
  if ((rc = dalloc(ctx, (void**)&col, sizeof(int32_t) * (nnz > 0 ? nnz : 1), "csr col")) ||
      (rc = dalloc(ctx, (void**)&val, sizeof(float) * (nnz > 0 ? nnz : 1), "csr val")) ||
      (rc = S.get((void**)&tkeys, sizeof(unsigned long long) * (items > 0 ? items : 1), "sort keys")) ||
      (rc = S.get((void**)&tvals, sizeof(uint32_t) * (items > 0 ? items : 1), "sort values"))) {
    dfree(ctx, row_ptr);
    dfree(ctx, col);
    dfree(ctx, val);
    dfree(ctx, offs);
    return rc;
  }
  // sampling and aggregation, [table sum, block sum,] trunc-log, scans
  int launches = launches_sample + (sliced ? 0 : 2) + 1 + extra_launches;
  if (p->upper)
    rc = radix_sort_pairs_to_csr(ctx, ikeys, ivals, tkeys, tvals, items, 2 * cbits, ((1ULL << cbits) - 1), col, val,
                                 &launches);
  else
    rc = radix_sort_sym_csr(ctx, ikeys, ivals, tkeys, tvals, items, cbits, upoff, looff, nnz, col, val, &launches);
  dfree(ctx, offs);
  if (rc) {
    dfree(ctx, row_ptr);
    dfree(ctx, col);
    dfree(ctx, val);
    return rc;
  }
  {
    int fl[kFlagWords];
    LNE_CUDA_TRY(cudaMemcpyAsync(fl, ctx->d_flags, sizeof(fl), cudaMemcpyDeviceToHost, st));
    LNE_CUDA_TRY(cudaStreamSynchronize(st));
    if (fl[kFlagSortOverflow]) {
      dfree(ctx, row_ptr);
      dfree(ctx, col);
      dfree(ctx, val);
      set_error("lne_sparsify: CSR entries do not match their rows (internal error)");
      return LNE_ERR_UNSUPPORTED;
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
    stats->kernel_launches = launches;
    stats->sliced = sliced ? 1 : 0;
  }
  ctx->launch_count += launches;
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
