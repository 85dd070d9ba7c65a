// Stable LSD radix sort of (u64 key, u32 value) pairs on the device, used to
// order the sparsifier's kept entries by (row, column).
//
// Each pass sorts by one digit of at most 8 bits (reduce-then-scan):
//   k_radix_hist     per-tile digit counts (tile = 2048 consecutive items,
//                    one warp each), stored digit-major, so that one
//                    exclusive scan over [digit][tile] gives every tile the
//                    output start of each of its digits;
//   k_radix_scatter  each warp ranks its 256 items of the tile by warp
//                    multisplit (lanes with equal digits found by one ballot
//                    per digit bit; rounds in index order), the warps'
//                    counts are combined into tile-local digit offsets, the
//                    tile is reordered by digit in shared memory and then
//                    written out in runs of equal digits, so that the global
//                    writes are contiguous.
// Items with equal digits keep their input order in every pass, so the sort
// is stable.
#include <cuda_runtime.h>

#include <algorithm>
#include <string>

#include "lne_internal.h"
#include "lne_math.cuh"
#include "radix.h"

namespace lne {

namespace {

constexpr int kRadixThreads = 256;
constexpr int kRadixWarps = kRadixThreads / 32;
constexpr int kRadixItems = 8;                             // per thread
constexpr int kRadixTile = kRadixThreads * kRadixItems;    // 2048 items
constexpr int kWarpItems = 32 * kRadixItems;               // 256 items per warp
constexpr int kMaxBins = 256;
constexpr unsigned kFull = 0xffffffffu;
constexpr size_t kTileBytes = (size_t)kRadixTile * (sizeof(unsigned long long) + sizeof(uint32_t));
constexpr size_t kScatterSmem = 2 * kTileBytes;  // raw tile + reordered tile

// 16-byte cp.async global -> shared; source bytes past `src_bytes` land as zeros.
__device__ __forceinline__ void cp_async16(uint32_t dst, const void* src, uint32_t src_bytes) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(dst), "l"(src), "r"(src_bytes) : "memory");
}

// Lanes of the warp whose `dbits`-bit digit equals this lane's, among the
// lanes with `valid` set: one ballot per digit bit (warp multisplit; the
// hardware match instruction is much slower for many distinct values).
__device__ __forceinline__ unsigned match_digit(unsigned d, bool valid, int dbits) {
  unsigned m = __ballot_sync(kFull, valid);
#pragma unroll
  for (int b = 0; b < 8; ++b) {
    if (b < dbits) {
      const bool bit = (d >> b) & 1u;
      const unsigned bb = __ballot_sync(kFull, bit);
      m &= bit ? bb : ~bb;
    }
  }
  return m;
}

// The digit of a key: bits shift.. of the key itself (the CSR sort), or of
// the key's pair-table slot hash64_2(key) & hmask (the insert partition).
enum DigitMode : int { kDigitKey = 0, kDigitSlot = 1 };
template <int MODE>
__device__ __forceinline__ unsigned digit_of(unsigned long long key, int shift, unsigned long long mask,
                                             unsigned long long hmask) {
  if (MODE == kDigitSlot) return (unsigned)(((hash64_2(key) & hmask) >> shift) & mask);
  return (unsigned)((key >> shift) & mask);
}

// One warp per tile: the warp counts its tile's digits into its own
// shared histogram (plain shared atomics) and writes the tile's column of
// the [digit][tile] table, so the per-tile work outside the counting is one
// pass over the bins.  No block-wide barrier.
static unsigned hist_grid(int64_t ntiles) { return (unsigned)((ntiles + kRadixWarps - 1) / kRadixWarps); }

template <int MODE>
__global__ void __launch_bounds__(kRadixThreads) k_radix_hist(const unsigned long long* __restrict__ keys,
                                                               int64_t count, int shift, int dbits, int64_t ntiles,
                                                               int64_t* __restrict__ hist, unsigned long long hmask) {
  const int bins = 1 << dbits;
  __shared__ unsigned int h[kRadixWarps][kMaxBins];
  const int lane = threadIdx.x & 31;
  const int64_t tile = (int64_t)blockIdx.x * kRadixWarps + (threadIdx.x >> 5);
  if (tile >= ntiles) return;  // the same for the whole warp
  unsigned int* my = h[threadIdx.x >> 5];
  for (int d = lane; d < bins; d += 32) my[d] = 0;
  __syncwarp();
  const int64_t base = tile * kRadixTile;
  const unsigned long long mask = (unsigned long long)(bins - 1);
#pragma unroll 8
  for (int r = 0; r < kRadixTile / 32; ++r) {
    const int64_t i = base + (int64_t)r * 32 + lane;
    if (i < count) atomicAdd(&my[digit_of<MODE>(keys[i], shift, mask, hmask)], 1u);
  }
  __syncwarp();
  for (int d = lane; d < bins; d += 32) hist[(int64_t)d * ntiles + tile] = my[d];
}

// Exclusive scan of v over the block's threads (kRadixThreads); returns the
// prefix of this thread.  `warp_tot` is kRadixWarps words of shared memory.
__device__ __forceinline__ unsigned block_excl_scan_u32(unsigned v, unsigned* warp_tot) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  unsigned incl = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const unsigned t = __shfl_up_sync(kFull, incl, o);
    if (lane >= o) incl += t;
  }
  if (lane == 31) warp_tot[wid] = incl;
  __syncthreads();
  unsigned before = 0;
  for (int w = 0; w < wid; ++w) before += warp_tot[w];
  return before + incl - v;
}

// Output of a pass (OUT):
//   kOutNext   key and value to the next pass's buffers;
//   kOutCsr    column = key & col_mask and the value (as float) to the CSR
//              arrays at the sorted position;
//   kOutUpper  an upper-triangle item (u << cb | v): its CSR entry at
//              off[u] + position, and its transpose (v << cb | u) to the
//              next pass's buffers at the sorted position;
//   kOutLower  a transposed item (v << cb | u): unless u == v, its CSR entry
//              at off[v] + position.
// A CSR position outside [0, nnz) (inconsistent counts) sets
// kFlagSortOverflow instead of being written.  The
// tile is first copied to shared memory with cp.async (24 KB in flight per
// CTA, no registers held), ranked from there, reordered into a second
// shared buffer and written out.
enum OutMode : int { kOutNext = 0, kOutCsr = 1, kOutUpper = 2, kOutLower = 3 };
template <int OUT, int MODE, bool VALS>
__global__ void __launch_bounds__(kRadixThreads, 4) k_radix_scatter(
    const unsigned long long* __restrict__ keys, const uint32_t* __restrict__ vals, int64_t count, int shift, int dbits,
    int64_t ntiles, const int64_t* __restrict__ offs, unsigned long long* __restrict__ okeys,
    uint32_t* __restrict__ ovals, int32_t* __restrict__ ocol, float* __restrict__ oval, unsigned long long col_mask,
    unsigned long long hmask, const int64_t* __restrict__ off = nullptr, int cb = 0, int64_t nnz = 0,
    int* __restrict__ flags = nullptr) {
  extern __shared__ __align__(16) unsigned char radix_smem[];
  unsigned long long* skey = reinterpret_cast<unsigned long long*>(radix_smem);
  uint32_t* sval = reinterpret_cast<uint32_t*>(radix_smem + sizeof(unsigned long long) * kRadixTile);
  unsigned long long* rkey = reinterpret_cast<unsigned long long*>(radix_smem + kTileBytes);
  uint32_t* rval = reinterpret_cast<uint32_t*>(radix_smem + kTileBytes + sizeof(unsigned long long) * kRadixTile);
  __shared__ unsigned short wcnt[kRadixWarps][kMaxBins];  // per-warp digit counts, then start offsets
  __shared__ unsigned short tile_start[kMaxBins];          // tile-local start of each digit
  __shared__ int64_t gstart[kMaxBins];                     // global start of each digit for this tile
  __shared__ unsigned warp_tot[kRadixWarps];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const unsigned lt = (1u << lane) - 1u;
  const int bins = 1 << dbits;
  const unsigned long long mask = (unsigned long long)(bins - 1);
  const int64_t tbase = (int64_t)blockIdx.x * kRadixTile;
  const int tcount = count - tbase < kRadixTile ? (int)(count - tbase) : kRadixTile;

  // Phase 0: the tile's keys and values into rkey / rval (zeros past the end)
  {
    const uint32_t kdst = (uint32_t)__cvta_generic_to_shared(rkey);
    const uint32_t vdst = (uint32_t)__cvta_generic_to_shared(rval);
    for (int c = threadIdx.x; c < kRadixTile / 2 + kRadixTile / 4; c += kRadixThreads) {
      if (c < kRadixTile / 2) {
        const int left = tcount - 2 * c;
        const uint32_t bytes = left >= 2 ? 16u : (left == 1 ? 8u : 0u);
        cp_async16(kdst + 16 * c, bytes ? (const void*)(keys + tbase + 2 * c) : (const void*)keys, bytes);
      } else if (VALS) {
        const int cv = c - kRadixTile / 2;
        const int left = tcount - 4 * cv;
        const uint32_t bytes = left >= 4 ? 16u : (left > 0 ? 4u * left : 0u);
        cp_async16(vdst + 16 * cv, bytes ? (const void*)(vals + tbase + 4 * cv) : (const void*)vals, bytes);
      }
    }
    asm volatile("cp.async.commit_group;\n\tcp.async.wait_group 0;" ::: "memory");
  }
  for (int d = threadIdx.x; d < bins; d += blockDim.x) gstart[d] = offs[(int64_t)d * ntiles + blockIdx.x];
  unsigned short* my = wcnt[wid];
  for (int d = lane; d < bins; d += 32) my[d] = 0;
  __syncwarp();

  __syncthreads();  // raw tile visible to every warp

  // Phase 1: warp-local stable ranks (rounds in index order, lanes in order).
  uint32_t rk[kRadixItems / 2];  // two 16-bit ranks per word
  const int wofs = wid * kWarpItems;
#pragma unroll
  for (int r = 0; r < kRadixItems; ++r) {
    const int li = wofs + r * 32 + lane;
    const bool valid = li < tcount;
    const unsigned long long key = rkey[li];
    const unsigned d = digit_of<MODE>(key, shift, mask, hmask);
    const unsigned peers = match_digit(d, valid, dbits);
    const unsigned before = valid ? my[d] : 0u;
    __syncwarp();
    const uint32_t rank = before + __popc(peers & lt);
    if (r & 1)
      rk[r >> 1] |= rank << 16;
    else
      rk[r >> 1] = rank;
    if (valid && lane == __ffs(peers) - 1) my[d] = (unsigned short)(before + __popc(peers));
    __syncwarp();
  }
  __syncthreads();

  // Phase 2: tile totals per digit, their exclusive scan, and each warp's
  // start per digit (warps in index order).
  const int d0 = threadIdx.x;  // bins <= kRadixThreads
  unsigned tot = 0;
  if (d0 < bins)
    for (int w = 0; w < kRadixWarps; ++w) tot += wcnt[w][d0];
  const unsigned start = block_excl_scan_u32(tot, warp_tot);
  if (d0 < bins) {
    tile_start[d0] = (unsigned short)start;
    unsigned s = start;
    for (int w = 0; w < kRadixWarps; ++w) {
      const unsigned c = wcnt[w][d0];
      wcnt[w][d0] = (unsigned short)s;
      s += c;
    }
  }
  __syncthreads();

  // Phase 3: reorder the tile by digit in shared memory.
#pragma unroll
  for (int r = 0; r < kRadixItems; ++r) {
    const int li = wofs + r * 32 + lane;
    if (li < tcount) {
      const unsigned long long key = rkey[li];
      const int d = (int)digit_of<MODE>(key, shift, mask, hmask);
      const unsigned pos = my[d] + ((rk[r >> 1] >> ((r & 1) * 16)) & 0xffffu);
      skey[pos] = key;
      if (VALS) sval[pos] = rval[li];
    }
  }
  __syncthreads();

  // Phase 4: write out; consecutive threads take consecutive items, which
  // fall into runs of equal digits with consecutive global positions.
  for (int j = threadIdx.x; j < tcount; j += kRadixThreads) {
    const unsigned long long key = skey[j];
    const int d = (int)digit_of<MODE>(key, shift, mask, hmask);
    const int64_t pos = gstart[d] + (j - (int)tile_start[d]);
    if (OUT == kOutCsr) {
      ocol[pos] = (int32_t)(key & col_mask);
      oval[pos] = __uint_as_float(sval[j]);
    } else if (OUT == kOutUpper) {
      const unsigned long long u = key >> cb, v = key & col_mask;
      const int64_t fp = __ldg(off + u) + pos;
      if (fp >= 0 && fp < nnz) {
        ocol[fp] = (int32_t)v;
        oval[fp] = __uint_as_float(sval[j]);
      } else {
        atomicOr(&flags[kFlagSortOverflow], 1);
      }
      okeys[pos] = (v << cb) | u;
      ovals[pos] = sval[j];
    } else if (OUT == kOutLower) {
      const unsigned long long v = key >> cb, u = key & col_mask;
      if (u != v) {
        const int64_t fp = __ldg(off + v) + pos;
        if (fp >= 0 && fp < nnz) {
          ocol[fp] = (int32_t)u;
          oval[fp] = __uint_as_float(sval[j]);
        } else {
          atomicOr(&flags[kFlagSortOverflow], 1);
        }
      }
    } else {
      okeys[pos] = key;
      if (VALS) ovals[pos] = sval[j];
    }
  }
}

}  // namespace

int radix_sort_pairs_to_csr(lne_ctx* ctx, unsigned long long* keys, uint32_t* vals, unsigned long long* keys_tmp,
                            uint32_t* vals_tmp, int64_t count, int key_bits, unsigned long long col_mask,
                            int32_t* out_col, float* out_val, int* launches) {
  if (count <= 0) return LNE_OK;
  if (key_bits < 1 || key_bits > 64) {
    set_error("radix sort: key_bits must be in [1, 64]");
    return LNE_ERR_INVALID;
  }
  cudaStream_t st = ctx->stream;
  const int passes = (key_bits + 7) / 8;
  const int dbits = (key_bits + passes - 1) / passes;  // <= 8
  const int bins = 1 << dbits;
  const int64_t ntiles = (count + kRadixTile - 1) / kRadixTile;
  if (ntiles > 0x7fffffffLL) {
    set_error("radix sort: too many items");
    return LNE_ERR_UNSUPPORTED;
  }
  const int64_t cells = (int64_t)bins * ntiles;
  char* mem = nullptr;
  const size_t hist_bytes = sizeof(int64_t) * (size_t)(cells + 1);
  const size_t scan_bytes = (scan_tmp_bytes(cells) + 255) & ~(size_t)255;
  int rc = dalloc(ctx, (void**)&mem, 2 * ((hist_bytes + 255) & ~(size_t)255) + scan_bytes, "radix histograms");
  if (rc) return rc;
  int64_t* hist = (int64_t*)mem;
  int64_t* offs = (int64_t*)(mem + ((hist_bytes + 255) & ~(size_t)255));
  void* scan_tmp = mem + 2 * ((hist_bytes + 255) & ~(size_t)255);
  cudaFuncSetAttribute(k_radix_scatter<kOutCsr, kDigitKey, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)kScatterSmem);
  cudaFuncSetAttribute(k_radix_scatter<kOutNext, kDigitKey, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)kScatterSmem);
  unsigned long long *src_k = keys, *dst_k = keys_tmp;
  uint32_t *src_v = vals, *dst_v = vals_tmp;
  for (int p = 0; p < passes; ++p) {
    const int shift = p * dbits;
    k_radix_hist<kDigitKey><<<hist_grid(ntiles), kRadixThreads, 0, st>>>(src_k, count, shift, dbits, ntiles, hist, 0);
    scan_exclusive_i64(hist, offs, cells, scan_tmp, st);
    if (p == passes - 1) {
      k_radix_scatter<kOutCsr, kDigitKey, true><<<(unsigned)ntiles, kRadixThreads, kScatterSmem, st>>>(
          src_k, src_v, count, shift, dbits, ntiles, offs, nullptr, nullptr, out_col, out_val, col_mask, 0);
    } else {
      k_radix_scatter<kOutNext, kDigitKey, true><<<(unsigned)ntiles, kRadixThreads, kScatterSmem, st>>>(
          src_k, src_v, count, shift, dbits, ntiles, offs, dst_k, dst_v, nullptr, nullptr, 0, 0);
      std::swap(src_k, dst_k);
      std::swap(src_v, dst_v);
    }
    if (launches) *launches += 5;  // histogram, 3-launch scan, scatter
  }
  dfree(ctx, mem);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_error(std::string("radix sort: kernel launch failed: ") + cudaGetErrorString(e));
    return LNE_ERR_CUDA;
  }
  return LNE_OK;
}

int radix_sort_sym_csr(lne_ctx* ctx, unsigned long long* keys, uint32_t* vals, unsigned long long* keys_tmp,
                       uint32_t* vals_tmp, int64_t count, int cbits, const int64_t* upoff, const int64_t* looff,
                       int64_t nnz, int32_t* out_col, float* out_val, int* launches) {
  if (count <= 0) return LNE_OK;
  if (cbits < 1 || cbits > 31) {
    set_error("radix sort: cbits must be in [1, 31]");
    return LNE_ERR_INVALID;
  }
  cudaStream_t st = ctx->stream;
  const int64_t ntiles = (count + kRadixTile - 1) / kRadixTile;
  if (ntiles > 0x7fffffffLL) {
    set_error("radix sort: too many items");
    return LNE_ERR_UNSUPPORTED;
  }
  const int key_bits = 2 * cbits;
  const int passes1 = (key_bits + 7) / 8, dbits1 = (key_bits + passes1 - 1) / passes1;
  const int passes2 = (cbits + 7) / 8, dbits2 = (cbits + passes2 - 1) / passes2;
  const int bins = 1 << std::max(dbits1, dbits2);
  const int64_t cells = (int64_t)bins * ntiles;
  char* mem = nullptr;
  const size_t hist_bytes = (sizeof(int64_t) * (size_t)(cells + 1) + 255) & ~(size_t)255;
  const size_t scan_bytes = (scan_tmp_bytes(cells) + 255) & ~(size_t)255;
  int rc = dalloc(ctx, (void**)&mem, 2 * hist_bytes + scan_bytes, "radix histograms");
  if (rc) return rc;
  int64_t* hist = (int64_t*)mem;
  int64_t* offs = (int64_t*)(mem + hist_bytes);
  void* scan_tmp = mem + 2 * hist_bytes;
  for (auto kern : {k_radix_scatter<kOutNext, kDigitKey, true>, k_radix_scatter<kOutUpper, kDigitKey, true>,
                    k_radix_scatter<kOutLower, kDigitKey, true>})
    cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kScatterSmem);
  const unsigned long long cmask = (1ULL << cbits) - 1;
  unsigned long long *src_k = keys, *dst_k = keys_tmp;
  uint32_t *src_v = vals, *dst_v = vals_tmp;
  // the upper items by (u, v); the last pass places them and writes their
  // transposes (v, u) to the other buffers
  for (int p = 0; p < passes1; ++p) {
    const int shift = p * dbits1, dbits = dbits1;
    const int64_t c = (int64_t)(1 << dbits) * ntiles;
    k_radix_hist<kDigitKey><<<hist_grid(ntiles), kRadixThreads, 0, st>>>(src_k, count, shift, dbits, ntiles, hist, 0);
    scan_exclusive_i64(hist, offs, c, scan_tmp, st);
    if (p == passes1 - 1)
      k_radix_scatter<kOutUpper, kDigitKey, true><<<(unsigned)ntiles, kRadixThreads, kScatterSmem, st>>>(
          src_k, src_v, count, shift, dbits, ntiles, offs, dst_k, dst_v, out_col, out_val, cmask, 0, upoff, cbits, nnz,
          ctx->d_flags);
    else
      k_radix_scatter<kOutNext, kDigitKey, true><<<(unsigned)ntiles, kRadixThreads, kScatterSmem, st>>>(
          src_k, src_v, count, shift, dbits, ntiles, offs, dst_k, dst_v, nullptr, nullptr, 0, 0);
    std::swap(src_k, dst_k);
    std::swap(src_v, dst_v);
    if (launches) *launches += 5;
  }
  // the transposes, already ordered by u, stably by v: the lower triangle
  for (int p = 0; p < passes2; ++p) {
    const int shift = cbits + p * dbits2, dbits = dbits2;
    const int64_t c = (int64_t)(1 << dbits) * ntiles;
    k_radix_hist<kDigitKey><<<hist_grid(ntiles), kRadixThreads, 0, st>>>(src_k, count, shift, dbits, ntiles, hist, 0);
    scan_exclusive_i64(hist, offs, c, scan_tmp, st);
    if (p == passes2 - 1)
      k_radix_scatter<kOutLower, kDigitKey, true><<<(unsigned)ntiles, kRadixThreads, kScatterSmem, st>>>(
          src_k, src_v, count, shift, dbits, ntiles, offs, nullptr, nullptr, out_col, out_val, cmask, 0, looff, cbits,
          nnz, ctx->d_flags);
    else
      k_radix_scatter<kOutNext, kDigitKey, true><<<(unsigned)ntiles, kRadixThreads, kScatterSmem, st>>>(
          src_k, src_v, count, shift, dbits, ntiles, offs, dst_k, dst_v, nullptr, nullptr, 0, 0);
    std::swap(src_k, dst_k);
    std::swap(src_v, dst_v);
    if (launches) *launches += 5;
  }
  dfree(ctx, mem);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_error(std::string("radix sort: kernel launch failed: ") + cudaGetErrorString(e));
    return LNE_ERR_CUDA;
  }
  return LNE_OK;
}

int partition_by_slot(lne_ctx* ctx, const unsigned long long* keys, unsigned long long* out, int64_t count,
                      int table_bits, int* launches) {
  if (count <= 0) return LNE_OK;
  const int dbits = table_bits < 8 ? (table_bits > 0 ? table_bits : 1) : 8;
  const int shift = table_bits - dbits > 0 ? table_bits - dbits : 0;
  const int bins = 1 << dbits;
  const unsigned long long hmask = table_bits >= 64 ? ~0ULL : ((1ULL << table_bits) - 1);
  const int64_t ntiles = (count + kRadixTile - 1) / kRadixTile;
  if (ntiles > 0x7fffffffLL) {
    set_error("partition: too many keys");
    return LNE_ERR_UNSUPPORTED;
  }
  const int64_t cells = (int64_t)bins * ntiles;
  char* mem = nullptr;
  const size_t hist_bytes = (sizeof(int64_t) * (size_t)(cells + 1) + 255) & ~(size_t)255;
  int rc = dalloc(ctx, (void**)&mem, 2 * hist_bytes + scan_tmp_bytes(cells), "partition histograms");
  if (rc) return rc;
  int64_t* hist = (int64_t*)mem;
  int64_t* offs = (int64_t*)(mem + hist_bytes);
  void* scan_tmp = mem + 2 * hist_bytes;
  cudaStream_t st = ctx->stream;
  cudaFuncSetAttribute(k_radix_scatter<kOutNext, kDigitSlot, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)kScatterSmem);
  k_radix_hist<kDigitSlot><<<hist_grid(ntiles), kRadixThreads, 0, st>>>(keys, count, shift, dbits, ntiles, hist,
                                                                       hmask);
  scan_exclusive_i64(hist, offs, cells, scan_tmp, st);
  k_radix_scatter<kOutNext, kDigitSlot, false><<<(unsigned)ntiles, kRadixThreads, kScatterSmem, st>>>(
      keys, nullptr, count, shift, dbits, ntiles, offs, out, nullptr, nullptr, nullptr, 0, hmask);
  if (launches) *launches += 5;
  dfree(ctx, mem);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_error(std::string("partition: kernel launch failed: ") + cudaGetErrorString(e));
    return LNE_ERR_CUDA;
  }
  return LNE_OK;
}

int partition_by_top_bits(lne_ctx* ctx, unsigned long long* keys, unsigned long long* tmp, int64_t count,
                          int top_bits, unsigned long long** result, int* launches) {
  *result = keys;
  if (count <= 0 || top_bits <= 0) return LNE_OK;
  if (top_bits > 24) {
    set_error("partition: at most 24 top bits");
    return LNE_ERR_UNSUPPORTED;
  }
  const int passes = (top_bits + 7) / 8;
  const int dbits = (top_bits + passes - 1) / passes;
  const int bins = 1 << dbits;
  const int64_t ntiles = (count + kRadixTile - 1) / kRadixTile;
  if (ntiles > 0x7fffffffLL) {
    set_error("partition: too many keys");
    return LNE_ERR_UNSUPPORTED;
  }
  const int64_t cells = (int64_t)bins * ntiles;
  char* mem = nullptr;
  const size_t hist_bytes = (sizeof(int64_t) * (size_t)(cells + 1) + 255) & ~(size_t)255;
  int rc = dalloc(ctx, (void**)&mem, 2 * hist_bytes + scan_tmp_bytes(cells), "partition histograms");
  if (rc) return rc;
  int64_t* hist = (int64_t*)mem;
  int64_t* offs = (int64_t*)(mem + hist_bytes);
  void* scan_tmp = mem + 2 * hist_bytes;
  cudaStream_t st = ctx->stream;
  cudaFuncSetAttribute(k_radix_scatter<kOutNext, kDigitKey, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)kScatterSmem);
  unsigned long long *src = keys, *dst = tmp;
  for (int p = 0; p < passes; ++p) {
    // digits from the least significant of the top bits up; the last digit
    // may extend past bit 63, where the shifted word is zero
    const int shift = 64 - top_bits + p * dbits;
    k_radix_hist<kDigitKey><<<hist_grid(ntiles), kRadixThreads, 0, st>>>(src, count, shift, dbits, ntiles, hist, 0);
    scan_exclusive_i64(hist, offs, cells, scan_tmp, st);
    k_radix_scatter<kOutNext, kDigitKey, false><<<(unsigned)ntiles, kRadixThreads, kScatterSmem, st>>>(
        src, nullptr, count, shift, dbits, ntiles, offs, dst, nullptr, nullptr, nullptr, 0, 0);
    std::swap(src, dst);
    if (launches) *launches += 5;
  }
  *result = src;
  dfree(ctx, mem);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_error(std::string("partition: kernel launch failed: ") + cudaGetErrorString(e));
    return LNE_ERR_CUDA;
  }
  return LNE_OK;
}

}  // namespace lne
