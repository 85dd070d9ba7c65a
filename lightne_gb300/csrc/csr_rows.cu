// Sorts the rows of a CSR by column in place, for the hash-range rounds of
// the sparsifier, which write every kept entry into its row (row_ptr is
// known from a first sweep) at an atomic cursor.
//
// Reference: the CSR build of path_embed::generate_trunc_log_matrix_v2
// (LightNE/PathEmbed.h:224-316), whose rows come out ordered by column.
//
//   k_row_sort_warp   rows of at most `warp_max` (<= 1024) entries: one warp
//                     per row, a bitonic network over 32 x KPL registers
//                     (exchanges between lanes by shuffle);
//   k_row_sort_bitmap longer rows: one thread block per row marks the row's
//                     columns in a shared-memory bitmap of the column range
//                     (or of one window of it at a time), takes a prefix
//                     count of the bitmap words, and writes each entry at
//                     its column's rank: O(entries + columns / 64) work per
//                     row, with no comparison of entries.
// Columns are distinct within a row, so the sorted order is unique and the
// result does not depend on the order the cursors left.
//
// Measured at config 2 (351M entries, 1.09M rows of at most 1024 entries,
// 46K longer rows) as the one-batch path's CSR build: the warp tier took
// 16.5 ms (about 19 instructions per entry) and the bitmap tier 5 ms, where
// that path's radix sort takes about 20 ms in all; the one-batch path
// therefore keeps the radix sort.
#include <cuda_runtime.h>

#include <algorithm>
#include <string>

#include "lne_internal.h"
#include "radix.h"

namespace lne {

namespace {

constexpr unsigned kFull = 0xffffffffu;
constexpr int kBmThreads = 1024;
constexpr int kBmWordsMax = 20480;  // 1,310,720 columns per window (160 KB of bitmap)
constexpr int kGroupWords = 32;     // bitmap words per prefix group

// Bitonic sort of one row of L <= 32 * KPL entries by one warp.  Entry i
// of the (padded) row is register i / 32 of lane i % 32, so the loads and
// stores are coalesced; a compare-exchange at distance j < 32 pairs lanes
// (shuffle), at j >= 32 registers of one lane.  The merge levels and the
// shuffle distances are runtime loops, which keeps the code small (fully
// unrolled networks for several row sizes did not fit the instruction
// cache).
template <int KPL>
__device__ __forceinline__ void warp_sort_row(const int32_t* scol, const float* sval, int32_t* dcol, float* dval,
                                              int64_t a, int L, int lane) {
  uint32_t k[KPL], v[KPL];
#pragma unroll
  for (int r = 0; r < KPL; ++r) {
    const int i = r * 32 + lane;
    k[r] = i < L ? (uint32_t)scol[a + i] : kFull;
    v[r] = i < L ? __float_as_uint(sval[a + i]) : 0u;
  }
  constexpr int P = 32 * KPL;
#pragma unroll 1
  for (int kk = 2; kk <= P; kk <<= 1) {
    // distances 32 * KPL / 2 .. 32 within a lane's registers
#pragma unroll
    for (int jr = KPL / 2; jr > 0; jr >>= 1) {
      if (jr * 32 < kk) {
#pragma unroll
        for (int r = 0; r < KPL; ++r) {
          if ((r & jr) == 0) {
            const int r2 = r | jr;
            const bool asc = ((r * 32 + lane) & kk) == 0;
            const bool sw = asc ? (k[r] > k[r2]) : (k[r] < k[r2]);
            const uint32_t tk = sw ? k[r2] : k[r], tv = sw ? v[r2] : v[r];
            k[r2] = sw ? k[r] : k[r2];
            v[r2] = sw ? v[r] : v[r2];
            k[r] = tk;
            v[r] = tv;
          }
        }
      }
    }
    // distances 16 .. 1 across lanes
#pragma unroll 1
    for (int j = (kk >= 64 ? 16 : kk >> 1); j > 0; j >>= 1) {
      const bool lower = (lane & j) == 0;
#pragma unroll
      for (int r = 0; r < KPL; ++r) {
        const uint32_t ok = __shfl_xor_sync(kFull, k[r], j);
        const uint32_t ov = __shfl_xor_sync(kFull, v[r], j);
        const bool asc = ((r * 32 + lane) & kk) == 0;
        // the lower index of an ascending pair keeps the smaller key
        const bool take = (lower == asc) ? (ok < k[r]) : (ok > k[r]);
        k[r] = take ? ok : k[r];
        v[r] = take ? ov : v[r];
      }
    }
  }
#pragma unroll
  for (int r = 0; r < KPL; ++r) {
    const int i = r * 32 + lane;
    if (i < L) {
      dcol[a + i] = (int32_t)k[r];
      dval[a + i] = __uint_as_float(v[r]);
    }
  }
}

// Rows of at most warp_max entries, one warp each; longer rows are listed
// in big[] (count in *nbig, the longest in *maxlen) for the bitmap sort.
__global__ void __launch_bounds__(256) k_row_sort_warp(const int64_t* __restrict__ row_ptr, int64_t n,
                                                        const int32_t* scol, const float* sval, int32_t* dcol,
                                                        float* dval, int warp_max, uint32_t* __restrict__ big,
                                                        unsigned long long* __restrict__ nbig,
                                                        unsigned long long* __restrict__ maxlen) {
  const int lane = threadIdx.x & 31;
  const int64_t nwarps = (int64_t)gridDim.x * (blockDim.x >> 5);
  const bool inplace = scol == dcol;
  for (int64_t r = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); r < n; r += nwarps) {
    const int64_t a = row_ptr[r];
    const int64_t len = row_ptr[r + 1] - a;
    if (len > warp_max) {
      if (lane == 0) {
        big[atomicAdd(nbig, 1ULL)] = (uint32_t)r;
        atomicMax(maxlen, (unsigned long long)len);
      }
      continue;
    }
    const int L = (int)len;
    if (L <= 1) {
      if (L == 1 && lane == 0 && !inplace) {
        dcol[a] = scol[a];
        dval[a] = sval[a];
      }
      continue;
    }
    if (L <= 32)
      warp_sort_row<1>(scol, sval, dcol, dval, a, L, lane);
    else if (L <= 64)
      warp_sort_row<2>(scol, sval, dcol, dval, a, L, lane);
    else if (L <= 128)
      warp_sort_row<4>(scol, sval, dcol, dval, a, L, lane);
    else if (L <= 256)
      warp_sort_row<8>(scol, sval, dcol, dval, a, L, lane);
    else if (L <= 512)
      warp_sort_row<16>(scol, sval, dcol, dval, a, L, lane);
    else
      warp_sort_row<32>(scol, sval, dcol, dval, a, L, lane);
  }
}

// Rows listed in big[], one thread block (kBmThreads) per row, rows taken
// in turn (block b: entries b, b + grid, ...; the next row's extent is
// loaded while the current one is sorted).  The row's columns are marked in
// a bitmap of bm_words 64-bit words per window of the column range
// [0, ncols); a warp-scan per 32-word group gives each word's count of
// marked columns before it in its group (16 bits), a scan over the groups
// their starts, and an entry's position in the sorted row is the number of
// marked columns below its own.  Rows of at most kBmRegs * kBmThreads
// entries stay in registers between the marking and the placing.
// stage != NULL (in-place sort): the row is first copied to this block's
// stage (stage_len entries) and sorted from there.
constexpr int kBmRegs = 4;
__global__ void __launch_bounds__(kBmThreads, 1) k_row_sort_bitmap(
    const int64_t* __restrict__ row_ptr, const uint32_t* __restrict__ big, const unsigned long long* __restrict__ nbig,
    int64_t ncols, int bm_words, const int32_t* scol, const float* sval, int32_t* dcol, float* dval,
    int32_t* __restrict__ stage_col, float* __restrict__ stage_val, int64_t stage_len, int* __restrict__ flags) {
  extern __shared__ __align__(16) unsigned char bm_smem[];
  unsigned long long* bm = reinterpret_cast<unsigned long long*>(bm_smem);
  uint16_t* wpre = reinterpret_cast<uint16_t*>(bm + bm_words);
  unsigned* gpre = reinterpret_cast<unsigned*>(wpre + bm_words);
  __shared__ unsigned win_total;
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  const int64_t win_cols = (int64_t)bm_words * 64;
  const int64_t nb = (int64_t)*nbig;
  int64_t bi = blockIdx.x;
  int64_t a = 0, L = 0;
  if (bi < nb) {
    const int64_t r = big[bi];
    a = row_ptr[r];
    L = row_ptr[r + 1] - a;
  }
  for (; bi < nb; bi += gridDim.x) {
    // the next row's extent
    int64_t an = 0, Ln = 0;
    if (bi + gridDim.x < nb) {
      const int64_t rn = big[bi + gridDim.x];
      an = row_ptr[rn];
      Ln = row_ptr[rn + 1] - an;
    }
    const int32_t* rc = scol + a;
    const float* rv = sval + a;
    bool ok = true;
    if (stage_col) {
      ok = L <= stage_len;  // always: stage_len is the longest listed row
      if (ok) {
        int32_t* sc = stage_col + (int64_t)blockIdx.x * stage_len;
        float* sv = stage_val + (int64_t)blockIdx.x * stage_len;
        for (int64_t i = tid; i < L; i += kBmThreads) {
          sc[i] = rc[i];
          sv[i] = rv[i];
        }
        rc = sc;
        rv = sv;
      }
      __syncthreads();  // the block's global writes are visible to the block
    }
    if (ok) {
      const bool in_regs = L <= (int64_t)kBmRegs * kBmThreads;
      int32_t ec[kBmRegs];
      float ev[kBmRegs];
      if (in_regs) {
#pragma unroll
        for (int q = 0; q < kBmRegs; ++q) {
          const int64_t i = tid + (int64_t)q * kBmThreads;
          ec[q] = i < L ? rc[i] : -1;
          ev[q] = i < L ? rv[i] : 0.0f;
        }
      }
      int64_t placed = 0;
      for (int64_t w0 = 0; w0 < ncols; w0 += win_cols) {
        const int64_t wcols = min(win_cols, ncols - w0);
        const int nw = (int)((wcols + 63) / 64);
        const int ng = (nw + kGroupWords - 1) / kGroupWords;
        for (int w = tid; w < ng * kGroupWords; w += kBmThreads) bm[w] = 0ULL;
        __syncthreads();
        if (in_regs) {
#pragma unroll
          for (int q = 0; q < kBmRegs; ++q) {
            const int64_t c = (int64_t)ec[q] - w0;
            if (ec[q] >= 0 && c >= 0 && c < wcols) atomicOr(&bm[c >> 6], 1ULL << (c & 63));
          }
        } else {
          for (int64_t i = tid; i < L; i += kBmThreads) {
            const int64_t c = (int64_t)rc[i] - w0;
            if (c >= 0 && c < wcols) atomicOr(&bm[c >> 6], 1ULL << (c & 63));
          }
        }
        __syncthreads();
        for (int g = wid; g < ng; g += kBmThreads / 32) {
          const int w = g * kGroupWords + lane;
          const unsigned x = (unsigned)__popcll(bm[w]);
          unsigned incl = x;
#pragma unroll
          for (int o = 1; o < 32; o <<= 1) {
            const unsigned t = __shfl_up_sync(kFull, incl, o);
            if (lane >= o) incl += t;
          }
          wpre[w] = (uint16_t)(incl - x);
          if (lane == 31) gpre[g] = incl;
        }
        __syncthreads();
        if (wid == 0) {
          unsigned carry = 0;
          for (int g0 = 0; g0 < ng; g0 += 32) {
            const int g = g0 + lane;
            const unsigned x = g < ng ? gpre[g] : 0u;
            unsigned incl = x;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
              const unsigned t = __shfl_up_sync(kFull, incl, o);
              if (lane >= o) incl += t;
            }
            if (g < ng) gpre[g] = carry + incl - x;
            carry += __shfl_sync(kFull, incl, 31);
          }
          if (lane == 0) win_total = carry;
        }
        __syncthreads();
        auto place = [&](int32_t col, float val) {
          const int64_t c = (int64_t)col - w0;
          if (col < 0 || c < 0 || c >= wcols) return;
          const int w = (int)(c >> 6);
          const unsigned long long below = bm[w] & ((1ULL << (c & 63)) - 1ULL);
          const int64_t pos = placed + gpre[w / kGroupWords] + wpre[w] + __popcll(below);
          if (pos < L) {
            dcol[a + pos] = col;
            dval[a + pos] = val;
          }
        };
        if (in_regs) {
#pragma unroll
          for (int q = 0; q < kBmRegs; ++q) place(ec[q], ev[q]);
        } else {
          for (int64_t i = tid; i < L; i += kBmThreads) place(rc[i], rv[i]);
        }
        placed += win_total;
        __syncthreads();  // the bitmap is cleared for the next window or row
      }
      // columns repeated within the row, or outside [0, ncols), leave fewer
      // marked columns than entries
      if (tid == 0 && placed != L) atomicOr(&flags[kFlagSortOverflow], 1);
    } else if (tid == 0) {
      atomicOr(&flags[kFlagSortOverflow], 1);
    }
    a = an;
    L = Ln;
  }
}

int bitmap_words(const lne_ctx* ctx, int64_t ncols) {
  int64_t w = ctx->row_sort_window_cols > 0 ? ctx->row_sort_window_cols / 64 : kBmWordsMax;
  w = std::min<int64_t>(w, kBmWordsMax);
  // shared memory: 8 + 2 bytes per word, 4 per group
  const int64_t fit = ((int64_t)ctx->smem_optin - 1024) / (10 + 4 / kGroupWords + 1);
  w = std::min<int64_t>(w, fit);
  const int64_t need = (ncols + 63) / 64;
  w = std::min<int64_t>(w, std::max<int64_t>(need, 1));
  w = (w + kGroupWords - 1) / kGroupWords * kGroupWords;
  return (int)w;
}

}  // namespace

int sort_csr_rows(lne_ctx* ctx, const int64_t* row_ptr, int64_t n, int64_t ncols, const int32_t* scol,
                  const float* sval, int32_t* dcol, float* dval, int* launches) {
  if (n <= 0) return LNE_OK;
  cudaStream_t st = ctx->stream;
  const bool inplace = scol == dcol;
  const int warp_max = ctx->row_sort_warp_max;
  char* mem = nullptr;
  const size_t big_bytes = ((sizeof(uint32_t) * (size_t)n + 255) & ~(size_t)255);
  int rc = dalloc(ctx, (void**)&mem, big_bytes + 64, "row sort lists");
  if (rc) return rc;
  uint32_t* big = (uint32_t*)mem;
  unsigned long long* cnt = (unsigned long long*)(mem + big_bytes);  // nbig, maxlen
  cudaError_t e = cudaMemsetAsync(cnt, 0, 64, st);
  if (e != cudaSuccess) {
    dfree(ctx, mem);
    set_error(std::string("row sort: ") + cudaGetErrorString(e));
    return LNE_ERR_CUDA;
  }
  const unsigned wgrid = (unsigned)std::min<int64_t>((n + 7) / 8, (int64_t)ctx->num_sms * 8);
  k_row_sort_warp<<<wgrid, 256, 0, st>>>(row_ptr, n, scol, sval, dcol, dval, warp_max, big, cnt, cnt + 1);
  int nl = 1;
  const int bm_words = bitmap_words(ctx, ncols);
  const size_t smem = (size_t)bm_words * 10 + (size_t)(bm_words / kGroupWords) * 4 + 16;
  e = cudaFuncSetAttribute(k_row_sort_bitmap, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) {
    dfree(ctx, mem);
    set_error(std::string("row sort: ") + cudaGetErrorString(e));
    return LNE_ERR_CUDA;
  }
  const unsigned bgrid = (unsigned)ctx->num_sms;
  int32_t* stage_col = nullptr;
  float* stage_val = nullptr;
  int64_t stage_len = 0;
  if (inplace) {
    // the in-place sort stages each long row; its length bounds the stage
    unsigned long long h[2] = {0, 0};
    e = cudaMemcpyAsync(h, cnt, sizeof(h), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
      dfree(ctx, mem);
      set_error(std::string("row sort: ") + cudaGetErrorString(e));
      return LNE_ERR_CUDA;
    }
    if (h[0] == 0) {
      dfree(ctx, mem);
      if (launches) *launches += nl;
      return LNE_OK;
    }
    stage_len = (int64_t)h[1];
    if ((rc = dalloc(ctx, (void**)&stage_col, sizeof(int32_t) * (size_t)stage_len * bgrid, "row sort stage")) ||
        (rc = dalloc(ctx, (void**)&stage_val, sizeof(float) * (size_t)stage_len * bgrid, "row sort stage"))) {
      dfree(ctx, stage_col);
      dfree(ctx, mem);
      return rc;
    }
  }
  k_row_sort_bitmap<<<bgrid, kBmThreads, smem, st>>>(row_ptr, big, cnt, ncols, bm_words, scol, sval, dcol, dval,
                                                      stage_col, stage_val, stage_len, ctx->d_flags);
  ++nl;
  if (launches) *launches += nl;
  dfree(ctx, stage_col);
  dfree(ctx, stage_val);
  dfree(ctx, mem);
  e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_error(std::string("row sort: kernel launch failed: ") + cudaGetErrorString(e));
    return LNE_ERR_CUDA;
  }
  return LNE_OK;
}

}  // namespace lne
