// SpMM front end: work-list planning, configuration dispatch and the
// public lne_spmm entry point (mkl_sparse_s_mm, row-major, non-transposed).
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <string>

#include "lne_internal.h"
#include "spmm_core.cuh"
#include "spmm_dispatch.cuh"

namespace lne {

template <class Rows>
__global__ void k_plan_count(Rows R, int64_t n, int64_t* __restrict__ is_short, int64_t* __restrict__ nchunk,
                             int64_t* __restrict__ is_long) {
  const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n) return;
  const int64_t len = R.end(r) - R.begin(r);
  const bool lg = len > kChunkNnz;
  is_short[r] = lg ? 0 : 1;
  is_long[r] = lg ? 1 : 0;
  nchunk[r] = lg ? (len + kChunkNnz - 1) / kChunkNnz : 0;
}

template <class Rows>
__global__ void k_plan_fill(Rows R, int64_t n, const int64_t* __restrict__ pos_short,
                            const int64_t* __restrict__ pos_chunk, const int64_t* __restrict__ pos_long,
                            SpmmPlan p) {
  const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n) return;
  const int64_t b = R.begin(r), len = R.end(r) - b;
  if (len <= kChunkNnz) {
    p.short_rows[pos_short[r]] = (uint32_t)r;
  } else {
    const int64_t L = pos_long[r], c0 = pos_chunk[r];
    p.long_rows[L] = (uint32_t)r;
    p.long_first[L] = c0;
    const int64_t nc = (len + kChunkNnz - 1) / kChunkNnz;
    for (int64_t c = 0; c < nc; ++c) {
      p.chunk_row[c0 + c] = (uint32_t)r;
      p.chunk_begin[c0 + c] = b + c * kChunkNnz;
    }
  }
  if (r == n - 1) p.long_first[pos_long[n]] = pos_chunk[n];
}

template <class Rows>
static int build_plan(lne_ctx* ctx, Rows R, int64_t n, SpmmPlan& plan) {
  cudaStream_t st = ctx->stream;
  int64_t* cnt = nullptr;  // 3 count arrays + 3 position arrays (n+1 each)
  void* tmp = nullptr;
  int rc;
  if ((rc = dalloc(ctx, (void**)&cnt, sizeof(int64_t) * 6 * (n + 1), "spmm plan counts"))) return rc;
  if ((rc = dalloc(ctx, &tmp, scan_tmp_bytes(n), "spmm plan scan"))) { dfree(ctx, cnt); return rc; }
  int64_t *is_short = cnt, *nchunk = cnt + (n + 1), *is_long = cnt + 2 * (n + 1);
  int64_t *pos_short = cnt + 3 * (n + 1), *pos_chunk = cnt + 4 * (n + 1), *pos_long = cnt + 5 * (n + 1);
  const unsigned g = (unsigned)((n + 255) / 256);
  k_plan_count<<<g, 256, 0, st>>>(R, n, is_short, nchunk, is_long);
  scan_exclusive_i64(is_short, pos_short, n, tmp, st);
  scan_exclusive_i64(nchunk, pos_chunk, n, tmp, st);
  scan_exclusive_i64(is_long, pos_long, n, tmp, st);
  int64_t tot[3];
  LNE_CUDA_TRY(cudaMemcpyAsync(&tot[0], pos_short + n, 8, cudaMemcpyDeviceToHost, st));
  LNE_CUDA_TRY(cudaMemcpyAsync(&tot[1], pos_chunk + n, 8, cudaMemcpyDeviceToHost, st));
  LNE_CUDA_TRY(cudaMemcpyAsync(&tot[2], pos_long + n, 8, cudaMemcpyDeviceToHost, st));
  LNE_CUDA_TRY(cudaStreamSynchronize(st));
  plan.n_short = tot[0];
  plan.n_chunks = tot[1];
  plan.n_long = tot[2];
  const size_t bytes = sizeof(uint32_t) * (plan.n_short + plan.n_chunks + plan.n_long) +
                       sizeof(int64_t) * (plan.n_chunks + plan.n_long + 1) + 64;
  char* m = nullptr;
  if ((rc = dalloc(ctx, (void**)&m, bytes, "spmm plan"))) { dfree(ctx, tmp); dfree(ctx, cnt); return rc; }
  plan.mem = m;
  plan.chunk_begin = (int64_t*)m;
  plan.long_first = plan.chunk_begin + plan.n_chunks;
  plan.short_rows = (uint32_t*)(plan.long_first + plan.n_long + 1);
  plan.chunk_row = plan.short_rows + plan.n_short;
  plan.long_rows = plan.chunk_row + plan.n_chunks;
  k_plan_fill<<<g, 256, 0, st>>>(R, n, pos_short, pos_chunk, pos_long, plan);
  dfree(ctx, tmp);
  dfree(ctx, cnt);
  LNE_CUDA_TRY(cudaGetLastError());
  return LNE_OK;
}

int build_plan_csr(lne_ctx* ctx, lne_csr* c) {
  if (c->plan_ready) return LNE_OK;
  CsrRows R{c->row_ptr, c->col, c->val};
  int rc = build_plan(ctx, R, c->n, c->plan);
  if (rc == LNE_OK) c->plan_ready = true;
  return rc;
}

int build_plan_graph(lne_ctx* ctx, lne_graph* g) {
  if (g->plan_ready) return LNE_OK;
  GraphRows R{g->vdata, g->nbrs};
  int rc = build_plan(ctx, R, g->n, g->plan);
  if (rc == LNE_OK) g->plan_ready = true;
  return rc;
}

void free_plan(SpmmPlan& p) {
  if (p.mem) cudaFree(p.mem);
  p = SpmmPlan();
}

// seg[r * np1 + p] = (first entry of row r with column >= bounds[p]) - row_ptr[r]
__global__ void k_panel_seg(const int64_t* __restrict__ row_ptr, const int32_t* __restrict__ col, int64_t n,
                            const int64_t* __restrict__ bounds, int np1, int32_t* __restrict__ seg) {
  const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n) return;
  const int64_t a = row_ptr[r], b = row_ptr[r + 1];
  seg[r * np1] = 0;
  int64_t lo = a;
  for (int p = 1; p < np1; ++p) {
    const int64_t bound = bounds[p];
    int64_t hi = b;
    while (lo < hi) {  // first index in [lo, b) with col >= bound
      const int64_t mid = (lo + hi) >> 1;
      if ((int64_t)col[mid] < bound) lo = mid + 1; else hi = mid;
    }
    seg[r * np1 + p] = (int32_t)(lo - a);
  }
}

// Entries of each row with a column below pw (rows sorted by column): one
// binary search per row, summed per block.
__global__ void k_hub_count(const int64_t* __restrict__ row_ptr, const int32_t* __restrict__ col, int64_t n,
                            int64_t pw, unsigned long long* __restrict__ total) {
  const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  unsigned long long c = 0;
  if (r < n) {
    int64_t lo = row_ptr[r], hi = row_ptr[r + 1];
    const int64_t a = lo;
    while (lo < hi) {
      const int64_t mid = (lo + hi) >> 1;
      if ((int64_t)col[mid] < pw) lo = mid + 1; else hi = mid;
    }
    c = (unsigned long long)(lo - a);
  }
  for (int o = 16; o > 0; o >>= 1) c += __shfl_down_sync(0xffffffffu, c, o);
  if ((threadIdx.x & 31) == 0 && c) atomicAdd(total, c);
}

int hub_share(lne_ctx* ctx, lne_csr* c, int64_t pw) {
  if (c->hub_share >= 0.0 && c->hub_cols == pw) return LNE_OK;
  unsigned long long* d = nullptr;
  int rc;
  if ((rc = dalloc(ctx, (void**)&d, sizeof(unsigned long long), "hub count"))) return rc;
  LNE_CUDA_TRY(cudaMemsetAsync(d, 0, sizeof(unsigned long long), ctx->stream));
  k_hub_count<<<(unsigned)((c->n + 255) / 256), 256, 0, ctx->stream>>>(c->row_ptr, c->col, c->n, pw, d);
  unsigned long long h = 0;
  LNE_CUDA_TRY(cudaMemcpyAsync(&h, d, sizeof(h), cudaMemcpyDeviceToHost, ctx->stream));
  LNE_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  dfree(ctx, d);
  LNE_CUDA_TRY(cudaGetLastError());
  c->hub_cols = pw;
  c->hub_share = c->nnz > 0 ? (double)h / (double)c->nnz : 0.0;
  return LNE_OK;
}

void free_panels(lne_csr* c) {
  for (auto& p : c->panel_plans) free_plan(p);
  c->panel_plans.clear();
  if (c->seg) cudaFree(c->seg);
  c->seg = nullptr;
  c->npanels = 0;
  c->panel_bounds.clear();
}

int build_panels(lne_ctx* ctx, lne_csr* c, const std::vector<int64_t>& bounds) {
  if (c->panel_bounds == bounds && c->seg) return LNE_OK;
  free_panels(c);
  const int64_t n = c->n;
  const int np = (int)bounds.size() - 1;
  int32_t* seg = nullptr;
  int64_t* d_bounds = nullptr;
  int rc;
  if ((rc = dalloc(ctx, (void**)&seg, sizeof(int32_t) * n * (np + 1), "spmm panel segments"))) return rc;
  if ((rc = dalloc(ctx, (void**)&d_bounds, sizeof(int64_t) * (np + 1), "spmm panel bounds"))) {
    dfree(ctx, seg);
    return rc;
  }
  LNE_CUDA_TRY(cudaMemcpyAsync(d_bounds, bounds.data(), sizeof(int64_t) * (np + 1), cudaMemcpyHostToDevice,
                               ctx->stream));
  k_panel_seg<<<(unsigned)((n + 255) / 256), 256, 0, ctx->stream>>>(c->row_ptr, c->col, n, d_bounds, np + 1, seg);
  LNE_CUDA_TRY(cudaGetLastError());
  LNE_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  dfree(ctx, d_bounds);
  c->seg = seg;
  c->npanels = np;
  c->panel_bounds = bounds;
  c->panel_plans.resize(np);
  for (int p = 0; p < np; ++p) {
    PanelRows R{c->row_ptr, seg, c->col, c->val, np + 1, p};
    if ((rc = build_plan(ctx, R, n, c->panel_plans[p]))) {
      free_panels(c);
      return rc;
    }
  }
  return LNE_OK;
}

// Y = alpha * acc + beta * Y on columns < d (beta == 0 does not read Y);
// later column panels add alpha * acc.
struct EpiAxpby {
  float alpha, beta;
  float* __restrict__ Y;
  int64_t ldy;
  int d;
  bool add;
  template <int N>
  __device__ __forceinline__ void operator()(int64_t r, int e0, const float (&a)[N]) const {
    float* y = Y + r * ldy + e0;
#pragma unroll
    for (int i = 0; i < N; ++i) {
      if (e0 + i < d)
        y[i] = add ? fmaf(alpha, a[i], y[i]) : (beta == 0.f ? alpha * a[i] : fmaf(alpha, a[i], beta * y[i]));
    }
  }
};

}  // namespace lne

using namespace lne;

extern "C" int lne_spmm(lne_ctx* ctx, const lne_csr* A, int x_prec, const void* X, int64_t ldx, int64_t d,
                        float alpha, float beta, float* Y, int64_t ldy) {
  LNE_CHECK_ARG(ctx && A && X && Y, "lne_spmm: NULL argument");
  LNE_CHECK_ARG(d >= 1 && ldx >= d && ldy >= d, "lne_spmm: need 1 <= d <= ldx, ldy");
  LNE_CHECK_ARG(x_prec == LNE_PREC_FP32 || x_prec == LNE_PREC_BF16 || x_prec == LNE_PREC_FP8 ||
                    x_prec == LNE_PREC_FP16,
                "lne_spmm: x_prec must be FP32, BF16, FP16 or FP8");
  LNE_CHECK_ARG(ldx % (x_prec == LNE_PREC_FP8 ? 16 : 8) == 0 && ((uintptr_t)X % 16) == 0,
                "lne_spmm: X rows must start on 16-byte boundaries (ldx a multiple of 8, 16 for FP8)");
  LNE_CUDA_TRY(cudaSetDevice(ctx->device));
  lne_csr* Am = const_cast<lne_csr*>(A);
  EpiAxpby epi{alpha, beta, Y, ldy, (int)d, false};
  int launches = 0, rc;
  if (x_prec == LNE_PREC_FP32)
    rc = spmm_csr_panels<float>(ctx, Am, (const float*)X, ldx, d, epi, &launches);
  else if (x_prec == LNE_PREC_FP8)
    rc = spmm_csr_panels<__nv_fp8_e4m3>(ctx, Am, (const __nv_fp8_e4m3*)X, ldx, d, epi, &launches);
  else if (x_prec == LNE_PREC_FP16)
    rc = spmm_csr_panels<__half>(ctx, Am, (const __half*)X, ldx, d, epi, &launches);
  else
    rc = spmm_csr_panels<__nv_bfloat16>(ctx, Am, (const __nv_bfloat16*)X, ldx, d, epi, &launches);
  if (rc == LNE_OK) ctx->launch_count += launches;
  return rc;
}
