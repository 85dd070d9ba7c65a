// Host-side launcher of the SpMM core: picks the lane layout for the row
// width and walks column slabs of at most 128 16-byte vectors.
#pragma once
#include <cuda_runtime.h>

#include "lne_internal.h"
#include "spmm_core.cuh"

#include <algorithm>

namespace lne {

template <typename XT, int G, int VPL, class Rows, class Epi>
static void spmm_launch(lne_ctx* ctx, Rows R, const SpmmPlan& plan, const XT* X, int64_t ldx, int C, float* partial,
                        int64_t ldp, int e_base, const Epi& epi) {
  const int64_t items = plan.n_short + plan.n_chunks;
  int64_t blocks = (items + 7) / 8;
  const int64_t cap = (int64_t)ctx->num_sms * 16;
  if (blocks > cap) blocks = cap;
  if (blocks < 1) blocks = 1;
  k_spmm<XT, G, VPL, Rows, Epi><<<(unsigned)blocks, 256, 0, ctx->stream>>>(R, plan, X, ldx, C, partial, ldp, e_base,
                                                                          epi);
}

// Copies columns [v0, v0 + C) (16-byte vectors) of the x_rows rows of X
// into a dense x_rows x C array.
static __global__ void k_slab_copy(const uint4* __restrict__ X, int64_t ldv, int64_t v0, int64_t x_rows, int C,
                            uint4* __restrict__ out) {
  const int64_t total = x_rows * C;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = i / C;
    const int c = (int)(i - r * C);
    out[i] = __ldg(X + r * ldv + v0 + c);
  }
}

// A narrow slab after the first (the tail columns of a 144-wide operand)
// is gathered from a dense copy of its columns when that copy is at most
// this size: rows of the copy are 32-64 bytes instead of one 128-byte line
// per row of X, so the copy stays in L2 while the slab's gathers run.
static constexpr int64_t kSlabCopyMaxBytes = (int64_t)96 << 20;

// Runs Y-epilogue(A * X) over all rows.  X rows: ldx elements, 16-byte
// aligned; d columns are produced (the epilogue sees element offsets).
// x_rows (the rows of X; 0 if unknown) enables the tail-slab copies.
template <typename XT, class Rows, class Epi>
static int spmm_run(lne_ctx* ctx, Rows R, const SpmmPlan& plan, const XT* X, int64_t ldx, int64_t d, const Epi& epi,
                    int* launches = nullptr, int64_t x_rows = 0) {
  constexpr int E = Vec16<XT>::E;
  const int64_t c_total = (d + E - 1) / E;
  float* partial = nullptr;
  int rc;
  int nl = 0;
  // Column slabs of a power-of-two number of 16-byte vectors (at most 128),
  // largest first: each slab fills its lane layout exactly (a 144-wide FP32
  // row is a 32-vector slab and a 4-vector slab, not 36 vectors on 32 lanes).
  int64_t c_off = 0;
  while (c_off < c_total) {
    int64_t rem = c_total - c_off, C2 = 1;
    while (C2 * 2 <= rem && C2 * 2 <= 128) C2 *= 2;
    // a 144-element row is one slab of three groups of 9 lanes: 9 FP8
    // vectors (one per lane) or 18 BF16 / FP16 vectors (two per lane), so
    // its tail shares the gathers of the row instead of a second pass
    if (E == 16 && rem == 9) C2 = 9;
    if (E == 8 && rem == 18) C2 = 18;
    const int C = (int)C2;
    const int64_t ldp = (int64_t)C * E;
    if (plan.n_chunks > 0 && partial == nullptr) {
      const int64_t w = (c_total < 128 ? c_total : 128) * E;
      if ((rc = dalloc(ctx, (void**)&partial, sizeof(float) * plan.n_chunks * w, "spmm partials"))) return rc;
    }
    const XT* Xs = X + c_off * E;
    int64_t ldxs = ldx;
    XT* slab = nullptr;
    if (c_off > 0 && x_rows > 0 && x_rows * C * 16 <= kSlabCopyMaxBytes) {
      if ((rc = dalloc(ctx, (void**)&slab, (size_t)(x_rows * C * 16), "spmm slab copy"))) {
        if (partial) dfree(ctx, partial);
        return rc;
      }
      const int64_t nv = x_rows * C;
      int64_t blocks = (nv + 255) / 256;
      if (blocks > (int64_t)ctx->num_sms * 16) blocks = (int64_t)ctx->num_sms * 16;
      k_slab_copy<<<(unsigned)blocks, 256, 0, ctx->stream>>>(reinterpret_cast<const uint4*>(X), ldx / E, c_off, x_rows,
                                                             C, reinterpret_cast<uint4*>(slab));
      ++nl;
      Xs = slab;
      ldxs = (int64_t)C * E;
    }
    const int e_base = (int)(c_off * E);
    if (E == 8 && C == 18) {
      if constexpr (E == 8) spmm_launch<XT, 9, 2>(ctx, R, plan, Xs, ldxs, C, partial, ldp, e_base, epi);
    } else if (E == 16 && (C == 1 || C == 9)) {
      // FP8: one lane per nonzero for one vector, three 9-lane groups for a
      // 144-element row (instantiated for FP8 only)
      if constexpr (E == 16) {
        if (C == 1)
          spmm_launch<XT, 1, 1>(ctx, R, plan, Xs, ldxs, C, partial, ldp, e_base, epi);
        else
          spmm_launch<XT, 9, 1>(ctx, R, plan, Xs, ldxs, C, partial, ldp, e_base, epi);
      }
    } else if (C <= 2)
      spmm_launch<XT, 2, 1>(ctx, R, plan, Xs, ldxs, C, partial, ldp, e_base, epi);
    else if (C <= 4)
      spmm_launch<XT, 4, 1>(ctx, R, plan, Xs, ldxs, C, partial, ldp, e_base, epi);
    else if (C <= 8)
      spmm_launch<XT, 8, 1>(ctx, R, plan, Xs, ldxs, C, partial, ldp, e_base, epi);
    else if (C <= 16)
      spmm_launch<XT, 16, 1>(ctx, R, plan, Xs, ldxs, C, partial, ldp, e_base, epi);
    else if (C <= 32)
      spmm_launch<XT, 32, 1>(ctx, R, plan, Xs, ldxs, C, partial, ldp, e_base, epi);
    else if (C <= 64)
      spmm_launch<XT, 32, 2>(ctx, R, plan, Xs, ldxs, C, partial, ldp, e_base, epi);
    else
      spmm_launch<XT, 32, 4>(ctx, R, plan, Xs, ldxs, C, partial, ldp, e_base, epi);
    ++nl;
    if (plan.n_long > 0) {
      int64_t blocks = (plan.n_long + 7) / 8;
      if (blocks > (int64_t)ctx->num_sms * 8) blocks = (int64_t)ctx->num_sms * 8;
      k_spmm_finish<Epi><<<(unsigned)blocks, 256, 0, ctx->stream>>>(plan, partial, ldp, (int)ldp, e_base, epi);
      ++nl;
    }
    if (slab) dfree(ctx, slab);
    c_off += C;
  }
  if (partial) dfree(ctx, partial);
  if (launches) *launches += nl;
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_error(std::string("spmm launch: ") + cudaGetErrorString(e));
    return LNE_ERR_CUDA;
  }
  return LNE_OK;
}

// Cache-blocked SpMM over a CSR: when the dense operand is larger than the
// context's panel budget, the columns are cut into panels whose slice of X
// fits in L2 and one pass per panel gathers only from that slice (panels of
// at most the budget each, or, with a negative budget, two panels: the
// lowest ids up to the budget, which on graphs whose hubs have low ids
// take most of the gathers, then the rest).  The epilogue is called with
// add = false on the first panel and add = true on the later ones (fixed
// panel order: reproducible sums).
template <typename XT, class EpiT>
static int spmm_csr_panels(lne_ctx* ctx, lne_csr* A, const XT* X, int64_t ldx, int64_t d, EpiT epi,
                           int* launches = nullptr, int64_t panel_bytes = 0) {
  const int64_t row_bytes = ldx * (int64_t)sizeof(XT);
  const int64_t xbytes = A->n * row_bytes;
  // the context's setting wins; otherwise the caller's suggestion
  const int64_t want = ctx->spmm_panel_bytes != 0 ? ctx->spmm_panel_bytes : panel_bytes;
  int64_t budget = want < 0 ? -want : want;
  int rc;
  if (want < 0 && budget > 0 && xbytes > budget) {
    // a two-panel split pays only when the first panel takes most entries
    const int64_t pw = std::max<int64_t>(1, budget / row_bytes);
    if (launches && !(A->hub_share >= 0.0 && A->hub_cols == pw)) *launches += 1;
    if ((rc = hub_share(ctx, A, pw))) return rc;
    if (A->hub_share < 0.5) budget = 0;
  }
  if (budget == 0 || xbytes <= budget) {
    if (!A->plan_ready && launches) *launches += kPlanLaunches;
    if ((rc = build_plan_csr(ctx, A))) return rc;
    CsrRows R{A->row_ptr, A->col, A->val};
    epi.add = false;
    return spmm_run<XT>(ctx, R, A->plan, X, ldx, d, epi, launches, A->n);
  }
  const int64_t pw = std::max<int64_t>(1, budget / row_bytes);
  std::vector<int64_t> bounds{0};
  if (want < 0) {
    bounds.push_back(pw);
  } else {
    for (int64_t b = pw; b < A->n; b += pw) bounds.push_back(b);
  }
  bounds.push_back(A->n);
  if (A->panel_bounds != bounds && launches) *launches += 1 + (int)(bounds.size() - 1) * kPlanLaunches;
  if ((rc = build_panels(ctx, A, bounds))) return rc;
  for (int p = 0; p < A->npanels; ++p) {
    PanelRows R{A->row_ptr, A->seg, A->col, A->val, A->npanels + 1, p};
    epi.add = p > 0;
    if ((rc = spmm_run<XT>(ctx, R, A->panel_plans[p], X, ldx, d, epi, launches))) return rc;
  }
  return LNE_OK;
}

}  // namespace lne
