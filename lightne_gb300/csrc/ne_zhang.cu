// -ne_method ne_zhang_et_al: the sparse log matrix of Zhang et al. (IJCAI
// 2019, sec. 3.1) that LightNE factorises instead of the NetSMF matrix,
// LightNE/PathEmbed.h:410-448.
//
// The matrix has the graph's structure (row i = the neighbours of i in file
// order) and values
//   M[i][v] = (float)(log(1 / d_i) - log(neg_v / sum_j neg_j)),
//   neg_v   = (sum over neighbours u of v of 1 / d_u)^0.75,
// all in FP64 before the narrowing, as the reference.  neg_v sums its
// neighbours in file order and the total is a fixed-order reduction; the
// reference's pbbs reductions use their own tree order, so a value can
// differ from the reference's in the last bit of the double, which the
// narrowing to float almost always removes.
#include <cuda_runtime.h>
#include <math.h>

#include <algorithm>
#include <string>
#include <vector>

#include "lne_internal.h"

namespace lne {

namespace {

constexpr int kNegBlocks = 1024;

__global__ void k_ne_negative(int64_t n, const Vertex* __restrict__ vd, const uint32_t* __restrict__ nbrs,
                              double* __restrict__ neg) {
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  const Vertex vj = vd[j];
  double s = 0.0;
  for (uint32_t e = 0; e < vj.deg; ++e) s += 1.0 / (double)vd[nbrs[vj.off + e]].deg;
  neg[j] = pow(s, 0.75);
}

// Block partials of sum(neg) in a fixed order (grid-stride per thread, then
// a fixed tree within the block); the host adds the partials in order.
__global__ void k_ne_sum_partial(int64_t n, const double* __restrict__ neg, double* __restrict__ part) {
  __shared__ double sh[256];
  double s = 0.0;
  for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < n; j += (int64_t)gridDim.x * blockDim.x)
    s += neg[j];
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = sh[0];
}

__global__ void k_ne_values(int64_t m_dir, const Vertex* __restrict__ vd, const uint32_t* __restrict__ src,
                            const uint32_t* __restrict__ nbrs, const double* __restrict__ neg, double neg_sum,
                            int32_t* __restrict__ col, float* __restrict__ val) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < m_dir; e += (int64_t)gridDim.x * blockDim.x) {
    const uint32_t u = src[e], v = nbrs[e];
    const double nominator = 1.0 / (double)vd[u].deg;
    const double denominator = neg[v] / neg_sum;
    col[e] = (int32_t)v;
    val[e] = (float)(log(nominator) - log(denominator));
  }
}

}  // namespace

}  // namespace lne

using namespace lne;

extern "C" int lne_ne_zhang_matrix(lne_ctx* ctx, const lne_graph* g, lne_csr** out) {
  LNE_CHECK_ARG(ctx && g && out, "lne_ne_zhang_matrix: NULL argument");
  *out = nullptr;
  LNE_CUDA_TRY(cudaSetDevice(ctx->device));
  cudaStream_t st = ctx->stream;
  const int64_t n = g->n, m = g->m_dir;
  double* neg = nullptr;
  int64_t* row_ptr = nullptr;
  int32_t* col = nullptr;
  float* val = nullptr;
  int rc;
  if ((rc = dalloc(ctx, (void**)&neg, sizeof(double) * ((n > 0 ? n : 1) + kNegBlocks), "ne negative"))) return rc;
  double* part = neg + (n > 0 ? n : 1);
  if ((rc = dalloc(ctx, (void**)&row_ptr, sizeof(int64_t) * (n + 1), "ne row_ptr")) ||
      (rc = dalloc(ctx, (void**)&col, sizeof(int32_t) * (m > 0 ? m : 1), "ne col")) ||
      (rc = dalloc(ctx, (void**)&val, sizeof(float) * (m > 0 ? m : 1), "ne val"))) {
    dfree(ctx, neg);
    dfree(ctx, row_ptr);
    dfree(ctx, col);
    return rc;
  }
  if (n > 0) k_ne_negative<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(n, g->vdata, g->nbrs, neg);
  k_ne_sum_partial<<<kNegBlocks, 256, 0, st>>>(n, neg, part);
  std::vector<double> h(kNegBlocks);
  LNE_CUDA_TRY(cudaMemcpyAsync(h.data(), part, sizeof(double) * kNegBlocks, cudaMemcpyDeviceToHost, st));
  LNE_CUDA_TRY(cudaMemcpyAsync(row_ptr, g->off64, sizeof(int64_t) * (n + 1), cudaMemcpyDeviceToDevice, st));
  LNE_CUDA_TRY(cudaStreamSynchronize(st));
  double neg_sum = 0.0;
  for (double x : h) neg_sum += x;
  if (m > 0) {
    const int64_t blocks = std::min<int64_t>((m + 255) / 256, (int64_t)ctx->num_sms * 32);
    k_ne_values<<<(unsigned)blocks, 256, 0, st>>>(m, g->vdata, g->src, g->nbrs, neg, neg_sum, col, val);
  }
  dfree(ctx, neg);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    dfree(ctx, row_ptr);
    dfree(ctx, col);
    dfree(ctx, val);
    set_error(std::string("lne_ne_zhang_matrix: kernel launch failed: ") + cudaGetErrorString(e));
    return LNE_ERR_CUDA;
  }
  lne_csr* c = new lne_csr();
  c->n = n;
  c->nnz = m;
  c->row_ptr = row_ptr;
  c->col = col;
  c->val = val;
  c->owned = true;
  c->stream = st;
  *out = c;
  return LNE_OK;
}
