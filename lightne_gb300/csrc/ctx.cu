// Context, errors, graph upload, CSR handles and the device scan.
#include <cuda_runtime.h>
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <string>

#include "lne_internal.h"
#include "lne_math.cuh"

namespace lne {

static thread_local std::string g_last_error;

void set_error(const std::string& msg) { g_last_error = msg; }
void clear_error() { g_last_error.clear(); }

int dalloc(lne_ctx* ctx, void** p, size_t bytes, const char* what) {
  *p = nullptr;
  if (bytes == 0) bytes = 16;
  cudaError_t e = cudaMallocAsync(p, bytes, ctx->stream);
  if (e != cudaSuccess) {
    cudaGetLastError();
    *p = nullptr;
    char buf[256];
    snprintf(buf, sizeof(buf), "device allocation of %zu bytes for %s failed: %s", bytes, what,
             cudaGetErrorString(e));
    set_error(buf);
    return LNE_ERR_ALLOC;
  }
  return LNE_OK;
}

void dfree(lne_ctx* ctx, void* p) {
  if (p) cudaFreeAsync(p, ctx->stream);
}

// ---------------------------------------------------------------------------
// Exclusive scan of int64 counts: per-tile scan, scan of tile totals (one
// block, sequential over chunks), then add the tile offsets.
// ---------------------------------------------------------------------------
static constexpr int kScanThreads = 1024;
static constexpr int kScanItems = 4;
static constexpr int kScanTile = kScanThreads * kScanItems;

__device__ __forceinline__ long long warp_incl_scan(long long v) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    long long t = __shfl_up_sync(0xffffffffu, v, d);
    if (lane >= d) v += t;
  }
  return v;
}

// Block-wide exclusive scan of one value per thread; returns the exclusive
// prefix and writes the block total to *total.
__device__ __forceinline__ long long block_excl_scan(long long v, long long* total) {
  __shared__ long long warp_sums[32];
  __shared__ long long block_total;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  long long inc = warp_incl_scan(v);
  if (lane == 31) warp_sums[wid] = inc;
  __syncthreads();
  if (wid == 0) {
    int nw = blockDim.x >> 5;
    long long w = lane < nw ? warp_sums[lane] : 0;
    long long wi = warp_incl_scan(w);
    if (lane < nw) warp_sums[lane] = wi - w;
    if (lane == nw - 1) block_total = wi;
  }
  __syncthreads();
  long long res = inc - v + warp_sums[wid];
  *total = block_total;
  __syncthreads();
  return res;
}

__global__ void k_scan_tiles(const int64_t* __restrict__ in, int64_t* __restrict__ out, int64_t n,
                             int64_t* __restrict__ tile_tot) {
  int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanItems;
  long long v[kScanItems];
  long long s = 0;
#pragma unroll
  for (int i = 0; i < kScanItems; ++i) {
    v[i] = (base + i < n) ? in[base + i] : 0;
    s += v[i];
  }
  long long tot;
  long long pre = block_excl_scan(s, &tot);
#pragma unroll
  for (int i = 0; i < kScanItems; ++i) {
    if (base + i < n) out[base + i] = pre;
    pre += v[i];
  }
  if (threadIdx.x == 0) tile_tot[blockIdx.x] = tot;
}

__global__ void k_scan_totals(int64_t* tile_tot, int64_t ntiles, int64_t* grand) {
  long long carry = 0;
  for (int64_t b = 0; b < ntiles; b += blockDim.x) {
    int64_t i = b + threadIdx.x;
    long long v = i < ntiles ? tile_tot[i] : 0;
    long long tot;
    long long pre = block_excl_scan(v, &tot);
    if (i < ntiles) tile_tot[i] = pre + carry;
    carry += tot;
  }
  if (threadIdx.x == 0) *grand = carry;
}

__global__ void k_scan_add(int64_t* out, int64_t n, const int64_t* tile_tot) {
  int64_t base = (int64_t)blockIdx.x * kScanTile;
  long long add = tile_tot[blockIdx.x];
  for (int i = threadIdx.x; i < kScanTile; i += blockDim.x)
    if (base + i < n) out[base + i] += add;
}

size_t scan_tmp_bytes(int64_t n) {
  int64_t ntiles = (n + kScanTile - 1) / kScanTile;
  return (size_t)(ntiles + 1) * sizeof(int64_t);
}

void scan_exclusive_i64(const int64_t* counts, int64_t* out, int64_t n, void* tmp,
                        cudaStream_t stream) {
  int64_t ntiles = (n + kScanTile - 1) / kScanTile;
  int64_t* tile_tot = (int64_t*)tmp;
  if (ntiles > 0) k_scan_tiles<<<(unsigned)ntiles, kScanThreads, 0, stream>>>(counts, out, n, tile_tot);
  k_scan_totals<<<1, kScanThreads, 0, stream>>>(tile_tot, ntiles, out + n);
  if (ntiles > 0) k_scan_add<<<(unsigned)ntiles, 256, 0, stream>>>(out, n, tile_tot);
}

// ---------------------------------------------------------------------------
// Graph upload: validate the CSR on the device and derive {offset, degree}
// pairs plus the source vertex of every directed entry.
// ---------------------------------------------------------------------------
// The maximum degree is reduced per warp first: one atomic per warp rather
// than a million on one address.
__global__ void k_graph_build(const int64_t* __restrict__ off, int64_t n, int64_t m_dir,
                              Vertex* __restrict__ vdata, int* __restrict__ bad,
                              unsigned long long* __restrict__ maxdeg) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  uint32_t d = 0;
  if (i < n) {
    const int64_t a = off[i], b = off[i + 1];
    if (a < 0 || b < a || b > m_dir) {
      atomicExch(bad, 1);
      vdata[i] = Vertex{0u, 0u, 1ull};
    } else {
      d = (uint32_t)(b - a);  // m_dir < 2^32
      vdata[i] = Vertex{(uint32_t)a, d, gm_magic(d > 0 ? d : 1u)};
    }
  }
  const uint32_t wmax = __reduce_max_sync(0xffffffffu, d);
  if ((threadIdx.x & 31) == 0 && wmax > 0) atomicMax(maxdeg, (unsigned long long)wmax);
}

// Also rejects an entry whose target has no neighbours: the graph must be
// symmetric, and a walk that reached such a vertex would take `rand % 0`.
__global__ void k_graph_src(const int64_t* __restrict__ off, int64_t n, int64_t m_dir,
                            const int32_t* __restrict__ nbrs_in, uint32_t* __restrict__ nbrs,
                            uint32_t* __restrict__ src, int* __restrict__ bad) {
  // one warp per vertex
  int64_t w = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  int lane = threadIdx.x & 31;
  if (w >= n) return;
  int64_t a = off[w], b = off[w + 1];
  if (a < 0 || b < a || b > m_dir) return;  // reported by k_graph_build
  for (int64_t e = a + lane; e < b; e += 32) {
    int32_t v = nbrs_in[e];
    if (v < 0 || (int64_t)v >= n) {
      atomicExch(bad, 2);
      v = (int32_t)w;  // keep later walks in bounds; the upload fails anyway
    } else if (off[v + 1] <= off[v]) {
      atomicExch(bad, 3);
    }
    nbrs[e] = (uint32_t)v;
    src[e] = (uint32_t)w;
  }
}

}  // namespace lne

using namespace lne;

extern "C" {

const char* lne_last_error(void) { return g_last_error.c_str(); }
const char* lne_version(void) { return "lightne_gb300 0.1 (sm_103a)"; }

int lne_ctx_create(lne_ctx** out, int device, void* stream) {
  LNE_CHECK_ARG(out != nullptr, "lne_ctx_create: out is NULL");
  *out = nullptr;
  int ndev = 0;
  LNE_CUDA_TRY(cudaGetDeviceCount(&ndev));
  LNE_CHECK_ARG(device >= 0 && device < ndev, "lne_ctx_create: bad device index");
  LNE_CUDA_TRY(cudaSetDevice(device));
  lne_ctx* c = new lne_ctx();
  c->device = device;
  // all work is ordered on the caller's stream (NULL: the default stream)
  c->stream = (cudaStream_t)stream;
  c->own_stream = false;
  cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, device);
  int optin = 0;
  cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, device);
  c->smem_optin = (size_t)optin;
  // Keep freed stream-ordered memory cached in the pool between calls.
  cudaMemPool_t pool;
  if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
    uint64_t thr = UINT64_MAX;
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
  }
  if (cudaMalloc(&c->d_flags, sizeof(int) * kFlagWords) != cudaSuccess) {
    cudaGetLastError();
    if (c->own_stream) cudaStreamDestroy(c->stream);
    delete c;
    set_error("lne_ctx_create: cannot allocate device flags");
    return LNE_ERR_ALLOC;
  }
  cudaMemset(c->d_flags, 0, sizeof(int) * kFlagWords);
  {
    // log(1 + j/128) and 1/(1 + j/128) as double-floats, from long double
    LogTable T;
    for (int j = 0; j < 128; ++j) {
      const long double cj = 1.0L + (long double)j / 128.0L, lg = logl(cj), inv = 1.0L / cj;
      T.log_hi[j] = (float)lg;
      T.log_lo[j] = (float)(lg - (long double)T.log_hi[j]);
      T.inv_hi[j] = (float)inv;
      T.inv_lo[j] = (float)(inv - (long double)T.inv_hi[j]);
    }
    if (cudaMalloc(&c->log_table, sizeof(LogTable)) != cudaSuccess ||
        cudaMemcpy(c->log_table, &T, sizeof(LogTable), cudaMemcpyHostToDevice) != cudaSuccess) {
      cudaGetLastError();
      cudaFree(c->d_flags);
      delete c;
      set_error("lne_ctx_create: cannot set up the log table");
      return LNE_ERR_ALLOC;
    }
  }
  *out = c;
  clear_error();
  return LNE_OK;
}

int lne_ctx_destroy(lne_ctx* ctx) {
  if (!ctx) return LNE_OK;
  cudaSetDevice(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  cudaFree(ctx->d_flags);
  cudaFree(ctx->log_table);
  if (ctx->own_stream) cudaStreamDestroy(ctx->stream);
  delete ctx;
  return LNE_OK;
}

int lne_ctx_set_spmm_panel_bytes(lne_ctx* ctx, int64_t bytes) {
  LNE_CHECK_ARG(ctx != nullptr, "lne_ctx_set_spmm_panel_bytes: bad argument");
  ctx->spmm_panel_bytes = bytes;
  return LNE_OK;
}

int lne_ctx_set_sparsify_slices(lne_ctx* ctx, int32_t slots, int32_t slice_bits) {
  LNE_CHECK_ARG(ctx != nullptr, "lne_ctx_set_sparsify_slices: ctx is NULL");
  LNE_CHECK_ARG(slots == 0 || (slots >= 64 && slots <= 8192 && (slots & (slots - 1)) == 0),
                "lne_ctx_set_sparsify_slices: slots must be 0 or a power of two in [64, 8192]");
  LNE_CHECK_ARG(slice_bits >= -1 && slice_bits <= 16, "lne_ctx_set_sparsify_slices: slice_bits must be in [-1, 16]");
  ctx->sparsify_slice_slots = slots;
  ctx->sparsify_slice_bits = slice_bits;
  return LNE_OK;
}

int lne_ctx_set_sparsify_batch(lne_ctx* ctx, int64_t keys) {
  LNE_CHECK_ARG(ctx != nullptr, "lne_ctx_set_sparsify_batch: ctx is NULL");
  LNE_CHECK_ARG(keys == 0 || (keys >= 1024 && keys <= ((int64_t)1 << 34)),
                "lne_ctx_set_sparsify_batch: keys must be 0 (default) or in [1024, 2^34]");
  ctx->sparsify_batch_keys = keys == 0 ? ((int64_t)1 << 30) : keys;
  return LNE_OK;
}

int lne_ctx_synchronize(lne_ctx* ctx) {
  LNE_CHECK_ARG(ctx != nullptr, "lne_ctx_synchronize: ctx is NULL");
  LNE_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  return LNE_OK;
}

int lne_ctx_set_sparsify_rounds(lne_ctx* ctx, int32_t mode, int32_t row_sort_max) {
  LNE_CHECK_ARG(ctx != nullptr && mode >= -1 && mode <= 1, "lne_ctx_set_sparsify_rounds: bad argument");
  LNE_CHECK_ARG(row_sort_max == 0 || (row_sort_max >= 32 && row_sort_max <= 1024 &&
                                      (row_sort_max & (row_sort_max - 1)) == 0),
                "lne_ctx_set_sparsify_rounds: row_sort_max must be 0 or a power of two in [32, 1024]");
  ctx->sparsify_rounds = mode;
  ctx->row_sort_warp_max = row_sort_max ? row_sort_max : 1024;
  return LNE_OK;
}

int lne_ctx_set_row_sort_window(lne_ctx* ctx, int64_t cols) {
  LNE_CHECK_ARG(ctx != nullptr && cols >= 0 && cols % 2048 == 0,
                "lne_ctx_set_row_sort_window: cols must be 0 or a positive multiple of 2048");
  ctx->row_sort_window_cols = cols;
  return LNE_OK;
}

int lne_ctx_set_core_svd_fp64(lne_ctx* ctx, int32_t mode) {
  LNE_CHECK_ARG(ctx != nullptr && mode >= -1 && mode <= 1, "lne_ctx_set_core_svd_fp64: mode must be -1, 0 or 1");
  ctx->core_svd_fp64 = mode;
  return LNE_OK;
}

int lne_ctx_launch_count(const lne_ctx* ctx, int64_t* out) {
  LNE_CHECK_ARG(ctx != nullptr && out != nullptr, "lne_ctx_launch_count: NULL argument");
  *out = ctx->launch_count;
  return LNE_OK;
}

}  // extern "C"

namespace lne {

// Byte copy through the SMs: 16-byte vectors where both ends allow, bytes
// at the edges.
__global__ void k_copy_sm(const uint8_t* __restrict__ src, uint8_t* __restrict__ dst, int64_t bytes) {
  const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t nth = (int64_t)gridDim.x * blockDim.x;
  const int64_t head = (int64_t)((16 - ((uintptr_t)src & 15)) & 15);
  const bool vec = (((uintptr_t)src ^ (uintptr_t)dst) & 15) == 0 && bytes > head;
  if (!vec) {
    for (int64_t i = tid; i < bytes; i += nth) dst[i] = src[i];
    return;
  }
  const int64_t n16 = (bytes - head) / 16;
  const uint4* s16 = reinterpret_cast<const uint4*>(src + head);
  uint4* d16 = reinterpret_cast<uint4*>(dst + head);
  for (int64_t i = tid; i < n16; i += nth) d16[i] = s16[i];
  if (tid < head) dst[tid] = src[tid];
  const int64_t tail0 = head + 16 * n16;
  if (tid < bytes - tail0) dst[tail0 + tid] = src[tail0 + tid];
}

int copy_async(lne_ctx* ctx, void* dst, const void* src, size_t bytes, cudaMemcpyKind kind) {
  if (bytes == 0) return LNE_OK;
  const void* host = kind == cudaMemcpyDeviceToHost ? dst : src;
  cudaPointerAttributes a;
  if ((kind == cudaMemcpyDeviceToHost || kind == cudaMemcpyHostToDevice) &&
      cudaPointerGetAttributes(&a, host) == cudaSuccess && a.type == cudaMemoryTypeHost &&
      a.devicePointer != nullptr && bytes >= ((size_t)1 << 20)) {
    const int64_t off = (const char*)host - (const char*)a.hostPointer;
    char* hd = (char*)a.devicePointer + (a.hostPointer ? off : 0);
    const uint8_t* s = kind == cudaMemcpyDeviceToHost ? (const uint8_t*)src : (const uint8_t*)hd;
    uint8_t* d = kind == cudaMemcpyDeviceToHost ? (uint8_t*)hd : (uint8_t*)dst;
    k_copy_sm<<<(unsigned)(ctx->num_sms * 4), 512, 0, ctx->stream>>>(s, d, (int64_t)bytes);
    LNE_CUDA_TRY(cudaGetLastError());
    return LNE_OK;
  }
  cudaGetLastError();  // a failed attribute query leaves an error behind
  LNE_CUDA_TRY(cudaMemcpyAsync(dst, src, bytes, kind, ctx->stream));
  return LNE_OK;
}

}  // namespace lne

extern "C" {

static int graph_build_common(lne_ctx* ctx, lne_graph* g, const int32_t* d_nbrs_in) {
  const int64_t n = g->n;
  int* d_bad = nullptr;
  unsigned long long* d_maxdeg = nullptr;
  int rc;
  // [0, 4): int bad flag; [8, 16): u64 max degree
  if ((rc = dalloc(ctx, (void**)&d_bad, 16, "graph check"))) return rc;
  d_maxdeg = (unsigned long long*)((char*)d_bad + 8);
  LNE_CUDA_TRY(cudaMemsetAsync(d_bad, 0, 16, ctx->stream));
  if (n > 0) {
    k_graph_build<<<(unsigned)((n + 255) / 256), 256, 0, ctx->stream>>>(g->off64, n, g->m_dir, g->vdata,
                                                                      d_bad, d_maxdeg);
    int64_t threads = n * 32;
    k_graph_src<<<(unsigned)((threads + 255) / 256), 256, 0, ctx->stream>>>(g->off64, n, g->m_dir, d_nbrs_in,
                                                                          g->nbrs, g->src, d_bad);
  }
  int h_bad = 0;
  unsigned long long h_max = 0;
  LNE_CUDA_TRY(cudaMemcpyAsync(&h_bad, d_bad, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  LNE_CUDA_TRY(cudaMemcpyAsync(&h_max, d_maxdeg, 8, cudaMemcpyDeviceToHost, ctx->stream));
  LNE_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  dfree(ctx, d_bad);
  LNE_CUDA_TRY(cudaGetLastError());
  if (h_bad == 1) { set_error("lne_graph_upload: offsets are not a monotone CSR ending at m"); return LNE_ERR_INVALID; }
  if (h_bad == 2) { set_error("lne_graph_upload: neighbour id out of range [0, n)"); return LNE_ERR_INVALID; }
  if (h_bad == 3) {
    set_error("lne_graph_upload: an edge points to a vertex without neighbours (the graph is not symmetric)");
    return LNE_ERR_INVALID;
  }
  g->max_degree = (int64_t)h_max;
  return LNE_OK;
}

static int graph_alloc(lne_ctx* ctx, int64_t n, int64_t m_dir, lne_graph* g) {
  int rc;
  g->n = n;
  g->m_dir = m_dir;
  if ((rc = dalloc(ctx, (void**)&g->off64, sizeof(int64_t) * (n + 1), "graph offsets"))) return rc;
  if ((rc = dalloc(ctx, (void**)&g->vdata, sizeof(Vertex) * (n > 0 ? n : 1), "graph vertex data"))) return rc;
  if ((rc = dalloc(ctx, (void**)&g->nbrs, sizeof(uint32_t) * (m_dir > 0 ? m_dir : 1), "graph neighbours"))) return rc;
  if ((rc = dalloc(ctx, (void**)&g->src, sizeof(uint32_t) * (m_dir > 0 ? m_dir : 1), "graph sources"))) return rc;
  return LNE_OK;
}

int lne_graph_free(lne_graph* g) {
  if (!g) return LNE_OK;
  free_plan(g->plan);
  cudaFree(g->off64);
  cudaFree(g->vdata);
  cudaFree(g->nbrs);
  cudaFree(g->src);
  delete g;
  return LNE_OK;
}

static int graph_upload_impl(lne_ctx* ctx, int64_t n, const int64_t* offsets, const int32_t* nbrs,
                             bool on_device, lne_graph** out) {
  LNE_CHECK_ARG(ctx && out && offsets, "lne_graph_upload: NULL argument");
  *out = nullptr;
  LNE_CHECK_ARG(n >= 1, "lne_graph_upload: n must be >= 1");
  if (n >= (int64_t)UINT32_MAX) { set_error("lne_graph_upload: n >= 2^32 unsupported"); return LNE_ERR_UNSUPPORTED; }
  LNE_CUDA_TRY(cudaSetDevice(ctx->device));
  int64_t m_dir = 0, first = 0;
  if (on_device) {
    LNE_CUDA_TRY(cudaMemcpyAsync(&m_dir, offsets + n, 8, cudaMemcpyDeviceToHost, ctx->stream));
    LNE_CUDA_TRY(cudaMemcpyAsync(&first, offsets, 8, cudaMemcpyDeviceToHost, ctx->stream));
    LNE_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  } else {
    m_dir = offsets[n];
    first = offsets[0];
  }
  LNE_CHECK_ARG(first == 0 && m_dir >= 0, "lne_graph_upload: offsets[0] must be 0 and offsets[n] >= 0");
  LNE_CHECK_ARG(m_dir == 0 || nbrs != nullptr, "lne_graph_upload: nbrs is NULL");
  if (m_dir >= (int64_t)UINT32_MAX) {
    set_error("lne_graph_upload: 2^32 or more directed entries unsupported");
    return LNE_ERR_UNSUPPORTED;
  }
  lne_graph* g = new lne_graph();
  int rc = graph_alloc(ctx, n, m_dir, g);
  if (rc) { lne_graph_free(g); return rc; }
  const int32_t* d_nbrs_in = nullptr;
  int32_t* staged = nullptr;
  cudaMemcpyKind kind = on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
  rc = copy_async(ctx, g->off64, offsets, sizeof(int64_t) * (n + 1), kind);
  if (rc == LNE_OK && m_dir > 0) {
    if (on_device) {
      d_nbrs_in = nbrs;
    } else {
      // Stage the host neighbours in the `src` buffer's twin: copy into nbrs
      // directly and let the build kernel rewrite in place.
      staged = (int32_t*)g->nbrs;
      rc = copy_async(ctx, staged, nbrs, sizeof(int32_t) * m_dir, cudaMemcpyHostToDevice);
      d_nbrs_in = staged;
    }
  }
  if (rc) {
    lne_graph_free(g);
    return rc;
  }
  rc = graph_build_common(ctx, g, d_nbrs_in);
  if (rc) { lne_graph_free(g); return rc; }
  *out = g;
  return LNE_OK;
}

int lne_graph_upload(lne_ctx* ctx, int64_t n, const int64_t* offsets, const int32_t* nbrs,
                     lne_graph** out) {
  return graph_upload_impl(ctx, n, offsets, nbrs, false, out);
}

int lne_graph_upload_device(lne_ctx* ctx, int64_t n, const int64_t* d_offsets, const int32_t* d_nbrs,
                            lne_graph** out) {
  return graph_upload_impl(ctx, n, d_offsets, d_nbrs, true, out);
}

int lne_device_alloc(lne_ctx* ctx, int64_t bytes, void** out) {
  LNE_CHECK_ARG(ctx && out && bytes >= 0, "lne_device_alloc: bad argument");
  LNE_CUDA_TRY(cudaSetDevice(ctx->device));
  return dalloc(ctx, out, (size_t)bytes, "lne_device_alloc");
}

int lne_device_free(lne_ctx* ctx, void* p) {
  LNE_CHECK_ARG(ctx != nullptr, "lne_device_free: ctx is NULL");
  dfree(ctx, p);
  return LNE_OK;
}

int lne_copy_to_host(lne_ctx* ctx, void* host_dst, const void* dev_src, int64_t bytes) {
  LNE_CHECK_ARG(ctx && host_dst && dev_src && bytes >= 0, "lne_copy_to_host: bad argument");
  LNE_CUDA_TRY(cudaSetDevice(ctx->device));
  int rc = copy_async(ctx, host_dst, dev_src, (size_t)bytes, cudaMemcpyDeviceToHost);
  if (rc) return rc;
  LNE_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  return LNE_OK;
}

int lne_copy_to_device(lne_ctx* ctx, void* dev_dst, const void* host_src, int64_t bytes) {
  LNE_CHECK_ARG(ctx && dev_dst && host_src && bytes >= 0, "lne_copy_to_device: bad argument");
  LNE_CUDA_TRY(cudaSetDevice(ctx->device));
  int rc = copy_async(ctx, dev_dst, host_src, (size_t)bytes, cudaMemcpyHostToDevice);
  if (rc) return rc;
  LNE_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  return LNE_OK;
}

int lne_csr_info(const lne_csr* c, int64_t* n, int64_t* nnz) {
  LNE_CHECK_ARG(c != nullptr, "lne_csr_info: csr is NULL");
  if (n) *n = c->n;
  if (nnz) *nnz = c->nnz;
  return LNE_OK;
}

int lne_csr_download(lne_ctx* ctx, const lne_csr* c, int64_t* row_ptr, int32_t* col, float* val) {
  LNE_CHECK_ARG(ctx && c, "lne_csr_download: NULL argument");
  int rc;
  if (row_ptr && (rc = copy_async(ctx, row_ptr, c->row_ptr, sizeof(int64_t) * (c->n + 1), cudaMemcpyDeviceToHost)))
    return rc;
  if (col && c->nnz && (rc = copy_async(ctx, col, c->col, sizeof(int32_t) * c->nnz, cudaMemcpyDeviceToHost)))
    return rc;
  if (val && c->nnz && (rc = copy_async(ctx, val, c->val, sizeof(float) * c->nnz, cudaMemcpyDeviceToHost)))
    return rc;
  LNE_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  return LNE_OK;
}

int lne_csr_device_ptrs(const lne_csr* c, const int64_t** row_ptr, const int32_t** col, const float** val) {
  LNE_CHECK_ARG(c != nullptr, "lne_csr_device_ptrs: csr is NULL");
  if (row_ptr) *row_ptr = c->row_ptr;
  if (col) *col = c->col;
  if (val) *val = c->val;
  return LNE_OK;
}

int lne_csr_wrap_device(lne_ctx* ctx, int64_t n, int64_t nnz, const int64_t* d_row_ptr, const int32_t* d_col,
                        const float* d_val, lne_csr** out) {
  LNE_CHECK_ARG(ctx && out && d_row_ptr && n >= 1 && nnz >= 0, "lne_csr_wrap_device: bad argument");
  LNE_CHECK_ARG(nnz == 0 || (d_col && d_val), "lne_csr_wrap_device: NULL col/val");
  lne_csr* c = new lne_csr();
  c->n = n;
  c->nnz = nnz;
  c->row_ptr = const_cast<int64_t*>(d_row_ptr);
  c->col = const_cast<int32_t*>(d_col);
  c->val = const_cast<float*>(d_val);
  c->owned = false;
  c->stream = ctx->stream;
  *out = c;
  return LNE_OK;
}

int lne_csr_free(lne_csr* c) {
  if (!c) return LNE_OK;
  free_plan(c->plan);
  free_panels(c);
  if (c->owned) {
    cudaFree(c->row_ptr);
    cudaFree(c->col);
    cudaFree(c->val);
  }
  delete c;
  return LNE_OK;
}

}  // extern "C"
