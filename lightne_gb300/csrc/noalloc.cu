// Allocation-free Gram: lne_gram_noalloc.
//
// Some callers cannot allocate device memory at the moment they need this
// product: a host process whose device memory is owned entirely by another
// allocator (a framework's caching pool, a fixed arena handed out by an
// embedding service), or code running under a hard per-process memory cap.
// For them this entry point computes the same G = A^T B as lne_gram (the
// streaming tensor-core Gram where it applies, else the CUDA-core one) but
// takes its scratch — the FP32 partial sums of at most ceil(n / 2048) row
// blocks — from a file-scope device array instead of cudaMallocAsync, and
// calls no cudaMalloc, cudaFree or allocating library routine.
//
// The array is a module-scope __device__ variable: every GPU that loads this
// library holds its 16 MiB until the process exits.  With CUDA's lazy module
// loading (the default since CUDA 12.2) the module that holds the array is
// loaded, and its 16 MiB committed, only when the array's address is first
// looked up: on the first call for a device.  A caller that will run under a
// memory cap should therefore make one call per device before the cap
// applies; a call with n = 0 does that set-up and only zeroes G.  In host
// code the array's name is a host-side stand-in, not a device address, so
// its device address is looked up with cudaGetSymbolAddress once per device,
// with that device current, on that first call (make it before any stream
// capture).  All calls share the one array and it keeps the last call's
// contents; every partial a call reads it has written first, so nothing
// needs clearing.  Calls whose work overlaps on the GPU (other streams,
// other host threads) race on the array and must be serialised by the
// caller.  The calling thread's current device is restored on return.
#include <cuda_runtime.h>

#include <algorithm>
#include <mutex>
#include <string>

#include "dense.h"
#include "lne_internal.h"

namespace lne {

// Largest scratch a call may use: ceil(n / 2048) * c1 * c2 partial sums.
static constexpr int64_t kNoAllocScratchFloats = (int64_t)1 << 22;  // 16 MiB of FP32

static __device__ __align__(256) float g_noalloc_scratch[kNoAllocScratchFloats];

namespace {

constexpr int kMaxDevices = 64;
std::mutex g_noalloc_mutex;
float* g_noalloc_ptr[kMaxDevices] = {};

// Device address of the scratch array on `device` (the current device).
int noalloc_scratch(int device, float** out) {
  if (device < 0 || device >= kMaxDevices) {
    set_error("lne_gram_noalloc: device index out of range");
    return LNE_ERR_INVALID;
  }
  std::lock_guard<std::mutex> lock(g_noalloc_mutex);
  if (!g_noalloc_ptr[device]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || p == nullptr) {
      cudaGetLastError();
      set_error(std::string("lne_gram_noalloc: cudaGetSymbolAddress failed: ") + cudaGetErrorString(e));
      return LNE_ERR_CUDA;
    }
    g_noalloc_ptr[device] = (float*)p;
  }
  *out = g_noalloc_ptr[device];
  return LNE_OK;
}

}  // namespace

}  // namespace lne

using namespace lne;

extern "C" int lne_gram_noalloc(lne_ctx* ctx, const float* A, int64_t lda, int64_t c1, const float* B, int64_t ldb,
                                int64_t c2, int64_t n, double* G) {
  LNE_CHECK_ARG(ctx && A && B && G && n >= 0 && c1 >= 1 && c2 >= 1 && lda >= c1 && ldb >= c2,
                "lne_gram_noalloc: bad argument");
  const int64_t nb = std::max<int64_t>(1, (n + 2047) / 2048);
  if (c1 > kNoAllocScratchFloats || c2 > kNoAllocScratchFloats || nb * c1 * c2 > kNoAllocScratchFloats) {
    set_error("lne_gram_noalloc: ceil(n / 2048) * c1 * c2 exceeds the 4,194,304 partial sums of the "
              "fixed 16 MiB scratch; use lne_gram");
    return LNE_ERR_UNSUPPORTED;
  }
  // the tensor-core Gram takes up to 256 columns; the CUDA-core Gram any
  // width, with one grid row per 2048-row block
  const bool tc = c1 <= 256 && c2 <= 256 && tc_gram_stream_supported(ctx, A, lda, (int)c1, B, ldb, (int)c2);
  if (!tc && nb > 65535) {
    set_error("lne_gram_noalloc: more than 65535 row blocks of 2048 on the CUDA-core path; use lne_gram");
    return LNE_ERR_UNSUPPORTED;
  }
  int prev = -1;
  if (cudaGetDevice(&prev) != cudaSuccess) {
    cudaGetLastError();
    prev = -1;
  }
  struct RestoreDevice {
    int dev;
    ~RestoreDevice() {
      if (dev >= 0) cudaSetDevice(dev);
    }
  } restore{prev};
  LNE_CUDA_TRY(cudaSetDevice(ctx->device));
  float* scratch = nullptr;
  int rc = noalloc_scratch(ctx->device, &scratch);
  if (rc) return rc;
  LNE_CUDA_TRY(cudaMemsetAsync(ctx->d_flags, 0, sizeof(int) * kFlagWords, ctx->stream));
  if (tc)
    rc = tc_gram_stream(ctx, A, lda, (int)c1, B, ldb, (int)c2, n, G, scratch, nb);
  else
    rc = gram_simt_into(ctx, A, lda, (int)c1, B, ldb, (int)c2, n, G, scratch);
  if (rc) return rc;
  LNE_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  int h = 0;
  LNE_CUDA_TRY(cudaMemcpy(&h, ctx->d_flags + kFlagNumeric, sizeof(int), cudaMemcpyDeviceToHost));
  if (h == 2) {
    set_error("lne_gram_noalloc: tensor-core wait timed out");
    return LNE_ERR_CUDA;
  }
  return LNE_OK;
}
