// Host-side internals shared by the library's translation units.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <string>
#include <vector>

#include "../../include/lightne_gb300.h"

namespace lne {

// Per-thread error message, returned by lne_last_error().
void set_error(const std::string& msg);
void clear_error();

// Device flags word layout (ctx->d_flags, int32[kFlagWords]).
enum FlagIndex : int {
  kFlagTableFull = 0,   // a probe sequence exceeded the probe limit
  kFlagCountOverflow = 1,
  kFlagSortOverflow = 2,  // a device buffer sized from host counts was too small (internal)
  kFlagNumeric = 3,     // 2: a tensor-core kernel's wait timed out (the other CTAs stop waiting)
  kFlagTimeoutGuard = 4,  // always 0: the no-abort flag of the final bounded wait
  kFlagSliceOverflow = 5,  // a slice of the sliced aggregation had more pairs than its shared table
  kFlagWords = 8,
};

// Per-vertex record of a graph: CSR offset and degree (offsets < 2^32), and
// the Granlund-Montgomery multiplier of the degree for `rand % degree`.
struct __align__(16) Vertex {
  uint32_t off;
  uint32_t deg;
  uint64_t magic;
};

// Work list of one sparse operator for the row-parallel SpMM (built once,
// cached on the matrix or graph): rows with at most kChunkNnz entries are
// one work item each; longer rows are cut into kChunkNnz-entry chunks.
static constexpr int kChunkNnz = 2048;
struct SpmmPlan {
  int64_t n_short = 0;              // rows with <= kChunkNnz entries (incl. empty rows)
  int64_t n_chunks = 0;             // chunks of long rows
  int64_t n_long = 0;               // long rows
  uint32_t* short_rows = nullptr;   // [n_short]
  uint32_t* chunk_row = nullptr;    // [n_chunks]
  int64_t* chunk_begin = nullptr;   // [n_chunks] first nonzero of each chunk
  uint32_t* long_rows = nullptr;    // [n_long]
  int64_t* long_first = nullptr;    // [n_long + 1] first chunk of each long row
  void* mem = nullptr;              // one allocation backing the arrays
};

}  // namespace lne

struct lne_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  int* d_flags = nullptr;       // device int32[kFlagWords]
  int num_sms = 0;
  size_t smem_optin = 0;
  void* log_table = nullptr;    // device lne::LogTable (double-float log(c_j), 1/c_j)
  // Column panels of the SpMM dense operand: > 0, panels of at most that
  // many bytes of L2; < 0, two panels, the lowest ids up to |bytes| of L2
  // first, then the rest; 0 (the default): no panels
  int64_t spmm_panel_bytes = 0;
  // Sliced aggregation of the sparsifier's samples (counts, one batch):
  // shared-memory table size per slice (0: always the pair table in HBM)
  // and the number of slice bits (-1: chosen from the sample count).
  int sparsify_slice_slots = 8192;
  int sparsify_slice_bits = -1;
  // samples per batch of the sparsifier's sample buffer (8 B each)
  int64_t sparsify_batch_keys = (int64_t)1 << 30;
  // hash-range rounds above one batch (counts): 0 when the pair table does
  // not fit, 1 always, -1 never
  int sparsify_rounds = 0;
  // row sort of the rounds' CSR: rows of at most row_sort_warp_max entries
  // (a power of two in [32, 1024]) are sorted by one warp in registers,
  // longer rows through a shared-memory bitmap of row_sort_window_cols
  // columns at a time (0: as many as shared memory holds)
  int row_sort_warp_max = 1024;
  int64_t row_sort_window_cols = 0;
  // FP64 Jacobi sweeps after the FP32 preconditioning in the core SVDs of
  // lne_randsvd and lne_dense_embed: 1 until they converge, 0 one sweep,
  // -1 (the default) one in the 16-bit forms of lne_randsvd, else until
  // they converge
  int core_svd_fp64 = -1;
  // kernels launched by the entry points that ran on this context (each
  // adds its own count when it returns successfully)
  int64_t launch_count = 0;
};

struct lne_graph {
  int64_t n = 0;
  int64_t m_dir = 0;            // directed CSR entries (2m)
  lne::Vertex* vdata = nullptr; // {offset, degree, magic} per vertex
  uint32_t* nbrs = nullptr;     // neighbour ids in file order
  uint32_t* src = nullptr;      // source vertex of each directed entry
  int64_t* off64 = nullptr;     // offsets as given (int64[n+1])
  int64_t max_degree = 0;
  lne::SpmmPlan plan;           // adjacency SpMM work list (propagation)
  bool plan_ready = false;
};

struct lne_csr {
  int64_t n = 0;
  int64_t nnz = 0;
  int64_t* row_ptr = nullptr;
  int32_t* col = nullptr;
  float* val = nullptr;
  bool owned = true;
  cudaStream_t stream = nullptr;
  lne::SpmmPlan plan;
  bool plan_ready = false;
  // column panels for the cache-blocked SpMM (built on first use for given
  // panel bounds): seg[r * (npanels + 1) + p] = first entry of row r with
  // column >= panel_bounds[p], relative to row_ptr[r]
  std::vector<int64_t> panel_bounds;
  int npanels = 0;
  // share of the entries whose column is below hub_cols (-1: not measured)
  int64_t hub_cols = 0;
  double hub_share = -1.0;
  int32_t* seg = nullptr;
  std::vector<lne::SpmmPlan> panel_plans;
};

#define LNE_CUDA_TRY(expr)                                                           \
  do {                                                                               \
    cudaError_t _e = (expr);                                                         \
    if (_e != cudaSuccess) {                                                         \
      ::lne::set_error(std::string(#expr) + ": " + cudaGetErrorString(_e));          \
      return LNE_ERR_CUDA;                                                           \
    }                                                                                \
  } while (0)

#define LNE_CHECK_ARG(cond, msg)               \
  do {                                         \
    if (!(cond)) {                             \
      ::lne::set_error(std::string(msg));      \
      return LNE_ERR_INVALID;                  \
    }                                          \
  } while (0)

namespace lne {

// Stream-ordered copy between host and device memory on ctx->stream.  A
// page-locked host buffer mapped into the device's address space (1 MiB or
// more) is copied by a kernel: the SMs' loads and stores over the CPU-GPU
// link reach more bandwidth than one copy engine.  Anything else goes
// through cudaMemcpyAsync.
int copy_async(lne_ctx* ctx, void* dst, const void* src, size_t bytes, cudaMemcpyKind kind);

// Stream-ordered allocation on the context's stream; returns LNE_OK or
// LNE_ERR_ALLOC with the message set.
int dalloc(lne_ctx* ctx, void** p, size_t bytes, const char* what);
void dfree(lne_ctx* ctx, void* p);

// Exclusive scan of int64 counts[0..n) into out[0..n] (out[n] = total),
// on ctx->stream.  tmp must hold scan_tmp_bytes(n).
size_t scan_tmp_bytes(int64_t n);
void scan_exclusive_i64(const int64_t* counts, int64_t* out, int64_t n, void* tmp,
                        cudaStream_t stream);

// SpMM work lists (built on ctx->stream; synchronises once): a count
// kernel, three exclusive scans of three launches each, a fill kernel.
static constexpr int kPlanLaunches = 11;
int build_plan_csr(lne_ctx* ctx, lne_csr* c);
int build_plan_graph(lne_ctx* ctx, lne_graph* g);
void free_plan(SpmmPlan& p);
// Column panels [bounds[p], bounds[p + 1]) for the cache-blocked SpMM
// (bounds[0] = 0, bounds.back() = n; synchronises).
int build_panels(lne_ctx* ctx, lne_csr* c, const std::vector<int64_t>& bounds);
void free_panels(lne_csr* c);
// The share of A's entries with a column below pw, cached on the matrix in
// hub_share (synchronises once per matrix and pw).
int hub_share(lne_ctx* ctx, lne_csr* c, int64_t pw);

}  // namespace lne
