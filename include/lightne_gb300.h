/*
 * lightne_gb300 — C ABI of the GB300-native LightNE embedding pipeline.
 *
 * One library (liblightne_gb300.so) exports the stages of LightNE's hot path
 * as plain C entry points: pointers and sizes, no C++ or torch types.  Every
 * function returns an int status (LNE_OK == 0) and never exits the process;
 * lne_last_error() gives the message of the calling thread's last failure.
 * Work is ordered on the context's CUDA stream; a context is used by one
 * host thread at a time.
 *
 * Reference interfaces replaced (paths inside the reference project):
 *   lne_sparsify        path_embed::generate_trunc_log_matrix_v2
 *                       (LightNE/PathEmbed.h:81-369), the NetSMF sparsifier:
 *                       path sampler, par_table aggregation, trunc-log and
 *                       CSR build
 *   lne_randsvd         mkl_redsvd::MKLRedSVD<FP> ctor + run()
 *                       (LightNE/mklredsvd/mklredsvd.cc:54-403) followed by
 *                       path_embed::compute_u_sigma_root
 *                       (LightNE/PathEmbed.h:371-408)
 *   lne_propagate       spectral_propagation::chebyshev_expansion up to the
 *                       (A+I)a product (LightNE/SpectralPropagation.h:45-221)
 *   lne_dense_embed     spectral_propagation::get_embedding_dense
 *                       (LightNE/SpectralPropagation.h:16-43)
 *   lne_spmm            mkl_sparse_s_mm on a CSR (the SpMM of
 *                       LightNE/mklredsvd/mklredsvd.cc:235-245)
 *   lne_core_svd        LAPACKE_gesvd(jobu 'S', jobvt 'N') of the rank x rank
 *                       core C = Z^T B (LightNE/mklredsvd/mklredsvd.cc:357-371)
 */
#ifndef LIGHTNE_GB300_H
#define LIGHTNE_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes. */
#define LNE_OK 0
#define LNE_ERR_INVALID 1      /* bad argument */
#define LNE_ERR_ALLOC 2        /* device or host allocation failed */
#define LNE_ERR_TABLE_FULL 3   /* pair table overflow: the reference prints
                                  "looping forever" and exits 0
                                  (LightNE/par_table.h:104-107) */
#define LNE_ERR_CUDA 4         /* CUDA runtime error */
#define LNE_ERR_UNSUPPORTED 5  /* size beyond what this build handles */
#define LNE_ERR_NUMERIC 6      /* factorisation failed (e.g. non-SPD Gram) */

/* Dense operand precision of SpMM / propagation.  The 16-bit forms store
 * the dense operand every SpMM gathers in 16 bits and accumulate in FP32;
 * FP16 keeps 11 significant bits (BF16: 8) in the same bytes, on values
 * scaled by a power of two into its range. */
#define LNE_PREC_FP32 0
#define LNE_PREC_BF16 1
#define LNE_PREC_FP8 2 /* e4m3; SpMM dense operand only (lne_spmm x_prec) */
#define LNE_PREC_FP16 3

typedef struct lne_ctx lne_ctx;
typedef struct lne_graph lne_graph;
typedef struct lne_csr lne_csr;

/* Last error message of the calling thread ("" if none). */
const char* lne_last_error(void);
/* Library version string. */
const char* lne_version(void);

/* Context: device and the cudaStream_t all of its work is ordered on
 * (NULL: the default stream). */
int lne_ctx_create(lne_ctx** out, int device, void* stream);
int lne_ctx_destroy(lne_ctx* ctx);
/* L2 tuning of the SpMM over a CSR (no reference counterpart): the dense
 * operand's rows are cut into column panels of A whose slice of the
 * operand fits in L2, one gather pass per panel.  bytes > 0: panels of at
 * most that many bytes; bytes < 0: two panels, the lowest ids up to |bytes|
 * then the rest (on graphs whose hubs have the lowest ids, most gathers hit
 * the first); 0 (the default): no panels. */
int lne_ctx_set_spmm_panel_bytes(lne_ctx* ctx, int64_t bytes);
/* Aggregation of the sparsifier's pair samples (no reference counterpart:
 * the reference always inserts into par_table, LightNE/par_table.h:86-109).
 * With counts (-sample 0) and one batch of samples, lne_sparsify counts the
 * pairs slice by slice in shared-memory tables of `slots` entries (a power
 * of two in [64, 8192]; default 8192) over 2^slice_bits slices of the
 * hash space (-1, the default: chosen from the sample count; at most 16),
 * and falls back to the pair table in HBM when a slice overflows.
 * slots = 0 always uses the pair table.  The output is the same either way. */
int lne_ctx_set_sparsify_slices(lne_ctx* ctx, int32_t slots, int32_t slice_bits);
/* Samples per batch of lne_sparsify's sample buffer (no reference
 * counterpart: the reference inserts every sample into par_table as it is
 * drawn).  Default 2^30 (8 GiB of keys; 0 restores it), at least 1024.
 * Batches are sampled one edge range at a time and added to the pair table
 * in turn; only a run that fits one batch takes the sliced aggregation. */
int lne_ctx_set_sparsify_batch(lne_ctx* ctx, int64_t keys);
/* Hash-range rounds of lne_sparsify (no reference counterpart): with counts
 * (-sample 0) and more samples than one batch, the sampler is replayed in
 * rounds that each keep the samples of one range of pair hashes (a batch's
 * worth), counted by the sliced aggregation; a first sweep counts each
 * row's kept entries, a second writes them into their rows, and the rows
 * are then sorted by column.  It needs the CSR plus one batch's buffers,
 * where the pair table path needs the table and twice the CSR's entries.
 * mode 0 (the default): rounds when the pair table path (the table and a
 * batch while sampling, then the CSR build's two copies of the entries) does
 * not fit in free device memory; 1: always; -1: never.  row_sort_max (a power of
 * two in [32, 1024]; 0: 1024): the rounds' rows with at most that many
 * entries are sorted by column by one warp, longer rows by a thread block
 * through a bitmap of the column range.  The output is the same either
 * way. */
int lne_ctx_set_sparsify_rounds(lne_ctx* ctx, int32_t mode, int32_t row_sort_max);
/* Columns per window of the bitmap row sort of the hash-range rounds (no
 * reference counterpart): a multiple of 2048, or 0 (the default) for as
 * many as shared memory holds (1,310,720); a row is swept once per window
 * of the column range.  The output is the same either way. */
int lne_ctx_set_row_sort_window(lne_ctx* ctx, int64_t cols);
/* FP64 sweeps of the r x r core SVDs of lne_randsvd (mklredsvd.cc:353-371,
 * LAPACKE_sgesvd in the reference) and lne_dense_embed
 * (SpectralPropagation.h:16-43), which start from a one-sided Jacobi in
 * FP32 (columns orthogonal to |cos| <= 4e-6): mode 1 runs FP64 sweeps until
 * they converge, mode 0 one FP64 sweep (|cos| to about its square).  -1
 * (the default): one in the 16-bit forms of lne_randsvd, else until they
 * converge.  lne_core_svd always runs them to convergence. */
int lne_ctx_set_core_svd_fp64(lne_ctx* ctx, int32_t mode);
/* Wait for all work queued on the context's stream. */
int lne_ctx_synchronize(lne_ctx* ctx);
/* Kernels the pipeline entry points (lne_sparsify, lne_randsvd,
 * lne_propagate, lne_propagate_adjoint, lne_dense_embed, lne_spmm) have
 * launched on this context so far, a diagnostic with no reference
 * counterpart. */
int lne_ctx_launch_count(const lne_ctx* ctx, int64_t* out);

/*
 * Device memory helpers for callers that do not link the CUDA runtime
 * (stream-ordered on the context's stream; copies synchronise).  A host
 * buffer that is page-locked and mapped (cudaHostAlloc or cudaHostRegister
 * memory) is copied by a kernel over the CPU-GPU link, faster than a copy
 * engine; pageable memory goes through cudaMemcpyAsync.  lne_graph_upload
 * and lne_csr_download copy the same way.
 */
int lne_device_alloc(lne_ctx* ctx, int64_t bytes, void** out);
int lne_device_free(lne_ctx* ctx, void* p);
int lne_copy_to_host(lne_ctx* ctx, void* host_dst, const void* dev_src, int64_t bytes);
int lne_copy_to_device(lne_ctx* ctx, void* dev_dst, const void* host_src, int64_t bytes);

/*
 * Graph: symmetric CSR, offsets int64[n+1] (offsets[n] = number of directed
 * entries), neighbours int32[offsets[n]], in the order of the AdjacencyGraph
 * file (the walk depends on it).  Host pointers; the graph is copied to the
 * device.  Replaces gbbs_io::read_unweighted_symmetric_graph's in-memory
 * result (ligra/graph_io.h:233-250).
 */
int lne_graph_upload(lne_ctx* ctx, int64_t n, const int64_t* offsets, const int32_t* nbrs,
                     lne_graph** out);
/* Same, from device pointers (already resident in HBM). */
int lne_graph_upload_device(lne_ctx* ctx, int64_t n, const int64_t* d_offsets,
                            const int32_t* d_nbrs, lne_graph** out);
int lne_graph_free(lne_graph* g);

/* Parameters of the sparsifier; names and meaning as the LightNE flags
 * (LightNE/LightNE.cc:31-43).  sample_ratio and mem_ratio are floats, as
 * LightNE.cc:42-43 narrows them. */
typedef struct lne_sparsify_params {
  uint64_t seed;        /* pbbs::random seed (reference: time(0)) */
  int64_t walk_len;     /* -walklen (T) */
  int64_t table_size;   /* -tablesz */
  int64_t negative;     /* -negative (b) */
  int32_t sample;       /* -sample: 0 = every path, 1 = effective-resistance sampling */
  int32_t upper;        /* -upper: keep the upper triangle only */
  float sample_ratio;   /* -sample_ratio */
  float mem_ratio;      /* -mem_ratio */
} lne_sparsify_params;

/* Diagnostics of one sparsifier call (the reference prints these). */
typedef struct lne_sparsify_stats {
  double logn, total_samples, inv_lambda, frac, factor, m_exact;
  int64_t exp_rv_rounded, table_size, capacity, samples_emitted, distinct, nnz_upper, nnz;
  float ms_sample, ms_trunclog, ms_csr; /* device time per stage (CUDA events) */
  int32_t kernel_launches;              /* kernels this call launched */
  int32_t sliced;                       /* 1: pairs counted by the sliced aggregation, 0: pair table,
                                           2: hash-range rounds */
} lne_sparsify_stats;

/*
 * NetSMF sparsifier: S1-S9 of the hot path.  Output CSR (device-resident,
 * owned by the caller, free with lne_csr_free) is canonical: rows ascending,
 * columns ascending within a row, int64 row_ptr, int32 col, float32 val.
 * Bit-exact with the reference's matrix (as a set of entries) for the same
 * seed when sample == 0.  stats may be NULL.
 */
int lne_sparsify(lne_ctx* ctx, const lne_graph* g, const lne_sparsify_params* p, lne_csr** out,
                 lne_sparsify_stats* stats);

/*
 * Diagnostic: the double the trunc-log map takes the log of `adj` to
 * (log(adjusted_wgh) at LightNE/PathEmbed.h:211) for n host values, as the
 * sparsifier computes it on the device.  Used to check the exact-log path.
 */
int lne_trunc_log_values(lne_ctx* ctx, const double* x, int64_t n, double* out);

/*
 * SpMM: Y = alpha * A * X + beta * Y (mkl_sparse_s_mm, row-major,
 * non-transposed, as LightNE/mklredsvd/mklredsvd.cc:235-245).  X is n x d
 * with leading dimension ldx (device, FP32, BF16, FP16 or FP8 e4m3 per
 * x_prec; rows on 16-byte boundaries: ldx a multiple of 8, of 16 for FP8), Y is
 * n x d FP32 with ldy.
 * beta == 0 does not read Y.  Sums are formed in a fixed order: the result
 * is bitwise reproducible.  The first call on a matrix builds its work list.
 */
int lne_spmm(lne_ctx* ctx, const lne_csr* A, int x_prec, const void* X, int64_t ldx, int64_t d, float alpha,
             float beta, float* Y, int64_t ldy);

/* Parameters of the randomized SVD; names as the LightNE flags
 * (LightNE/LightNE.cc:34-50). */
typedef struct lne_randsvd_params {
  int64_t rank;                 /* -rank: sketch width r (oversampled) */
  int64_t dim;                  /* -dim: embedding dimension d <= r */
  int32_t normalize;            /* -normalize: L2-normalise embedding rows */
  int32_t precision;            /* LNE_PREC_FP32: every operand FP32.  LNE_PREC_BF16 and
                                   LNE_PREC_FP16: the sketch product A * Omega reads an FP8
                                   (e4m3) copy of Omega (exact: the sketch's values are
                                   e4m3-representable), and A * Q reads a BF16 copy of Q, or an
                                   FP16 copy of 2^12 * Q (|Q| <= 1); FP32 accumulation */
  uint64_t seed;                /* Gaussian sketch seed (the reference's VSL seed is 777) */
  int32_t random_project_only;  /* -random_project_only: return (A * Omega)[:, :dim] */
  int32_t sparse_project;       /* -sparse_project: Omega is the very sparse random projection
                                   (mklredsvd.cc:148-226) instead of the Gaussian sketch */
  double sparse_project_s;      /* -sparse_project_s: s of the projection (density 1/s, values
                                   +-sqrt(s)); below 1 means s = sqrt(n), as the reference */
} lne_randsvd_params;

typedef struct lne_randsvd_stats {
  float ms_sketch, ms_qr, ms_spmm2, ms_core, ms_total; /* device time per stage */
  int32_t jacobi_sweeps;        /* FP64 sweeps of the core SVD */
  int32_t kernel_launches;
  double spmm_nnz;
  int32_t jacobi_sweeps_fp32;   /* FP32 preconditioning sweeps before them (0: none) */
  int32_t reserved;
} lne_randsvd_stats;

/*
 * Randomized SVD of A (n x n CSR, general) and the embedding
 * emb = U[:, :dim] * sqrt(S[:dim]) (R1-R7).  d_emb: device n x dim FP32,
 * row-major.  h_S: host float[rank] singular values of the r x r core
 * (descending), may be NULL.  stats may be NULL.  Replaces
 * MKLRedSVD(...).run() + compute_u_sigma_root
 * (LightNE/mklredsvd/mklredsvd.cc:54-403, LightNE/PathEmbed.h:371-408).
 */
int lne_randsvd(lne_ctx* ctx, const lne_csr* A, const lne_randsvd_params* p, float* d_emb, float* h_S,
                lne_randsvd_stats* stats);

/*
 * The Gaussian sketch generator lne_randsvd uses: rows x cols N(0,1) values
 * of stream stream_id (0: Omega, 1: P) into device memory with leading
 * dimension ld.  Omega's values are rounded to FP8 (e4m3)-representable
 * floats, the other streams' to BF16-representable floats, so the FP32 and
 * BF16 forms share one sketch (the BF16 form gathers Omega from an FP8
 * copy).  Exposed so that a checker can rebuild the same sketches
 * (the reference's VSL SFMT19937 stream, mklredsvd.cc:141, has no
 * counterpart without MKL).
 */
int lne_gaussian(lne_ctx* ctx, uint64_t seed, uint64_t stream_id, int64_t rows, int64_t cols, float* d_out,
                 int64_t ld);

/*
 * -ne_method ne_zhang_et_al: the matrix NE_Zhang_et_al factorises
 * (LightNE/PathEmbed.h:410-448): the graph's structure (neighbours in file
 * order) with values (float)(log(1/d_i) - log(neg_v / sum neg)),
 * neg_v = (sum over neighbours u of v of 1/d_u)^0.75, in FP64.  The CSR is
 * passed to lne_randsvd with normalize = 1, as the reference does.
 */
int lne_ne_zhang_matrix(lne_ctx* ctx, const lne_graph* g, lne_csr** out);

/*
 * The very sparse random projection lne_randsvd uses with sparse_project
 * (mklredsvd.cc:148-226): n x rank, row i with Binomial(rank, 1/s)
 * nonzeros at distinct columns, values +-sqrt(s) (s as in
 * lne_randsvd_params.sparse_project_s), written densely into device memory
 * with leading dimension ld; *nnz_out (optional) receives its nonzero count.
 * The reference draws it from MKL's VSL stream and time(0); this generator
 * is counter-based, so a checker can rebuild the same sketch from the seed.
 */
int lne_sparse_projection(lne_ctx* ctx, uint64_t seed, int64_t n, int64_t rank, double s, float* d_out, int64_t ld,
                          int64_t* nnz_out);

/* Parameters of the spectral propagation (chebyshev_expansion). */
typedef struct lne_propagate_params {
  int64_t dim;        /* columns of the embedding (rank == dim in LightNE.cc:114) */
  int32_t order;      /* -order: number of Chebyshev terms K */
  int32_t precision;  /* LNE_PREC_FP32, LNE_PREC_BF16 or LNE_PREC_FP16: the type of the
                         vectors the SpMMs gather (FP32 accumulation and FP32 state in
                         every form; the FP16 form scales its input by a power of two so
                         that its largest |value| lies in [64, 128), and unscales the
                         outputs: an exact scaling) */
  double mu;          /* 0.2 in LightNE.cc:114 (narrowed to float, as the reference) */
  double s;           /* 0.5 in LightNE.cc:114 (Bessel argument, narrowed to float) */
} lne_propagate_params;

typedef struct lne_propagate_stats {
  float ms_total;
  int32_t kernel_launches;
  int32_t spmm_calls;
} lne_propagate_stats;

/*
 * Spectral propagation (P1, P2, P4): y = (A + I)(a - sum_k c_k T_k(X) a)
 * with X = M^2/2 - I, M = I - D~^-1 (A + I) - mu I, c_k the Bessel weights.
 * d_a (input) and d_y (output): device n x dim FP32, row-major; y must not
 * alias a.  d_a_out (optional, may be NULL) receives a - conv, the value the
 * reference leaves in its mutated argument.  Replaces
 * spectral_propagation::chebyshev_expansion up to the (A+I)a product
 * (LightNE/SpectralPropagation.h:45-221).
 */
int lne_propagate(lne_ctx* ctx, const lne_graph* g, const lne_propagate_params* p, const float* d_a, float* d_y,
                  float* d_a_out, lne_propagate_stats* stats);

/* The Chebyshev/Bessel weights c_0..c_{max(order,2)-1} as float, computed
 * in extended precision and narrowed as the reference's axpy calls do
 * (SpectralPropagation.h:129-197). */
int lne_chebyshev_coefficients(int32_t order, double s, float* out);

/*
 * Adjoint of lne_propagate (P3; no counterpart in the reference): for
 * y = (A + I)(a - sum_k c_k(s) T_k(X(mu)) a) and an output gradient g
 * (device n x dim), d_ga = dL/da (device n x dim, may be NULL), *h_dmu =
 * dL/dmu and *h_ds = dL/ds (host, may be NULL; they need d_a).  Uses
 * M^T = D~ M D~^-1, so dL/da = h - D~ sum_k c_k T_k(X) D~^-1 h with
 * h = (A + I) g; dL/ds = -sum_k c_k'(s) <h, T_k a>; dL/dmu from the forward
 * tangent T'_1 = -M a, T'_{k+1} = 2 X T'_k - T'_{k-1} - 2 M T_k.
 * The derivatives are of the real-valued map (mu, s not rounded to float).
 */
int lne_propagate_adjoint(lne_ctx* ctx, const lne_graph* g, const lne_propagate_params* p, const float* d_a,
                          const float* d_gy, float* d_ga, double* h_dmu, double* h_ds, lne_propagate_stats* stats);

/*
 * Dense embedding (P5): SVD of x (device n x dim FP32) and
 * emb = U * sqrt(S) with rows L2-normalised (norm > 1e-5), as
 * spectral_propagation::get_embedding_dense (LightNE/SpectralPropagation.h:16-43).
 * h_S (host float[dim]) may be NULL.
 */
int lne_dense_embed(lne_ctx* ctx, const float* d_x, int64_t n, int64_t dim, float* d_emb, float* h_S);

/*
 * SVD of a small dense matrix, the core step of the randomized SVD:
 * d_C (device r x r FP64, row-major, not modified) = U diag(S) V^T with
 * d_U (device r x r FP64, row-major, column j = left singular vector j) and
 * d_S (device r FP64), singular values descending; V is not formed, as
 * LAPACKE_gesvd(jobu 'S', jobvt 'N') at LightNE/mklredsvd/mklredsvd.cc:357-371
 * (which the reference runs in FP32).  One-sided Jacobi in FP64 (r <= 160:
 * FP32 sweeps first, then FP64 sweeps from the FP64-orthogonalised FP32
 * basis); r <= 1024.  h_sweeps (host int[2], may be NULL): FP64 sweeps,
 * FP32 sweeps.
 */
int lne_core_svd(lne_ctx* ctx, const double* d_C, int32_t r, double* d_U, double* d_S, int32_t* h_sweeps);

/*
 * Dense building blocks of the randomized SVD (device pointers, FP32 in):
 * G (c1 x c2, FP64 row-major) = A^T B for A (n x c1, lda) and B (n x c2, ldb)
 * [the Gram of CholeskyQR, mklredsvd.cc:262 via util.cc:40-79, and C = Z^T B,
 * mklredsvd.cc:330-345]; Out (n x c2, ldo) = In (n x k, ldi) W (k x c2
 * row-major) [the cblas_sgemm calls of mklredsvd.cc:297-312 and :382-397].
 * Up to 256 columns they run on the tcgen05 tensor core with split TF32
 * operands (FP32-level accuracy); columns c2..ldo-1 of Out are zeroed.
 */
int lne_gram(lne_ctx* ctx, const float* A, int64_t lda, int64_t c1, const float* B, int64_t ldb, int64_t c2,
             int64_t n, double* G);
int lne_gemm_tall(lne_ctx* ctx, const float* In, int64_t ldi, int64_t k, const float* W, int64_t c2, int64_t n,
                  float* Out, int64_t ldo);

/*
 * Allocation-free lne_gram, with no counterpart in the reference: for
 * callers that cannot allocate device memory when they need the product (a
 * process whose device memory belongs to another allocator or fixed arena,
 * or one under a hard memory cap).  The same product as lne_gram to FP32
 * accuracy (the row blocks may differ); its scratch is a 16 MiB file-scope
 * device array that every GPU loading the library holds until exit, so
 * ceil(max(n, 1) / 2048) * c1 * c2 must be at most 4,194,304 (else
 * LNE_ERR_UNSUPPORTED).  Up to 256 columns it runs on the tensor cores,
 * wider operands on the CUDA cores.  n = 0 writes zeros to G.  The first
 * call on a device looks up the array's device address, which (with CUDA's
 * lazy module loading) loads the array and commits its 16 MiB: make that
 * call, for example with n = 0, before a memory cap applies and before any
 * stream capture.  Calls share the array: calls that overlap on the GPU
 * race.  The caller's current device is restored on return.
 */
int lne_gram_noalloc(lne_ctx* ctx, const float* A, int64_t lda, int64_t c1, const float* B, int64_t ldb, int64_t c2,
                     int64_t n, double* G);

/* CSR accessors. */
int lne_csr_info(const lne_csr* c, int64_t* n, int64_t* nnz);
int lne_csr_download(lne_ctx* ctx, const lne_csr* c, int64_t* row_ptr, int32_t* col, float* val);
int lne_csr_device_ptrs(const lne_csr* c, const int64_t** row_ptr, const int32_t** col,
                        const float** val);
/* Wrap caller-owned device arrays as a CSR (not freed by lne_csr_free). */
int lne_csr_wrap_device(lne_ctx* ctx, int64_t n, int64_t nnz, const int64_t* d_row_ptr,
                        const int32_t* d_col, const float* d_val, lne_csr** out);
int lne_csr_free(lne_csr* c);

#ifdef __cplusplus
}
#endif
#endif /* LIGHTNE_GB300_H */
