/*
 * Declarations-only stand-in for <mkl.h>.  Test infrastructure: it lets the
 * reference's header-only sampler / par_table / trunc-log / CSR code
 * (LightNE/PathEmbed.h:81-369, LightNE/par_table.h) compile without Intel
 * MKL so that it can serve as the bit-exact checker of the sparsifier.
 *
 * Only types, enum constants and function declarations are provided.  No MKL
 * routine is defined: the sparsifier path never calls one, and the MKL
 * wrappers in LightNE/mklredsvd/mklhelper.h are inline members that are never
 * emitted, so nothing refers to these names at link time.  Any attempt to
 * call one fails to link, which is the intended behaviour.
 */
#pragma once
#include <cstddef>
#include <cstdint>

typedef long long MKL_INT;   /* MKL_ILP64 */
typedef long long lapack_int;
typedef void* VSLStreamStatePtr;

typedef enum { SPARSE_STATUS_SUCCESS = 0, SPARSE_STATUS_NOT_INITIALIZED = 1 } sparse_status_t;
typedef enum { SPARSE_INDEX_BASE_ZERO = 0, SPARSE_INDEX_BASE_ONE = 1 } sparse_index_base_t;
typedef enum { SPARSE_OPERATION_NON_TRANSPOSE = 10, SPARSE_OPERATION_TRANSPOSE = 11 } sparse_operation_t;
typedef enum { SPARSE_LAYOUT_ROW_MAJOR = 101, SPARSE_LAYOUT_COLUMN_MAJOR = 102 } sparse_layout_t;
typedef enum { SPARSE_MATRIX_TYPE_GENERAL = 20, SPARSE_MATRIX_TYPE_SYMMETRIC = 21 } sparse_matrix_type_t;
typedef enum { SPARSE_FILL_MODE_LOWER = 40, SPARSE_FILL_MODE_UPPER = 41 } sparse_fill_mode_t;
typedef enum { SPARSE_DIAG_NON_UNIT = 50, SPARSE_DIAG_UNIT = 51 } sparse_diag_type_t;
typedef enum { SPARSE_MEMORY_NONE = 80, SPARSE_MEMORY_AGGRESSIVE = 81 } sparse_memory_usage_t;
struct sparse_matrix;
typedef struct sparse_matrix* sparse_matrix_t;
struct matrix_descr {
  sparse_matrix_type_t type;
  sparse_fill_mode_t mode;
  sparse_diag_type_t diag;
};
typedef enum { CblasRowMajor = 101, CblasColMajor = 102 } CBLAS_LAYOUT;
typedef enum { CblasNoTrans = 111, CblasTrans = 112 } CBLAS_TRANSPOSE;
#define LAPACK_ROW_MAJOR 101
#define VSL_BRNG_SFMT19937 0
#define VSL_RNG_METHOD_GAUSSIAN_BOXMULLER 0
#define VSL_RNG_METHOD_GAUSSIAN_BOXMULLER2 1
#define VSL_RNG_METHOD_BINOMIAL_BTPE 0
#define VSL_STATUS_OK 0

/* Every MKL entry point the reference names, declared as an undefined
 * variadic template: any argument list type-checks, nothing is defined. */
#define LNE_SHIM_DECL(ret, name) template <class... A> ret name(A...);
LNE_SHIM_DECL(sparse_status_t, mkl_sparse_s_create_coo)
LNE_SHIM_DECL(sparse_status_t, mkl_sparse_d_create_coo)
LNE_SHIM_DECL(sparse_status_t, mkl_sparse_s_create_csr)
LNE_SHIM_DECL(sparse_status_t, mkl_sparse_d_create_csr)
LNE_SHIM_DECL(sparse_status_t, mkl_sparse_convert_csr)
LNE_SHIM_DECL(sparse_status_t, mkl_sparse_destroy)
LNE_SHIM_DECL(sparse_status_t, mkl_sparse_set_mm_hint)
LNE_SHIM_DECL(sparse_status_t, mkl_sparse_set_memory_hint)
LNE_SHIM_DECL(sparse_status_t, mkl_sparse_optimize)
LNE_SHIM_DECL(sparse_status_t, mkl_sparse_s_mm)
LNE_SHIM_DECL(sparse_status_t, mkl_sparse_d_mm)
LNE_SHIM_DECL(sparse_status_t, mkl_sparse_s_sp2md)
LNE_SHIM_DECL(sparse_status_t, mkl_sparse_d_sp2md)
LNE_SHIM_DECL(sparse_status_t, mkl_sparse_s_spmmd)
LNE_SHIM_DECL(sparse_status_t, mkl_sparse_d_spmmd)
LNE_SHIM_DECL(int, vsRngGaussian)
LNE_SHIM_DECL(int, vdRngGaussian)
LNE_SHIM_DECL(int, viRngBinomial)
LNE_SHIM_DECL(int, vslNewStream)
LNE_SHIM_DECL(int, vslDeleteStream)
LNE_SHIM_DECL(lapack_int, LAPACKE_sgeqrf)
LNE_SHIM_DECL(lapack_int, LAPACKE_dgeqrf)
LNE_SHIM_DECL(lapack_int, LAPACKE_sorgqr)
LNE_SHIM_DECL(lapack_int, LAPACKE_dorgqr)
LNE_SHIM_DECL(lapack_int, LAPACKE_sgesvd)
LNE_SHIM_DECL(lapack_int, LAPACKE_dgesvd)
LNE_SHIM_DECL(void, cblas_sgemm)
LNE_SHIM_DECL(void, cblas_dgemm)
LNE_SHIM_DECL(void, cblas_saxpy)
LNE_SHIM_DECL(void, cblas_daxpy)
LNE_SHIM_DECL(void, cblas_scopy)
LNE_SHIM_DECL(void, cblas_dcopy)
LNE_SHIM_DECL(float, cblas_snrm2)
LNE_SHIM_DECL(double, cblas_dnrm2)
LNE_SHIM_DECL(void, cblas_sscal)
LNE_SHIM_DECL(void, cblas_dscal)
LNE_SHIM_DECL(void*, mkl_calloc)
LNE_SHIM_DECL(void*, mkl_malloc)
LNE_SHIM_DECL(void, mkl_free)
#undef LNE_SHIM_DECL
