/*
 * MKL-API shim for building the LPM-C reference sources without Intel MKL.
 *
 * TEST INFRASTRUCTURE ONLY: this header and mkl_shim.c exist so that the
 * reference sources (src/, all C files) compile and link here, to serve as the oracle for
 * the GPU library.  Nothing in the product library includes or links it.
 *
 * Every declaration follows the public MKL / CBLAS / LAPACKE / RCI ISS /
 * Inspector-executor sparse BLAS interface that the reference calls
 * (call sites: src/solver.c:49-79,195-253, src/constitutive.c:1213,1227,
 * src/lpm_basic.c:19,41,212, src/stiffness.c:164-389, src/boundary.c:88,176,
 * src/initialization.c:289-823).  Semantics are written from the published
 * API contracts; no MKL code or headers were used.  It is not MKL: CG
 * iterates are not bit-equal to MKL's dcg, only its documented stopping
 * test is honoured.
 */
#ifndef LPM_MKL_SHIM_H
#define LPM_MKL_SHIM_H

#ifdef __cplusplus
extern "C" {
#endif

typedef int MKL_INT;

/* ---- CBLAS ---------------------------------------------------------- */
typedef enum { CblasRowMajor = 101, CblasColMajor = 102 } CBLAS_LAYOUT;
typedef enum { CblasNoTrans = 111, CblasTrans = 112, CblasConjTrans = 113 } CBLAS_TRANSPOSE;

double cblas_dnrm2(const MKL_INT n, const double *x, const MKL_INT incx);
void cblas_dgemv(const CBLAS_LAYOUT layout, const CBLAS_TRANSPOSE trans,
                 const MKL_INT m, const MKL_INT n, const double alpha,
                 const double *a, const MKL_INT lda, const double *x,
                 const MKL_INT incx, const double beta, double *y,
                 const MKL_INT incy);
void cblas_dgemm(const CBLAS_LAYOUT layout, const CBLAS_TRANSPOSE transa,
                 const CBLAS_TRANSPOSE transb, const MKL_INT m, const MKL_INT n,
                 const MKL_INT k, const double alpha, const double *a,
                 const MKL_INT lda, const double *b, const MKL_INT ldb,
                 const double beta, double *c, const MKL_INT ldc);

/* ---- LAPACKE -------------------------------------------------------- */
#define LAPACK_ROW_MAJOR 101
#define LAPACK_COL_MAJOR 102
MKL_INT LAPACKE_dgesv(int matrix_layout, MKL_INT n, MKL_INT nrhs, double *a,
                      MKL_INT lda, MKL_INT *ipiv, double *b, MKL_INT ldb);

/* ---- RCI conjugate gradient (dcg_*) --------------------------------- */
void dcg_init(const MKL_INT *n, const double *x, const double *b,
              MKL_INT *rci_request, MKL_INT *ipar, double *dpar, double *tmp);
void dcg_check(const MKL_INT *n, const double *x, const double *b,
               MKL_INT *rci_request, MKL_INT *ipar, double *dpar, double *tmp);
void dcg(const MKL_INT *n, double *x, double *b, MKL_INT *rci_request,
         MKL_INT *ipar, double *dpar, double *tmp);
void dcg_get(const MKL_INT *n, const double *x, const double *b,
             const MKL_INT *rci_request, const MKL_INT *ipar,
             const double *dpar, const double *tmp, MKL_INT *itercount);

/* ---- Inspector-executor sparse BLAS (CSR, double) ------------------- */
typedef enum {
    SPARSE_STATUS_SUCCESS = 0,
    SPARSE_STATUS_NOT_INITIALIZED = 1,
    SPARSE_STATUS_ALLOC_FAILED = 2,
    SPARSE_STATUS_INVALID_VALUE = 3,
    SPARSE_STATUS_EXECUTION_FAILED = 4,
    SPARSE_STATUS_INTERNAL_ERROR = 5,
    SPARSE_STATUS_NOT_SUPPORTED = 6
} sparse_status_t;
typedef enum { SPARSE_OPERATION_NON_TRANSPOSE = 10, SPARSE_OPERATION_TRANSPOSE = 11,
               SPARSE_OPERATION_CONJUGATE_TRANSPOSE = 12 } sparse_operation_t;
typedef enum { SPARSE_MATRIX_TYPE_GENERAL = 20, SPARSE_MATRIX_TYPE_SYMMETRIC = 21,
               SPARSE_MATRIX_TYPE_HERMITIAN = 22, SPARSE_MATRIX_TYPE_TRIANGULAR = 23,
               SPARSE_MATRIX_TYPE_DIAGONAL = 24 } sparse_matrix_type_t;
typedef enum { SPARSE_FILL_MODE_LOWER = 40, SPARSE_FILL_MODE_UPPER = 41,
               SPARSE_FILL_MODE_FULL = 42 } sparse_fill_mode_t;
typedef enum { SPARSE_DIAG_NON_UNIT = 50, SPARSE_DIAG_UNIT = 51 } sparse_diag_type_t;
typedef enum { SPARSE_INDEX_BASE_ZERO = 0, SPARSE_INDEX_BASE_ONE = 1 } sparse_index_base_t;

struct matrix_descr {
    sparse_matrix_type_t type;
    sparse_fill_mode_t mode;
    sparse_diag_type_t diag;
};
struct lpm_shim_csr;
typedef struct lpm_shim_csr *sparse_matrix_t;

sparse_status_t mkl_sparse_d_create_csr(sparse_matrix_t *A, const sparse_index_base_t indexing,
                                        const MKL_INT rows, const MKL_INT cols,
                                        MKL_INT *rows_start, MKL_INT *rows_end,
                                        MKL_INT *col_indx, double *values);
sparse_status_t mkl_sparse_d_mv(const sparse_operation_t operation, const double alpha,
                                const sparse_matrix_t A, const struct matrix_descr descr,
                                const double *x, const double beta, double *y);
sparse_status_t mkl_sparse_destroy(sparse_matrix_t A);

/* ---- PARDISO / service ---------------------------------------------- */
void PARDISO(void *pt, const MKL_INT *maxfct, const MKL_INT *mnum, const MKL_INT *mtype,
             const MKL_INT *phase, const MKL_INT *n, const void *a, const MKL_INT *ia,
             const MKL_INT *ja, MKL_INT *perm, const MKL_INT *nrhs, MKL_INT *iparm,
             const MKL_INT *msglvl, void *b, void *x, MKL_INT *error);
void mkl_free_buffers(void);

/* Oracle knob: CG tolerance overrides applied in dcg_check (squared norms).
 * rtol_sq <= 0 keeps the caller's dpar[0]; atol_sq < 0 keeps dpar[1].
 * Used only by the oracle driver: the reference hard-codes 1e-8/1e-12
 * (src/solver.c:221-222). */
void lpm_shim_set_cg_tol(double rtol_sq, double atol_sq);
/* Number of dcg iterations of the last completed solve (oracle reporting). */
int lpm_shim_last_cg_iters(void);

#ifdef __cplusplus
}
#endif

#endif
