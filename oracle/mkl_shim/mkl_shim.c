/*
 * MKL-API shim: implementations of the 12 MKL entry points the LPM-C
 * reference links against (cblas_dnrm2/dgemv/dgemm, LAPACKE_dgesv,
 * dcg_init/dcg_check/dcg/dcg_get, mkl_sparse_d_create_csr/mv, PARDISO,
 * mkl_free_buffers).
 *
 * TEST INFRASTRUCTURE ONLY: linked into oracle/_ref (the reference built
 * from its own sources) and into the oracle restatement.  Written from the
 * public API contracts; arithmetic is plain, serial and deterministic.
 */
#include <stdio.h>
#include <stdlib.h>
#include <math.h>
#include "mkl.h"
#include "../cg_rci.h"

/* Euclidean norm: plain sum of squares, then sqrt (deterministic order). */
double cblas_dnrm2(const MKL_INT n, const double *x, const MKL_INT incx)
{
    double s = 0.0;
    for (MKL_INT i = 0; i < n; i++)
        s += x[(size_t)i * incx] * x[(size_t)i * incx];
    return sqrt(s);
}

/* y = alpha*op(A)*x + beta*y; beta == 0 means y is not read. */
void cblas_dgemv(const CBLAS_LAYOUT layout, const CBLAS_TRANSPOSE trans,
                 const MKL_INT m, const MKL_INT n, const double alpha,
                 const double *a, const MKL_INT lda, const double *x,
                 const MKL_INT incx, const double beta, double *y,
                 const MKL_INT incy)
{
    int t = (trans != CblasNoTrans);
    int rowmajor = (layout == CblasRowMajor);
    MKL_INT ny = t ? n : m, nx = t ? m : n;
    for (MKL_INT i = 0; i < ny; i++) {
        double s = 0.0;
        for (MKL_INT j = 0; j < nx; j++) {
            /* element op(A)[i][j] */
            MKL_INT r = t ? j : i, c = t ? i : j;
            double aij = rowmajor ? a[(size_t)r * lda + c] : a[(size_t)c * lda + r];
            s += aij * x[(size_t)j * incx];
        }
        double v = alpha * s;
        if (beta != 0.0)
            v += beta * y[(size_t)i * incy];
        y[(size_t)i * incy] = v;
    }
}

/* C = alpha*op(A)*op(B) + beta*C; beta == 0 means C is not read. */
void cblas_dgemm(const CBLAS_LAYOUT layout, const CBLAS_TRANSPOSE transa,
                 const CBLAS_TRANSPOSE transb, const MKL_INT m, const MKL_INT n,
                 const MKL_INT k, const double alpha, const double *a,
                 const MKL_INT lda, const double *b, const MKL_INT ldb,
                 const double beta, double *c, const MKL_INT ldc)
{
    int ta = (transa != CblasNoTrans), tb = (transb != CblasNoTrans);
    int rm = (layout == CblasRowMajor);
    for (MKL_INT i = 0; i < m; i++) {
        for (MKL_INT j = 0; j < n; j++) {
            double s = 0.0;
            for (MKL_INT l = 0; l < k; l++) {
                MKL_INT ar = ta ? l : i, ac = ta ? i : l;
                MKL_INT br = tb ? j : l, bc = tb ? l : j;
                double av = rm ? a[(size_t)ar * lda + ac] : a[(size_t)ac * lda + ar];
                double bv = rm ? b[(size_t)br * ldb + bc] : b[(size_t)bc * ldb + br];
                s += av * bv;
            }
            size_t ci = rm ? (size_t)i * ldc + j : (size_t)j * ldc + i;
            double v = alpha * s;
            if (beta != 0.0)
                v += beta * c[ci];
            c[ci] = v;
        }
    }
}

/*
 * Solve A X = B by LU with partial pivoting (first maximal |pivot| wins).
 * Returns 0, or i > 0 when U(i,i) is exactly zero (then X is not computed),
 * or -1 for a bad argument.
 */
MKL_INT LAPACKE_dgesv(int matrix_layout, MKL_INT n, MKL_INT nrhs, double *a,
                      MKL_INT lda, MKL_INT *ipiv, double *b, MKL_INT ldb)
{
    if (n < 0 || nrhs < 0)
        return -1;
    int rm = (matrix_layout == LAPACK_ROW_MAJOR);
#define A_(r, c) (*(rm ? &a[(size_t)(r) * lda + (c)] : &a[(size_t)(c) * lda + (r)]))
#define B_(r, c) (*(rm ? &b[(size_t)(r) * ldb + (c)] : &b[(size_t)(c) * ldb + (r)]))
    MKL_INT info = 0;
    for (MKL_INT k = 0; k < n; k++) {
        MKL_INT piv = k;
        double best = fabs(A_(k, k));
        for (MKL_INT i = k + 1; i < n; i++) {
            double v = fabs(A_(i, k));
            if (v > best) {
                best = v;
                piv = i;
            }
        }
        ipiv[k] = piv + 1;
        if (A_(piv, k) == 0.0) {
            if (info == 0)
                info = k + 1;
            continue;
        }
        if (piv != k) {
            for (MKL_INT c = 0; c < n; c++) {
                double t = A_(k, c);
                A_(k, c) = A_(piv, c);
                A_(piv, c) = t;
            }
        }
        double d = A_(k, k);
        for (MKL_INT i = k + 1; i < n; i++) {
            double l = A_(i, k) / d;
            A_(i, k) = l;
            if (l != 0.0)
                for (MKL_INT c = k + 1; c < n; c++)
                    A_(i, c) -= l * A_(k, c);
        }
    }
    if (info != 0)
        return info;
    for (MKL_INT r = 0; r < nrhs; r++) {
        for (MKL_INT k = 0; k < n; k++) {
            MKL_INT p = ipiv[k] - 1;
            if (p != k) {
                double t = B_(k, r);
                B_(k, r) = B_(p, r);
                B_(p, r) = t;
            }
        }
        for (MKL_INT i = 1; i < n; i++) {
            double s = B_(i, r);
            for (MKL_INT c = 0; c < i; c++)
                s -= A_(i, c) * B_(c, r);
            B_(i, r) = s;
        }
        for (MKL_INT i = n - 1; i >= 0; i--) {
            double s = B_(i, r);
            for (MKL_INT c = i + 1; c < n; c++)
                s -= A_(i, c) * B_(c, r);
            B_(i, r) = s / A_(i, i);
        }
    }
#undef A_
#undef B_
    return 0;
}

/* ---- RCI CG ----------------------------------------------------------- */
static double g_rtol_override = -1.0, g_atol_override = -1.0;
static int g_last_iters = 0;

void lpm_shim_set_cg_tol(double rtol_sq, double atol_sq)
{
    g_rtol_override = rtol_sq;
    g_atol_override = atol_sq;
}
int lpm_shim_last_cg_iters(void) { return g_last_iters; }

void dcg_init(const MKL_INT *n, const double *x, const double *b,
              MKL_INT *rci_request, MKL_INT *ipar, double *dpar, double *tmp)
{
    (void)x; (void)b; (void)tmp;
    lpm_rci_init(*n, rci_request, ipar, dpar);
}

void dcg_check(const MKL_INT *n, const double *x, const double *b,
               MKL_INT *rci_request, MKL_INT *ipar, double *dpar, double *tmp)
{
    (void)x; (void)b; (void)tmp;
    if (g_rtol_override > 0.0)
        dpar[0] = g_rtol_override;
    if (g_atol_override >= 0.0)
        dpar[1] = g_atol_override;
    lpm_rci_check(*n, rci_request, ipar, dpar);
}

void dcg(const MKL_INT *n, double *x, double *b, MKL_INT *rci_request,
         MKL_INT *ipar, double *dpar, double *tmp)
{
    lpm_rci_step(*n, x, b, rci_request, ipar, dpar, tmp);
    if (*rci_request <= 0)
        g_last_iters = ipar[3];
}

void dcg_get(const MKL_INT *n, const double *x, const double *b,
             const MKL_INT *rci_request, const MKL_INT *ipar,
             const double *dpar, const double *tmp, MKL_INT *itercount)
{
    (void)n; (void)x; (void)b; (void)rci_request; (void)dpar; (void)tmp;
    *itercount = ipar[3];
}

/* ---- sparse CSR ----------------------------------------------------- */
struct lpm_shim_csr {
    int base, rows, cols;
    MKL_INT *rs, *re, *ci;
    double *v;
};

sparse_status_t mkl_sparse_d_create_csr(sparse_matrix_t *A, const sparse_index_base_t indexing,
                                        const MKL_INT rows, const MKL_INT cols,
                                        MKL_INT *rows_start, MKL_INT *rows_end,
                                        MKL_INT *col_indx, double *values)
{
    struct lpm_shim_csr *m = (struct lpm_shim_csr *)malloc(sizeof(*m));
    if (!m)
        return SPARSE_STATUS_ALLOC_FAILED;
    m->base = (indexing == SPARSE_INDEX_BASE_ONE) ? 1 : 0;
    m->rows = rows;
    m->cols = cols;
    m->rs = rows_start;
    m->re = rows_end;
    m->ci = col_indx;
    m->v = values;
    *A = m;
    return SPARSE_STATUS_SUCCESS;
}

sparse_status_t mkl_sparse_destroy(sparse_matrix_t A)
{
    free(A);
    return SPARSE_STATUS_SUCCESS;
}

/*
 * y = alpha*op(A)*x + beta*y.  For SPARSE_MATRIX_TYPE_SYMMETRIC only the
 * triangle named by descr.mode is used (diagonal included) and mirrored.
 */
sparse_status_t mkl_sparse_d_mv(const sparse_operation_t operation, const double alpha,
                                const sparse_matrix_t A, const struct matrix_descr descr,
                                const double *x, const double beta, double *y)
{
    const struct lpm_shim_csr *m = A;
    int nr = m->rows;
    double *acc = (double *)calloc((size_t)(nr > m->cols ? nr : m->cols), sizeof(double));
    if (!acc)
        return SPARSE_STATUS_ALLOC_FAILED;
    int sym = (descr.type == SPARSE_MATRIX_TYPE_SYMMETRIC);
    int upper = (descr.mode == SPARSE_FILL_MODE_UPPER);
    for (int i = 0; i < nr; i++) {
        for (MKL_INT k = m->rs[i] - m->base; k < m->re[i] - m->base; k++) {
            int j = m->ci[k] - m->base;
            double a = m->v[k];
            if (sym) {
                if (upper ? (j < i) : (j > i))
                    continue;
                acc[i] += a * x[j];
                if (j != i)
                    acc[j] += a * x[i];
            } else if (operation == SPARSE_OPERATION_NON_TRANSPOSE) {
                acc[i] += a * x[j];
            } else {
                acc[j] += a * x[i];
            }
        }
    }
    int ny = (!sym && operation != SPARSE_OPERATION_NON_TRANSPOSE) ? m->cols : nr;
    for (int i = 0; i < ny; i++) {
        double v = alpha * acc[i];
        if (beta != 0.0)
            v += beta * y[i];
        y[i] = v;
    }
    free(acc);
    return SPARSE_STATUS_SUCCESS;
}

/* ---- PARDISO / service ------------------------------------------------ */
void PARDISO(void *pt, const MKL_INT *maxfct, const MKL_INT *mnum, const MKL_INT *mtype,
             const MKL_INT *phase, const MKL_INT *n, const void *a, const MKL_INT *ia,
             const MKL_INT *ja, MKL_INT *perm, const MKL_INT *nrhs, MKL_INT *iparm,
             const MKL_INT *msglvl, void *b, void *x, MKL_INT *error)
{
    (void)pt; (void)maxfct; (void)mnum; (void)mtype; (void)phase; (void)n; (void)a;
    (void)ia; (void)ja; (void)perm; (void)nrhs; (void)iparm; (void)msglvl; (void)b; (void)x;
    /* The direct solver is not part of this shim; report "not supported". */
    *error = -99;
}

void mkl_free_buffers(void) {}
