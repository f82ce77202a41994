// Per-row arithmetic of the multigrid V-cycle kernels (k_amg.cu), shared
// with a host emulation of the same launch sequence (tests/amg_harness.cpp),
// so that the index arithmetic of every kernel is exercised on the CPU.
// Vectors are plain double arrays: level-0 vectors hold 4 doubles per
// particle (x, y, z, unused), coarse-level vectors 6 per aggregate.
#pragma once
#include <cstddef>
#include <cstdint>

#ifdef __CUDACC__
#define AMG_HD __host__ __device__ __forceinline__
#else
#define AMG_HD inline
#endif

namespace lpm {

enum { SM_SMOOTH = 0, SM_RESID = 1 };
enum { BM_SET = 0, BM_ADD = 1, BM_SMOOTH = 2, BM_RESID = 3 };

// Four consecutive values of one stiffness component (16-byte aligned for
// FP32, 32-byte for FP64: rows start at multiples of 4 blocks and hold a
// multiple of 4), one vector load on the device.
AMG_HD void load4(const float *p, float (&v)[4])
{
#ifdef __CUDA_ARCH__
    const float4 t = __ldcs(reinterpret_cast<const float4 *>(p));
    v[0] = t.x;
    v[1] = t.y;
    v[2] = t.z;
    v[3] = t.w;
#else
    for (int j = 0; j < 4; j++)
        v[j] = p[j];
#endif
}
AMG_HD void load4(const double *p, double (&v)[4])
{
#ifdef __CUDA_ARCH__
    const double2 a = __ldcs(reinterpret_cast<const double2 *>(p));
    const double2 b = __ldcs(reinterpret_cast<const double2 *>(p) + 1);
    v[0] = a.x;
    v[1] = a.y;
    v[2] = b.x;
    v[3] = b.y;
#else
    for (int j = 0; j < 4; j++)
        v[j] = p[j];
#endif
}

// Level 0: partial product of block row `row` of the stiffness (device
// layout: npad[row] blocks at rowoff[row], npad a multiple of 4,
// component-major values) over the groups of 4 consecutive blocks
// b0 = 4 sub, 4 (sub + nl), ...; products in V.
template <typename V>
AMG_HD void k0_row_partial(const long long *rowoff, const int *npad, const int *cols, const V *val,
                           const double *x, int row, int sub, int nl, V &y0, V &y1, V &y2)
{
    const long long off = rowoff[row];
    const int np = npad[row];
    const V *vr = val + 9 * off;
    for (int b0 = 4 * sub; b0 < np; b0 += 4 * nl) {
        V v[9][4];
        for (int k = 0; k < 9; k++)
            load4(vr + (size_t)k * np + b0, v[k]);
        for (int j = 0; j < 4; j++) {
            const double *xv = x + 4 * (size_t)cols[off + b0 + j];
            const V x0 = (V)xv[0], x1 = (V)xv[1], x2 = (V)xv[2];
            y0 += v[0][j] * x0 + v[1][j] * x1 + v[2][j] * x2;
            y1 += v[3][j] * x0 + v[4][j] * x1 + v[5][j] * x2;
            y2 += v[6][j] * x0 + v[7][j] * x1 + v[8][j] * x2;
        }
    }
}

// d = P^-1 r with the 3x3 block inverses stored [9][n]
AMG_HD void pinv_apply(const double *P, int n, int i, const double (&r)[3], double (&d)[3])
{
    for (int a = 0; a < 3; a++)
        d[a] = P[(size_t)(3 * a) * n + i] * r[0] + P[(size_t)(3 * a + 1) * n + i] * r[1] +
               P[(size_t)(3 * a + 2) * n + i] * r[2];
}

// Level-0 epilogue of row `row` given K x (y): SM_RESID out = mask(b - y);
// SM_SMOOTH out = mask(x + omega Pinv mask(b - y)).
AMG_HD void k0_epilogue(int mode, int n, int row, uint8_t m, const double *Pinv, double omega, const double *x,
                        const double *b, double *out, double y0, double y1, double y2)
{
    const double *bb = b + 4 * (size_t)row;
    double r[3] = {(m & 1) ? bb[0] - y0 : 0.0, (m & 2) ? bb[1] - y1 : 0.0, (m & 4) ? bb[2] - y2 : 0.0};
    double *o = out + 4 * (size_t)row;
    if (mode == SM_RESID) {
        o[0] = r[0];
        o[1] = r[1];
        o[2] = r[2];
    } else {
        double d[3];
        pinv_apply(Pinv, n, row, r, d);
        const double *xr = x + 4 * (size_t)row;
        o[0] = (m & 1) ? xr[0] + omega * d[0] : 0.0;
        o[1] = (m & 2) ? xr[1] + omega * d[1] : 0.0;
        o[2] = (m & 4) ? xr[2] + omega * d[2] : 0.0;
    }
    o[3] = 0.0;
}

// Level 0, first sweep from zero: out = mask(omega Pinv mask(b))
AMG_HD void jacobi0_row(int n, int i, uint8_t m, const double *Pinv, double omega, const double *b, double *out)
{
    const double *bb = b + 4 * (size_t)i;
    const double r[3] = {(m & 1) ? bb[0] : 0.0, (m & 2) ? bb[1] : 0.0, (m & 4) ? bb[2] : 0.0};
    double d[3];
    pinv_apply(Pinv, n, i, r, d);
    double *o = out + 4 * (size_t)i;
    o[0] = (m & 1) ? omega * d[0] : 0.0;
    o[1] = (m & 2) ? omega * d[1] : 0.0;
    o[2] = (m & 4) ? omega * d[2] : 0.0;
    o[3] = 0.0;
}

// Block-CSR level: partial y of block row `row` (R x C row-major blocks of
// VT, FP64 for the coarse operators, FP32 for the prolongation and
// restriction; block column j of x at x[j * SX]) over the blocks
// ptr[row] + sub, + nl, ...; products and sums in FP64.
template <int R, int C, typename VT>
AMG_HD void bsr_row_partial(const long long *ptr, const int *col, const VT *val, const double *x, int SX,
                            int row, int sub, int nl, double (&y)[R])
{
    for (long long k = ptr[row] + sub; k < ptr[row + 1]; k += nl) {
        const VT *blk = val + (size_t)k * (R * C);
        const double *xc = x + (size_t)col[k] * SX;
        double xv[C];
        for (int c = 0; c < C; c++)
            xv[c] = xc[c];
        for (int r = 0; r < R; r++)
            for (int c = 0; c < C; c++)
                y[r] += (double)blk[r * C + c] * xv[c];
    }
}

// BM_SET: out[row * SY + r] = y_r; BM_ADD: += y_r; BM_SMOOTH (R = C = 6):
// out = x_row + omega Dinv (b - y); BM_RESID: out = b - y.
template <int R, int MODE>
AMG_HD void bsr_epilogue(int row, const double (&y)[R], const double *x, int SX, double *out, int SY, const double *b,
                         const double *dinv, double omega)
{
    double *o = out + (size_t)row * SY;
    if (MODE == BM_SET) {
        for (int r = 0; r < R; r++)
            o[r] = y[r];
    } else if (MODE == BM_ADD) {
        for (int r = 0; r < R; r++)
            o[r] += y[r];
    } else {
        double rr[R];
        for (int r = 0; r < R; r++)
            rr[r] = b[(size_t)row * R + r] - y[r];
        if (MODE == BM_RESID) {
            for (int r = 0; r < R; r++)
                o[r] = rr[r];
        } else {
            const double *D = dinv + (size_t)row * (R * R);
            const double *xr = x + (size_t)row * SX;
            for (int r = 0; r < R; r++) {
                double s = 0.0;
                for (int c = 0; c < R; c++)
                    s += D[r * R + c] * rr[c];
                o[r] = xr[r] + omega * s;
            }
        }
    }
}

// 6-DOF level, first sweep from zero: out = omega Dinv b
AMG_HD void jacobi6_row(int i, const double *dinv, double omega, const double *b, double *out)
{
    const double *D = dinv + (size_t)i * 36;
    for (int r = 0; r < 6; r++) {
        double s = 0.0;
        for (int c = 0; c < 6; c++)
            s += D[r * 6 + c] * b[(size_t)i * 6 + c];
        out[(size_t)i * 6 + r] = omega * s;
    }
}

// Coarsest level, entry k of Cinv b over the columns j = sub, sub + nl, ...
// (entry j of a vector at (j / B) * S + j % B)
AMG_HD double dense_row_partial(int nc, const double *Cinv, const double *b, int B, int S, int k, int sub, int nl)
{
    const double *row = Cinv + (size_t)k * nc;
    double s = 0.0;
    for (int j = sub; j < nc; j += nl)
        s += row[j] * b[(size_t)(j / B) * S + j % B];
    return s;
}

}  // namespace lpm
