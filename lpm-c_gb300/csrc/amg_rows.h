// Per-row arithmetic of the multigrid V-cycle kernels (k_amg.cu), shared
// with a host emulation of the same launch sequence (tests/amg_harness.cpp),
// so that the index arithmetic of every kernel is exercised on the CPU.
// Level-0 vectors hold 4 values per particle (x, y, z, unused), coarse-level
// vectors 6 per aggregate.  The device instantiates everything with FP32
// vectors, values and arithmetic (T = float): the V-cycle is the PCG's
// preconditioner, FP32 costs it nothing in iterations, and FP64 arithmetic
// is ALU-bound on GB300 (measured: the FP64 products of the prolongation,
// restriction and coarse operators kept the FP64 pipe 77-86 % busy at 11-34 %
// of the DRAM bandwidth).  The host emulation also runs them with T = double.
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

#ifdef __CUDACC__
// four FP16 values (the smoother's stiffness copy), one 8-byte load; as float
__device__ __forceinline__ void load4(const __half *p, float (&v)[4])
{
    const uint2 t = __ldcs(reinterpret_cast<const uint2 *>(p));
    const float2 a = __half22float2(*reinterpret_cast<const __half2 *>(&t.x));
    const float2 b = __half22float2(*reinterpret_cast<const __half2 *>(&t.y));
    v[0] = a.x;
    v[1] = a.y;
    v[2] = b.x;
    v[3] = b.y;
}
#endif

// x, y, z of a level-0 vector entry (4 values per particle): one 16-byte
// load for FP32 on the device
template <typename T>
AMG_HD void load_xyz(const float *p, T &a, T &b, T &c)
{
#ifdef __CUDA_ARCH__
    const float4 t = __ldg(reinterpret_cast<const float4 *>(p));
    a = (T)t.x;
    b = (T)t.y;
    c = (T)t.z;
#else
    a = (T)p[0];
    b = (T)p[1];
    c = (T)p[2];
#endif
}
template <typename T>
AMG_HD void load_xyz(const double *p, T &a, T &b, T &c)
{
    a = (T)p[0];
    b = (T)p[1];
    c = (T)p[2];
}

// one level-0 entry (x, y, z, 0): a single 16-byte store for FP32 on the
// device; an FP64 output gets the rounded FP32 values
template <typename T>
AMG_HD void store_xyz(float *p, T a, T b, T c)
{
#ifdef __CUDA_ARCH__
    *reinterpret_cast<float4 *>(p) = make_float4((float)a, (float)b, (float)c, 0.f);
#else
    p[0] = (float)a;
    p[1] = (float)b;
    p[2] = (float)c;
    p[3] = 0.f;
#endif
}
template <typename T>
AMG_HD void store_xyz(double *p, T a, T b, T c)
{
    p[0] = (double)a;
    p[1] = (double)b;
    p[2] = (double)c;
    p[3] = 0.0;
}

// Level 0: partial product of block row `row` of the stiffness (device
// layout: npad[row] blocks at rowoff[row], npad a multiple of 4,
// component-major values of type V) over the groups of 4 consecutive blocks
// b0 = 4 sub, 4 (sub + nl), ...; products in A (the device stores the
// smoother's stiffness in FP16, scaled, and multiplies in FP32).
template <typename V, typename X, typename A = V>
AMG_HD void k0_row_partial(const long long *rowoff, const int *npad, const int *cols, const V *val,
                           const X *x, int row, int sub, int nl, A &y0, A &y1, A &y2)
{
    const long long off = rowoff[row];
    const int np = npad[row];
    const V *vr = val + 9 * off;
    for (int b0 = 4 * sub; b0 < np; b0 += 4 * nl) {
        A v[9][4];
        for (int k = 0; k < 9; k++)
            load4(vr + (size_t)k * np + b0, v[k]);
        for (int j = 0; j < 4; j++) {
            A x0, x1, x2;
            load_xyz<A>(x + 4 * (size_t)cols[off + b0 + j], x0, x1, x2);
            y0 += v[0][j] * x0 + v[1][j] * x1 + v[2][j] * x2;
            y1 += v[3][j] * x0 + v[4][j] * x1 + v[5][j] * x2;
            y2 += v[6][j] * x0 + v[7][j] * x1 + v[8][j] * x2;
        }
    }
}

// d = P^-1 r with the 3x3 block inverses stored [9][n]
template <typename T, typename PT>
AMG_HD void pinv_apply(const PT *P, int n, int i, const T (&r)[3], T (&d)[3])
{
    for (int a = 0; a < 3; a++)
        d[a] = (T)P[(size_t)(3 * a) * n + i] * r[0] + (T)P[(size_t)(3 * a + 1) * n + i] * r[1] +
               (T)P[(size_t)(3 * a + 2) * n + i] * r[2];
}

// d = P r with the row's 3x3 block inverse in registers (row-major)
template <typename T>
AMG_HD void pinv_apply9(const T (&P)[9], const T (&r)[3], T (&d)[3])
{
    for (int a = 0; a < 3; a++)
        d[a] = P[3 * a] * r[0] + P[3 * a + 1] * r[1] + P[3 * a + 2] * r[2];
}

// Level-0 epilogue of row `row` given K x (y) and the row's block inverse P:
// SM_RESID out = mask(b - y); SM_SMOOTH out = mask(x + omega P mask(b - y)).
template <typename T, typename O>
AMG_HD void k0_epilogue(int mode, int row, uint8_t m, const T (&P)[9], T omega, const T *x, const T *b, O *out,
                        T y0, T y1, T y2)
{
    T b0, b1, b2;
    load_xyz<T>(b + 4 * (size_t)row, b0, b1, b2);
    T r[3] = {(m & 1) ? b0 - y0 : T(0), (m & 2) ? b1 - y1 : T(0), (m & 4) ? b2 - y2 : T(0)};
    O *o = out + 4 * (size_t)row;
    if (mode == SM_RESID) {
        store_xyz<T>(o, r[0], r[1], r[2]);
    } else {
        T d[3];
        pinv_apply9<T>(P, r, d);
        T x0, x1, x2;
        load_xyz<T>(x + 4 * (size_t)row, x0, x1, x2);
        store_xyz<T>(o, (m & 1) ? x0 + omega * d[0] : T(0), (m & 2) ? x1 + omega * d[1] : T(0),
                     (m & 4) ? x2 + omega * d[2] : T(0));
    }
}

// Level 0, first sweep from zero: out = mask(omega Pinv mask(b)), and the
// right-hand side in the iteration's precision (bt = b)
template <typename T, typename PT, typename B>
AMG_HD void jacobi0_row(int n, int i, uint8_t m, const PT *Pinv, T omega, const B *b, T *bt, T *out)
{
    T b0, b1, b2;
    load_xyz<T>(b + 4 * (size_t)i, b0, b1, b2);
    const T r[3] = {(m & 1) ? b0 : T(0), (m & 2) ? b1 : T(0), (m & 4) ? b2 : T(0)};
    store_xyz<T>(bt + 4 * (size_t)i, r[0], r[1], r[2]);
    T d[3];
    pinv_apply<T, PT>(Pinv, n, i, r, d);
    store_xyz<T>(out + 4 * (size_t)i, (m & 1) ? omega * d[0] : T(0), (m & 2) ? omega * d[1] : T(0),
                 (m & 4) ? omega * d[2] : T(0));
}

// One R x C block (N = R C values, row-major) into registers: on the device
// FP32 blocks of 36 values (144 B, 16-byte aligned) load as nine float4, of
// 18 values (72 B, 8-byte aligned) as nine float2; streaming loads.
template <int N, typename T>
AMG_HD void load_block(const T *p, T (&b)[N])
{
#ifdef __CUDA_ARCH__
    if constexpr (sizeof(T) == 4 && N % 4 == 0) {
        for (int q = 0; q < N / 4; q++) {
            const float4 v = __ldcs(reinterpret_cast<const float4 *>(p) + q);
            b[4 * q] = v.x;
            b[4 * q + 1] = v.y;
            b[4 * q + 2] = v.z;
            b[4 * q + 3] = v.w;
        }
        return;
    } else if constexpr (sizeof(T) == 4 && N % 2 == 0) {
        for (int q = 0; q < N / 2; q++) {
            const float2 v = __ldcs(reinterpret_cast<const float2 *>(p) + q);
            b[2 * q] = v.x;
            b[2 * q + 1] = v.y;
        }
        return;
    }
#endif
    for (int q = 0; q < N; q++)
        b[q] = p[q];
}

#ifdef __CUDACC__
// FP16 blocks (the device's prolongation, restriction and coarse operators)
// as float: 36 values (72 B, 8-byte aligned) as nine 8-byte loads, 18 values
// (36 B, 4-byte aligned) as nine half2
template <int N>
__device__ __forceinline__ void load_block(const __half *p, float (&b)[N])
{
    if constexpr (N % 4 == 0) {
        for (int q = 0; q < N / 4; q++) {
            const uint2 t = __ldcs(reinterpret_cast<const uint2 *>(p) + q);
            const float2 u = __half22float2(*reinterpret_cast<const __half2 *>(&t.x));
            const float2 w = __half22float2(*reinterpret_cast<const __half2 *>(&t.y));
            b[4 * q] = u.x;
            b[4 * q + 1] = u.y;
            b[4 * q + 2] = w.x;
            b[4 * q + 3] = w.y;
        }
    } else {
        for (int q = 0; q < N / 2; q++) {
            const unsigned t = __ldcs(reinterpret_cast<const unsigned *>(p) + q);
            const float2 u = __half22float2(*reinterpret_cast<const __half2 *>(&t));
            b[2 * q] = u.x;
            b[2 * q + 1] = u.y;
        }
    }
}
#endif

// C consecutive vector entries starting at p (p 8-byte aligned: SX and C
// even); float2 loads of FP32 on the device
template <int C, typename T>
AMG_HD void load_entries(const T *p, T (&v)[C])
{
#ifdef __CUDA_ARCH__
    if constexpr (sizeof(T) == 4 && C % 2 == 0) {
        for (int q = 0; q < C / 2; q++) {
            const float2 t = __ldg(reinterpret_cast<const float2 *>(p) + q);
            v[2 * q] = t.x;
            v[2 * q + 1] = t.y;
        }
        return;
    }
#endif
    for (int c = 0; c < C; c++)
        v[c] = p[c];
}

// Block-CSR level: partial y of block row `row` (R x C row-major blocks of
// V; block column j of x at x[j * SX]) over the blocks ptr[row] + sub,
// + nl, ...; products and sums in T (the device stores FP16 blocks, scaled,
// and multiplies in FP32; the caller applies the scale to the row sums)
template <int R, int C, typename T, typename V = T>
AMG_HD void bsr_row_partial(const long long *ptr, const int *col, const V *val, const T *x, int SX, int row,
                            int sub, int nl, T (&y)[R])
{
    for (long long k = ptr[row] + sub; k < ptr[row + 1]; k += nl) {
        T blk[R * C];
        load_block<R * C>(val + (size_t)k * (R * C), blk);
        T xv[C];
        load_entries<C, T>(x + (size_t)col[k] * SX, xv);
        for (int r = 0; r < R; r++)
            for (int c = 0; c < C; c++)
                y[r] += blk[r * C + c] * xv[c];
    }
}

// BM_SET: out[row * SY + r] = y_r; BM_ADD: += y_r; BM_SMOOTH (R = C = 6):
// out = x_row + omega Dinv (b - y); BM_RESID: out = b - y.
template <int R, int MODE, typename T>
AMG_HD void bsr_epilogue(int row, const T (&y)[R], const T *x, int SX, T *out, int SY, const T *b, const T *dinv,
                         T omega)
{
    T *o = out + (size_t)row * SY;
    if (MODE == BM_SET) {
        for (int r = 0; r < R; r++)
            o[r] = y[r];
    } else if (MODE == BM_ADD) {
        for (int r = 0; r < R; r++)
            o[r] += y[r];
    } else {
        T rr[R];
        for (int r = 0; r < R; r++)
            rr[r] = b[(size_t)row * R + r] - y[r];
        if (MODE == BM_RESID) {
            for (int r = 0; r < R; r++)
                o[r] = rr[r];
        } else {
            const T *D = dinv + (size_t)row * (R * R);
            const T *xr = x + (size_t)row * SX;
            for (int r = 0; r < R; r++) {
                T s = 0;
                for (int c = 0; c < R; c++)
                    s += D[r * R + c] * rr[c];
                o[r] = xr[r] + omega * s;
            }
        }
    }
}

// 6-DOF level, first sweep from zero: out = omega Dinv b
template <typename T>
AMG_HD void jacobi6_row(int i, const T *dinv, T omega, const T *b, T *out)
{
    const T *D = dinv + (size_t)i * 36;
    for (int r = 0; r < 6; r++) {
        T s = 0;
        for (int c = 0; c < 6; c++)
            s += D[r * 6 + c] * b[(size_t)i * 6 + c];
        out[(size_t)i * 6 + r] = omega * s;
    }
}

// Coarsest level, entry k of Cinv b over the columns j = sub, sub + nl, ...
// (entry j of a vector at (j / B) * S + j % B); FP64 sums
template <typename T>
AMG_HD double dense_row_partial(int nc, const double *Cinv, const T *b, int B, int S, int k, int sub, int nl)
{
    const double *row = Cinv + (size_t)k * nc;
    double s = 0.0;
    for (int j = sub; j < nc; j += nl)
        s += row[j] * (double)b[(size_t)(j / B) * S + j % B];
    return s;
}

}  // namespace lpm
