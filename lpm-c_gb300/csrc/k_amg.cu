// Smoothed-aggregation multigrid V-cycle as the preconditioner of the PCG
// that replaces the reference's CG (src/solver.c:188-270), and the PCG steps
// around it.  The hierarchy is built on the host (amg_setup.cpp) and kept on
// the device (AmgDev).
//
// V-cycle on level l (operator A_l, block-Jacobi inverse D_l^-1, damping
// omega_l = 4/3 / rho(D_l^-1 A_l)), nu = opts.amg_sweeps:
//     x = omega D^-1 b                      (first sweep, from zero)
//     nu - 1 sweeps x += omega D^-1 (b - A x)
//     b_{l+1} = P_l^T (b - A x)             (residual, restriction)
//     e = V-cycle_{l+1}(b_{l+1})            (dense inverse on the coarsest level)
//     x += P_l e                            (prolongation)
//     nu sweeps x += omega D^-1 (b - A x)
// The same number of Jacobi sweeps before and after makes the cycle a
// symmetric positive definite operator, as CG needs.  On level 0 the
// operator is the stiffness in FP32 (Kf: the assembled one under mixed
// precision, a copy of the FP64 Kd otherwise; the PCG product keeps Kd),
// with FP32 products as in the mixed SpMV; b is the CG residual r, x the
// scratch vector q (free between the update and the next product) and y the
// preconditioned residual z; the DOF mask zeroes the constrained DOFs of
// every level-0 output.
//
// PCG iteration: q = K p (with p.q and alpha, k_spmv), x += alpha p and
// r -= alpha q (k_amg_update, |r|^2 and the convergence test), z = V(r),
// r.z and beta (k_amg_rz), p = z + beta p (k_cg_p in k_solve.cu).  Every
// kernel returns at once when the solve is marked done, so a CUDA graph of a
// whole chunk of iterations stays valid after convergence.  Reductions are
// deterministic (per-block partials, summed in a fixed order by the last
// block).
#include <algorithm>
#include <chrono>
#include <cmath>
#include <omp.h>
#include <cuda_fp16.h>
#include "amg.h"
#include "amg_rows.h"
#include "lpm_internal.h"
#include "stream_pipe.h"

namespace lpm {

constexpr int ATPB = 256;

__device__ __forceinline__ double amg_warp_sum(double s)
{
    for (int o = 16; o > 0; o >>= 1)
        s += __shfl_xor_sync(0xffffffffu, s, o);
    return s;
}

// Block partials of NV values, the last block sums them in block order and
// calls fin(totals) on its thread 0.  Every thread of the grid calls it.
template <int NV, typename Fin>
__device__ void amg_reduce(double (&v)[NV], double *partials, unsigned *counter, Fin fin)
{
    __shared__ double red[NV][ATPB / 32];
    __shared__ bool last;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < NV; k++) {
        const double s = amg_warp_sum(v[k]);
        if (lane == 0)
            red[k][wid] = s;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < NV; k++) {
            double s = 0.0;
            for (int w = 0; w < ATPB / 32; w++)
                s += red[k][w];
            partials[(size_t)k * gridDim.x + blockIdx.x] = s;
        }
        __threadfence();
        last = (atomicAdd(counter, 1u) == gridDim.x - 1);
    }
    __syncthreads();
    if (!last)
        return;
    __threadfence();
#pragma unroll
    for (int k = 0; k < NV; k++) {
        double s = 0.0;
        for (unsigned b = threadIdx.x; b < gridDim.x; b += ATPB)
            s += __ldcg(&partials[(size_t)k * gridDim.x + b]);
        s = amg_warp_sum(s);
        if (lane == 0)
            red[k][wid] = s;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double tot[NV];
#pragma unroll
        for (int k = 0; k < NV; k++) {
            double s = 0.0;
            for (int w = 0; w < ATPB / 32; w++)
                s += red[k][w];
            tot[k] = s;
        }
        fin(tot);
        *counter = 0u;
    }
}

__device__ __forceinline__ dvec4 amg_mask(dvec4 v, uint8_t m)
{
    return make_dvec4((m & 1) ? v.x : 0.0, (m & 2) ? v.y : 0.0, (m & 4) ? v.z : 0.0, 0.0);
}

struct AmgVec {
    int n;
    const uint8_t *mask;
    double *partials;
    unsigned *counter;
    CgScalars *sc;
};

// ---- PCG steps ------------------------------------------------------------------

// x = 0, r = mask(b) * scale, |r|^2, tolerance, counters
__global__ void __launch_bounds__(ATPB) k_amg_init(AmgVec a, const dvec4 *b, double scale, dvec4 *x, dvec4 *r,
                                                   double rtol, int maxit, double delta2)
{
    double v[1] = {0.0};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.n; i += gridDim.x * blockDim.x) {
        dvec4 bb = amg_mask(b[i], a.mask[i]);
        bb.x *= scale;
        bb.y *= scale;
        bb.z *= scale;
        x[i] = make_dvec4(0.0, 0.0, 0.0, 0.0);
        r[i] = bb;
        v[0] += bb.x * bb.x + bb.y * bb.y + bb.z * bb.z;
    }
    CgScalars *sc = a.sc;
    amg_reduce<1>(v, a.partials, a.counter, [sc, rtol, maxit, delta2](const double *t) {
        sc->rz = 0.0;
        sc->rz_old = 0.0;
        sc->rr = t[0];
        sc->rr_max = t[0];
        sc->bnorm2 = t[0];
        sc->tol2 = rtol * rtol * t[0];
        sc->upd_delta2 = delta2;
        sc->it = 0;
        sc->maxit = maxit;
        sc->done = (t[0] <= sc->tol2 || !(t[0] == t[0])) ? 1 : 0;
        sc->alpha = 0.0;
        sc->beta = 0.0;
        sc->upd_req = 0;
    });
}

// x += alpha p, r -= alpha q, |r|^2 and the convergence test
__global__ void __launch_bounds__(ATPB) k_amg_update(AmgVec a, dvec4 *x, dvec4 *r, const dvec4 *p,
                                                     const dvec4 *q)
{
    CgScalars *sc = a.sc;
    if (sc->done)
        return;
    const double al = sc->alpha;
    double v[1] = {0.0};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.n; i += gridDim.x * blockDim.x) {
        dvec4 xv = x[i], rv = r[i];
        const dvec4 pv = p[i], qv = q[i];
        xv.x += al * pv.x;
        xv.y += al * pv.y;
        xv.z += al * pv.z;
        rv.x -= al * qv.x;
        rv.y -= al * qv.y;
        rv.z -= al * qv.z;
        x[i] = xv;
        r[i] = rv;
        v[0] += rv.x * rv.x + rv.y * rv.y + rv.z * rv.z;
    }
    amg_reduce<1>(v, a.partials, a.counter, [sc](const double *t) {
        sc->rr = t[0];
        sc->it += 1;
        if (t[0] <= sc->tol2)
            sc->done = 1;
        else if (!(t[0] == t[0]))
            sc->done = 3;
        else if (sc->it >= sc->maxit)
            sc->done = 2;
        else if (t[0] < sc->upd_delta2 * sc->rr_max)
            sc->upd_req = 1;  // raised as done = 4 once p is updated (k_cg_p)
        if (t[0] > sc->rr_max)
            sc->rr_max = t[0];
    });
}

// Reliable update: r = mask(rtrue) (the FP64 true residual in the units of
// the iteration), |r|^2; the search direction is kept.
__global__ void __launch_bounds__(ATPB) k_amg_reliable(AmgVec a, const dvec4 *rtrue, dvec4 *r)
{
    double v[1] = {0.0};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.n; i += gridDim.x * blockDim.x) {
        const dvec4 rv = amg_mask(rtrue[i], a.mask[i]);
        r[i] = rv;
        v[0] += rv.x * rv.x + rv.y * rv.y + rv.z * rv.z;
    }
    CgScalars *sc = a.sc;
    amg_reduce<1>(v, a.partials, a.counter, [sc](const double *t) {
        sc->rr = t[0];
        sc->rr_max = t[0];
        sc->done = !(t[0] == t[0]) ? 3 : 0;
        sc->upd_req = 0;
    });
}

enum { RZ_INIT = 0, RZ_ITER = 1, RZ_RELIABLE = 2 };

// r.z after the V-cycle: INIT also sets p = z (and its two FP32 parts when
// split is given); ITER sets beta
template <int MODE>
__global__ void __launch_bounds__(ATPB) k_amg_rz(AmgVec a, const dvec4 *r, const dvec4 *z, dvec4 *p,
                                                 float4 *split = nullptr)
{
    CgScalars *sc = a.sc;
    if (sc->done)
        return;
    double v[1] = {0.0};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.n; i += gridDim.x * blockDim.x) {
        const dvec4 rv = r[i], zv = z[i];
        if (MODE == RZ_INIT) {
            p[i] = zv;
            if (split) {
                const float hx = __double2float_rn(zv.x), hy = __double2float_rn(zv.y),
                            hz = __double2float_rn(zv.z);
                split[2 * (size_t)i] = make_float4(hx, hy, hz, 0.f);
                split[2 * (size_t)i + 1] =
                    make_float4(__double2float_rn(zv.x - (double)hx), __double2float_rn(zv.y - (double)hy),
                                __double2float_rn(zv.z - (double)hz), 0.f);
            }
        }
        v[0] += rv.x * zv.x + rv.y * zv.y + rv.z * zv.z;
    }
    amg_reduce<1>(v, a.partials, a.counter, [sc](const double *t) {
        if (MODE == RZ_INIT) {
            sc->rz = t[0];
            sc->rz_old = t[0];
        } else if (MODE == RZ_ITER) {
            sc->rz_old = sc->rz;
            sc->rz = t[0];
            sc->beta = (sc->rz_old != 0.0) ? t[0] / sc->rz_old : 0.0;
        } else {
            sc->rz = t[0];
        }
    });
}

// ---- level 0: the stiffness ---------------------------------------------------


// MODE SM_SMOOTH: out = x + omega Pinv mask(b - K x); SM_RESID: out = mask(b - K x).
// Half a warp per block row, lanes over the row's blocks (padding included:
// zero values, column of the row itself).  The stiffness is the FP16 copy
// Kh = Kf / s (s in *kscale): products and sums in FP32, the row sums
// multiplied by s.  FP32 vectors and arithmetic otherwise (amg_rows.h).  O:
// float (an iterate of the cycle) or double (its last sweep, the PCG's z).
// The smoother's operator is only the preconditioner's: rounded to FP16 (or
// even to 8 significand bits) it leaves the PCG iteration counts of the numpy
// checks unchanged.
template <int MODE, typename O, int L0_LANES = 16>
__global__ void __launch_bounds__(ATPB) k_amg_k0(int n, const long long *__restrict__ rowoff,
                                                 const int *__restrict__ npad, const int *__restrict__ cols,
                                                 const uint8_t *__restrict__ mask, const __half *__restrict__ val,
                                                 const float *__restrict__ kscale, const float *__restrict__ Prow,
                                                 float omega, const float *__restrict__ x,
                                                 const float *__restrict__ b, O *__restrict__ out,
                                                 const CgScalars *sc)
{
    if (sc && sc->done)
        return;
    const float s = *kscale;
    const int sub = threadIdx.x & (L0_LANES - 1);
    const unsigned gmask = ((1u << L0_LANES) - 1u) << ((threadIdx.x & 31) & ~(L0_LANES - 1));
    const int g = (blockIdx.x * blockDim.x + threadIdx.x) / L0_LANES;
    const int ng = (gridDim.x * blockDim.x) / L0_LANES;
    for (int row = g; row < n; row += ng) {
        float y0 = 0.f, y1 = 0.f, y2 = 0.f;
        k0_row_partial<__half, float, float>(rowoff, npad, cols, val, x, row, sub, L0_LANES, y0, y1, y2);
#pragma unroll
        for (int o = L0_LANES / 2; o > 0; o >>= 1) {
            y0 += __shfl_xor_sync(gmask, y0, o);
            y1 += __shfl_xor_sync(gmask, y1, o);
            y2 += __shfl_xor_sync(gmask, y2, o);
        }
        // the row's block inverse ([n][9], 36 contiguous bytes): one value per
        // lane, then to lane 0
        float P[9];
        if constexpr (L0_LANES >= 9) {
            const float pv = sub < 9 ? Prow[(size_t)row * 9 + sub] : 0.f;
#pragma unroll
            for (int k = 0; k < 9; k++)
                P[k] = __shfl_sync(gmask, pv, k, L0_LANES);
        } else {
#pragma unroll
            for (int k = 0; k < 9; k++)
                P[k] = Prow[(size_t)row * 9 + k];
        }
        if (sub == 0)
            k0_epilogue<float, O>(MODE, row, mask[row], P, omega, x, b, out, s * y0, s * y1, s * y2);
    }
}

// k_amg_k0 (16 lanes per block row, the same arithmetic per row) with the
// FP16 stiffness streamed through a ring of shared-memory stages by the
// bulk-copy engine (stream_pipe.h).  A tile's FP16 values start 8 bytes off a
// 16-byte boundary for half of the tiles (18 bytes per block, rows start at
// multiples of 4 blocks): the copy starts at the boundary below and ends at
// the one above (the value array is padded by 16 bytes), and the rows index
// from the offset.  The row's own entries (block inverse, mask, b, x) are
// loaded ahead of the stage wait.
// ROWS rows per tile, a half-warp per row: 16 (256 threads) or 8 (128
// threads, six CTAs per SM)
template <int MODE, typename O, int ROWS>
__global__ void __launch_bounds__(ROWS * 16, ROWS == 16 ? 1 : 6)
    k_amg_k0_stream(int n, const long long *__restrict__ rowoff, const int *__restrict__ cols,
                    const uint8_t *__restrict__ mask, const __half *__restrict__ val, const float *__restrict__ kscale,
                    const float *__restrict__ Prow, float omega, const float *__restrict__ x,
                    const float *__restrict__ b, O *__restrict__ out, const CgScalars *sc, StreamLayout lay,
                    int *status)
{
    constexpr int NT = ROWS * 16;
    constexpr unsigned RO_BYTES = (ROWS + 2) * 8;
    extern __shared__ __align__(128) unsigned char stage_mem[];
    __shared__ unsigned long long full[STREAM_MAX_STAGES], empty[STREAM_MAX_STAGES];
    __shared__ volatile int abort_k;
    if (sc && sc->done)
        return;
    const float s = *kscale;
    const int S = lay.stages;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int sub = lane & 15, rl = 2 * wid + (lane >> 4);
    const unsigned gmask = 0xffffu << (lane & 16);
    const int ntiles = (n + ROWS - 1) / ROWS;
    const int mine = (int)blockIdx.x < ntiles ? (ntiles - 1 - (int)blockIdx.x) / (int)gridDim.x + 1 : 0;
    if (threadIdx.x == 0) {
        for (int k = 0; k < S; k++) {
            mbar_init(&full[k], 1);
            mbar_init(&empty[k], NT / 32);
        }
        abort_k = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    auto first_row = [&](int i) { return ((int)blockIdx.x + i * (int)gridDim.x) * ROWS; };
    auto fail = [&]() {
        atomicOr(status, LPM_STATUS_DEVICE_WAIT);
        abort_k = 1;
    };
    int issued = 0, jb = -32;
    long long pb0 = 0, pb1 = 0;
    auto issue_next = [&]() -> bool {  // warp 0, warp-uniform
        const int j = issued, st_i = j % S;
        if (j - jb >= 32) {
            jb += 32;
            if (jb + lane < mine) {
                const int r0 = first_row(jb + lane);
                pb0 = rowoff[r0];
                pb1 = rowoff[min(r0 + ROWS, n)];
            }
        }
        const long long b0 = __shfl_sync(0xffffffffu, pb0, j - jb);
        const long long b1 = __shfl_sync(0xffffffffu, pb1, j - jb);
        if (j >= S && !warp_mbar_wait(&empty[st_i], (unsigned)((j / S) - 1) & 1u))
            return false;
        if (lane == 0) {
            unsigned char *st = stage_mem + (size_t)st_i * lay.stage_bytes;
            const unsigned nb = (unsigned)(b1 - b0);
            const long long v0 = (18 * b0) & ~15LL, v1 = (18 * b1 + 15) & ~15LL;
            const unsigned vb = nb ? (unsigned)(v1 - v0) : 0u;
            mbar_expect_tx(&full[st_i], RO_BYTES + 4u * nb + vb);
            bulk_g2s(st, rowoff + first_row(j), RO_BYTES, &full[st_i]);
            if (nb) {
                bulk_g2s(st + lay.cols_off, cols + b0, 4u * nb, &full[st_i]);
                bulk_g2s(st + lay.vals_off, reinterpret_cast<const unsigned char *>(val) + v0, vb, &full[st_i]);
            }
        }
        __syncwarp();
        issued++;
        return true;
    };
    if (wid == 0) {
        while (issued < mine && issued < S - 1)
            issue_next();
    }
    int i = 0;
    for (; i < mine; i++) {
        if (__any_sync(0xffffffffu, abort_k != 0))
            break;
        if (wid == 0 && issued < mine && !issue_next()) {
            fail();
            break;
        }
        const int st_i = i % S;
        const int row = first_row(i) + rl;
        float pv = 0.f;
        uint8_t m = 0;
        float4 bq = make_float4(0.f, 0.f, 0.f, 0.f), xq = bq;
        if (row < n) {
            if (sub < 9)
                pv = Prow[(size_t)row * 9 + sub];
            if (sub == 0) {
                m = mask[row];
                bq = __ldg(reinterpret_cast<const float4 *>(b) + row);
                if (MODE == SM_SMOOTH)
                    xq = __ldg(reinterpret_cast<const float4 *>(x) + row);
            }
        }
        if (!warp_mbar_wait(&full[st_i], (unsigned)(i / S) & 1u)) {
            fail();
            break;
        }
        if (row < n) {
            const unsigned char *st = stage_mem + (size_t)st_i * lay.stage_bytes;
            const long long *ro = reinterpret_cast<const long long *>(st);
            const int o = (int)(ro[rl] - ro[0]), np = (int)(ro[rl + 1] - ro[rl]);
            const int *cs = reinterpret_cast<const int *>(st + lay.cols_off) + o;
            const __half *vr = reinterpret_cast<const __half *>(st + lay.vals_off + ((18 * ro[0]) & 15)) +
                               9 * (size_t)o;
            float y0 = 0.f, y1 = 0.f, y2 = 0.f;
            for (int b0 = 4 * sub; b0 < np; b0 += 64) {
                const int4 c4 = *reinterpret_cast<const int4 *>(cs + b0);
                const int cc[4] = {c4.x, c4.y, c4.z, c4.w};
                float v[9][4];
#pragma unroll
                for (int k = 0; k < 9; k++) {
                    const uint2 t = *reinterpret_cast<const uint2 *>(vr + (size_t)k * np + b0);
                    const float2 lo = __half22float2(*reinterpret_cast<const __half2 *>(&t.x));
                    const float2 hi = __half22float2(*reinterpret_cast<const __half2 *>(&t.y));
                    v[k][0] = lo.x;
                    v[k][1] = lo.y;
                    v[k][2] = hi.x;
                    v[k][3] = hi.y;
                }
#pragma unroll
                for (int j = 0; j < 4; j++) {
                    float x0, x1, x2;
                    load_xyz<float>(x + 4 * (size_t)cc[j], x0, x1, x2);
                    y0 += v[0][j] * x0 + v[1][j] * x1 + v[2][j] * x2;
                    y1 += v[3][j] * x0 + v[4][j] * x1 + v[5][j] * x2;
                    y2 += v[6][j] * x0 + v[7][j] * x1 + v[8][j] * x2;
                }
            }
#pragma unroll
            for (int off = 8; off > 0; off >>= 1) {
                y0 += __shfl_xor_sync(gmask, y0, off);
                y1 += __shfl_xor_sync(gmask, y1, off);
                y2 += __shfl_xor_sync(gmask, y2, off);
            }
            float P[9];
#pragma unroll
            for (int k = 0; k < 9; k++)
                P[k] = __shfl_sync(gmask, pv, k, 16);
            if (sub == 0) {
                y0 *= s;
                y1 *= s;
                y2 *= s;
                const float r[3] = {(m & 1) ? bq.x - y0 : 0.f, (m & 2) ? bq.y - y1 : 0.f,
                                    (m & 4) ? bq.z - y2 : 0.f};
                O *po = out + 4 * (size_t)row;
                if (MODE == SM_RESID) {
                    store_xyz<float>(po, r[0], r[1], r[2]);
                } else {
                    float d[3];
                    pinv_apply9<float>(P, r, d);
                    store_xyz<float>(po, (m & 1) ? xq.x + omega * d[0] : 0.f, (m & 2) ? xq.y + omega * d[1] : 0.f,
                                     (m & 4) ? xq.z + omega * d[2] : 0.f);
                }
            }
        }
        __syncwarp();
        if (lane == 0)
            mbar_arrive(&empty[st_i]);
    }
    if (wid == 0) {
        for (int k = i; k < issued; k++)
            if (!warp_mbar_wait(&full[k % S], (unsigned)(k / S) & 1u))
                break;
    }
}

// out = omega Pinv mask(b): the first sweep from zero on level 0; bt = the
// right-hand side (the PCG residual, FP64) in FP32 for the later sweeps
__global__ void __launch_bounds__(ATPB) k_amg_jacobi0(int n, const uint8_t *__restrict__ mask,
                                                      const float *__restrict__ Pinv, float omega,
                                                      const double *__restrict__ b, float *__restrict__ bt,
                                                      float *__restrict__ out, const CgScalars *sc)
{
    if (sc && sc->done)
        return;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        jacobi0_row<float, float, double>(n, i, mask[i], Pinv, omega, b, bt, out);
}

// ---- block-CSR levels -------------------------------------------------------------

constexpr int BL_LANES = 8;  // lanes per block row of the coarse-level kernels

// R x C blocks, 8 lanes per block row, epilogue by MODE (amg_rows.h):
// restriction (BM_SET), prolongation (BM_ADD), coarse smoothing (BM_SMOOTH)
// and residual (BM_RESID).  Blocks in FP16 times vscale (1 for the
// prolongation and restriction, whose weights lie well inside FP16's range;
// max |A| / 2^14 for the coarse operators), FP32 vectors and arithmetic.
template <int R, int C, int MODE>
__global__ void __launch_bounds__(ATPB) k_amg_bsr(int nbr, const long long *__restrict__ ptr,
                                                  const int *__restrict__ col, const __half *__restrict__ val,
                                                  float vscale, const float *__restrict__ x, int SX,
                                                  float *__restrict__ out, int SY, const float *__restrict__ b,
                                                  const float *__restrict__ dinv, float omega,
                                                  const CgScalars *sc)
{
    static_assert(MODE == BM_SET || MODE == BM_ADD || (R == 6 && C == 6), "operator rows are 6 x 6");
    if (sc && sc->done)
        return;
    const int sub = threadIdx.x & (BL_LANES - 1);
    const unsigned gmask = 0xffu << ((threadIdx.x & 31) & ~(BL_LANES - 1));
    const int g = (blockIdx.x * blockDim.x + threadIdx.x) / BL_LANES;
    const int ng = (gridDim.x * blockDim.x) / BL_LANES;
    for (int row = g; row < nbr; row += ng) {
        float y[R];
#pragma unroll
        for (int r = 0; r < R; r++)
            y[r] = 0.f;
        bsr_row_partial<R, C, float, __half>(ptr, col, val, x, SX, row, sub, BL_LANES, y);
#pragma unroll
        for (int o = BL_LANES / 2; o > 0; o >>= 1)
#pragma unroll
            for (int r = 0; r < R; r++)
                y[r] += __shfl_xor_sync(gmask, y[r], o);
        if (sub == 0) {
#pragma unroll
            for (int r = 0; r < R; r++)
                y[r] *= vscale;
            bsr_epilogue<R, MODE, float>(row, y, x, SX, out, SY, b, dinv, omega);
        }
    }
}

// out = omega Dinv b on a 6-DOF level: the first sweep from zero
__global__ void __launch_bounds__(ATPB) k_amg_jacobi6(int nb, const float *__restrict__ dinv, float omega,
                                                      const float *__restrict__ b, float *__restrict__ out,
                                                      const CgScalars *sc)
{
    if (sc && sc->done)
        return;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nb; i += gridDim.x * blockDim.x)
        jacobi6_row<float>(i, dinv, omega, b, out);
}

// Coarsest level: out = Cinv b (dense, nc x nc, FP64 sums), one warp per
// output entry.  Entry k of a vector lives at (k / B) * S + k % B (B DOFs per
// block row, stride S: 6/6 above level 0, 3/4 when level 0 is the coarsest).
template <typename BT, typename OT>
__global__ void __launch_bounds__(ATPB) k_amg_dense(int nc, const double *__restrict__ Cinv,
                                                    const BT *__restrict__ b, OT *__restrict__ out, int B, int S,
                                                    const CgScalars *sc)
{
    if (sc && sc->done)
        return;
    const int lane = threadIdx.x & 31;
    const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    for (int k = w; k < nc; k += nw) {
        const double s = amg_warp_sum(dense_row_partial<BT>(nc, Cinv, b, B, S, k, lane, 32));
        if (lane == 0)
            out[(size_t)(k / B) * S + k % B] = (OT)s;
    }
}

// ---- launchers ----------------------------------------------------------------------

static int grid_for(const Ctx &c, long long rows_x_threads)
{
    const long long blocks = (rows_x_threads + ATPB - 1) / ATPB;
    const long long cap = (long long)(c.tune.sms > 0 ? c.tune.sms : 152) * 16;
    return (int)std::max(1LL, std::min(blocks, cap));
}

static AmgVec amg_vec(Ctx &c) { return AmgVec{c.n, c.mask, c.partials, c.counter, c.sc}; }

template <int MODE, typename O, int L>
static void k0_launch_l(Ctx &c, float omega, const float *x, const float *b, O *out, const CgScalars *sc)
{
    const int g = grid_for(c, (long long)c.n * L);
    k_amg_k0<MODE, O, L><<<g, ATPB, 0, c.stream>>>(c.n, c.rowoff, c.npad, c.cols, c.mask,
                                                   reinterpret_cast<const __half *>(c.Kh), c.kh_scale, c.Pinv_rf,
                                                   omega, x, b, out, sc);
}

// Stage layouts of the streamed smoother's variants for rows of at most
// max_npad blocks (FP16 values: 18 bytes per block plus 16 for the aligned
// copy): tiles of 16 rows with one or two CTAs per SM, tiles of 8 rows with
// six; 0 stages where fewer than two fit.  Also lifts the kernels' dynamic
// shared-memory limit.
template <int ROWS>
static void stream_smoother_limit(int bytes)
{
    cudaFuncSetAttribute(k_amg_k0_stream<SM_SMOOTH, float, ROWS>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    cudaFuncSetAttribute(k_amg_k0_stream<SM_SMOOTH, double, ROWS>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         bytes);
    cudaFuncSetAttribute(k_amg_k0_stream<SM_RESID, float, ROWS>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    cudaFuncSetAttribute(k_amg_k0_stream<SM_RESID, double, ROWS>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
}

void init_stream_smoother(Ctx &c, int max_npad)
{
    auto up = [](int v, int a) { return (v + a - 1) / a * a; };
    int optin = 0, per_sm = 0;
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, c.device);
    cudaDeviceGetAttribute(&per_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, c.device);
    const int rows[3] = {16, 16, 8}, ctas[3] = {1, 2, 6};
    for (int k = 0; k < 3; k++) {
        c.smooth_cols_off[k] = up((rows[k] + 2) * 8, 128);
        c.smooth_vals_off[k] = c.smooth_cols_off[k] + up(rows[k] * max_npad * 4, 128);
        c.smooth_stage_bytes[k] = c.smooth_vals_off[k] + up(rows[k] * max_npad * 18 + 16, 128);
        const int avail = std::min(optin, per_sm / ctas[k]) - 2048;
        const int st = avail > 0 ? std::min(STREAM_MAX_STAGES, avail / c.smooth_stage_bytes[k]) : 0;
        c.smooth_stages[k] = st >= 2 ? st : 0;
    }
    // one limit per kernel instantiation: the largest of the variants using it
    int max16 = 0, max8 = 0;
    for (int k = 0; k < 3; k++) {
        const int bytes = c.smooth_stages[k] * c.smooth_stage_bytes[k];
        int &m = rows[k] == 16 ? max16 : max8;
        m = std::max(m, bytes);
    }
    if (max16 > 0)
        stream_smoother_limit<16>(max16);
    if (max8 > 0)
        stream_smoother_limit<8>(max8);
    cudaGetLastError();
}

// level-0 pass with the autotuner's shape: streamed (tune.smooth_stream) or
// register-fed with tune.smooth_variant's lanes per block row
template <int MODE, typename O>
static void k0_launch_m(Ctx &c, float omega, const float *x, const float *b, O *out, const CgScalars *sc)
{
    const int ss = c.tune.smooth_stream;
    if (ss >= 1 && ss <= 3 && c.smooth_stages[ss - 1] >= 2) {
        const int k = ss - 1;
        const StreamLayout lay = {c.smooth_stages[k], c.smooth_stage_bytes[k], c.smooth_cols_off[k],
                                  c.smooth_vals_off[k]};
        const size_t smem = (size_t)lay.stages * lay.stage_bytes;
        const int sms = c.tune.sms > 0 ? c.tune.sms : 152;
        const __half *kh = reinterpret_cast<const __half *>(c.Kh);
        if (ss == 3)
            k_amg_k0_stream<MODE, O, 8><<<sms * 6, 128, smem, c.stream>>>(
                c.n, c.rowoff, c.cols, c.mask, kh, c.kh_scale, c.Pinv_rf, omega, x, b, out, sc, lay, c.status);
        else
            k_amg_k0_stream<MODE, O, 16><<<sms * ss, 256, smem, c.stream>>>(
                c.n, c.rowoff, c.cols, c.mask, kh, c.kh_scale, c.Pinv_rf, omega, x, b, out, sc, lay, c.status);
        return;
    }
    switch (c.tune.smooth_variant) {
    case 1:
        k0_launch_l<MODE, O, 8>(c, omega, x, b, out, sc);
        break;
    case 2:
        k0_launch_l<MODE, O, 4>(c, omega, x, b, out, sc);
        break;
    default:
        k0_launch_l<MODE, O, 16>(c, omega, x, b, out, sc);
    }
}

template <typename O>
static void k0_launch(Ctx &c, int mode, float omega, const float4 *xv, const float4 *bv, O *out)
{
    const float *x = (const float *)xv, *b = (const float *)bv;
    if (mode == SM_SMOOTH)
        k0_launch_m<SM_SMOOTH, O>(c, omega, x, b, out, c.sc);
    else
        k0_launch_m<SM_RESID, O>(c, omega, x, b, out, c.sc);
}

// one residual pass on the scratch vectors without the solve's early exit,
// for the autotuner's timing
void launch_amg_smoother_pass(Ctx &c)
{
    k0_launch_m<SM_RESID, float>(c, 1.0f, (const float *)c.x_f, (const float *)c.r_f, (float *)c.q_f, nullptr);
}

__global__ void k_to_float(long long count, const double *__restrict__ in, float *__restrict__ out)
{
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < count;
         k += (long long)gridDim.x * blockDim.x)
        out[k] = (float)in[k];
}

void launch_amg_stiffness32(Ctx &c)
{
    const long long count = 9 * c.nblk;
    k_to_float<<<grid_for(c, count), ATPB, 0, c.stream>>>(count, c.Kd, c.Kf);
}

__global__ void k_to_double(long long count, const float *__restrict__ in, double *__restrict__ out)
{
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < count;
         k += (long long)gridDim.x * blockDim.x)
        out[k] = (double)in[k];
}

void launch_stiffness64_of32(Ctx &c)
{
    const long long count = 9 * c.nblk;
    k_to_double<<<grid_for(c, count), ATPB, 0, c.stream>>>(count, c.Kf, c.Kc);
}

// max |v| as the bits of a non-negative float (which order like unsigned ints)
__global__ void __launch_bounds__(ATPB) k_absmax(long long count, const float *__restrict__ v, unsigned *out)
{
    float m = 0.f;
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < count;
         k += (long long)gridDim.x * blockDim.x)
        m = fmaxf(m, fabsf(v[k]));
    for (int o = 16; o > 0; o >>= 1)
        m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0)
        atomicMax(out, __float_as_uint(m));
}

// Kh = half(Kf / s) with s = max |Kf| / 2^14 (the largest value maps to 16384,
// well inside FP16's range; values below 2^-24 of the largest underflow)
__global__ void k_to_half(long long count, const float *__restrict__ in, __half *__restrict__ out,
                          const unsigned *__restrict__ maxbits, float *__restrict__ scale)
{
    const float mx = __uint_as_float(*maxbits);
    const float s = mx > 0.f ? mx * (1.0f / 16384.0f) : 1.0f;
    const float inv = 1.0f / s;
    if (blockIdx.x == 0 && threadIdx.x == 0)
        *scale = s;
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < count;
         k += (long long)gridDim.x * blockDim.x)
        out[k] = __float2half_rn(in[k] * inv);
}

void launch_amg_stiffness16(Ctx &c)
{
    const long long count = 9 * c.nblk;
    cudaMemsetAsync(c.kh_max, 0, sizeof(unsigned), c.stream);
    k_absmax<<<grid_for(c, count), ATPB, 0, c.stream>>>(count, c.Kf, c.kh_max);
    k_to_half<<<grid_for(c, count), ATPB, 0, c.stream>>>(count, c.Kf, reinterpret_cast<__half *>(c.Kh), c.kh_max,
                                                         c.kh_scale);
}

template <int R, int C, int MODE>
static void bsr_launch(Ctx &c, int nbr, const long long *ptr, const int *col, const unsigned short *val,
                       float vscale, const float *x, int SX, float *out, int SY, const float *b = nullptr,
                       const float *dinv = nullptr, float omega = 0.f)
{
    const int g = grid_for(c, (long long)nbr * BL_LANES);
    k_amg_bsr<R, C, MODE><<<g, ATPB, 0, c.stream>>>(nbr, ptr, col, reinterpret_cast<const __half *>(val), vscale,
                                                    x, SX, out, SY, b, dinv, omega, c.sc);
}

// FP32 throughout; level 0 works on the float4 buffers r_f (the right-hand
// side in FP32), x_f and q_f (the iterate and the residual), which the
// multigrid PCG does not otherwise use, and its last sweep writes z (FP64).
// With nu sweeps before and after the coarse correction, the iterate starts
// in one scratch buffer and changes buffer with every sweep but the first
// (2 nu - 1 times); the residual goes to the buffer the iterate is not in.
void launch_amg_vcycle(Ctx &c, const dvec4 *r, dvec4 *z)
{
    AmgDev &H = *c.amg;
    const int L = (int)H.lv.size();
    const int nu = std::max(1, c.opts.amg_sweeps);
    const int gd = grid_for(c, (long long)H.nc * 32);
    if (L == 0) {
        // level 0 is the coarsest: z = Cinv r over the 3 DOFs of each particle
        k_amg_dense<double, double><<<gd, ATPB, 0, c.stream>>>(H.nc, H.cinv, (const double *)r, (double *)z, 3, 4,
                                                               c.sc);
        return;
    }
    float4 *bt = c.r_f;
    // down
    for (int l = 0; l < L; l++) {
        AmgDevLevel &v = H.lv[l];
        float *bnext = (l + 1 < L) ? H.lv[l + 1].b : H.cb;
        const float om = (float)v.omega;
        if (l == 0) {
            float4 *it = c.x_f, *ot = c.q_f;
            k_amg_jacobi0<<<grid_for(c, c.n), ATPB, 0, c.stream>>>(c.n, c.mask, c.Pinv_f, om, (const double *)r,
                                                                   (float *)bt, (float *)it, c.sc);
            for (int s = 1; s < nu; s++) {
                k0_launch<float>(c, SM_SMOOTH, om, it, bt, (float *)ot);
                std::swap(it, ot);
            }
            k0_launch<float>(c, SM_RESID, om, it, bt, (float *)ot);
            bsr_launch<6, 3, BM_SET>(c, v.nnext, v.pt_ptr, v.pt_col, v.pt_val, 1.0f, (const float *)ot, 4, bnext, 6);
        } else {
            float *it = v.x, *ot = v.y;
            k_amg_jacobi6<<<grid_for(c, v.nb), ATPB, 0, c.stream>>>(v.nb, v.dinv, om, v.b, it, c.sc);
            for (int s = 1; s < nu; s++) {
                bsr_launch<6, 6, BM_SMOOTH>(c, v.nb, v.a_ptr, v.a_col, v.a_val, v.a_scale, it, 6, ot, 6, v.b, v.dinv, om);
                std::swap(it, ot);
            }
            bsr_launch<6, 6, BM_RESID>(c, v.nb, v.a_ptr, v.a_col, v.a_val, v.a_scale, it, 6, ot, 6, v.b);
            bsr_launch<6, 6, BM_SET>(c, v.nnext, v.pt_ptr, v.pt_col, v.pt_val, 1.0f, ot, 6, bnext, 6);
        }
    }
    k_amg_dense<float, float><<<gd, ATPB, 0, c.stream>>>(H.nc, H.cinv, H.cb, H.cx, 6, 6, c.sc);
    // up: the iterate is where the down sweep left it (the first buffer after
    // an even number of swaps, the second after an odd one)
    for (int l = L - 1; l >= 0; l--) {
        AmgDevLevel &v = H.lv[l];
        const float *e = (l + 1 < L) ? H.lv[l + 1].y : H.cx;
        const float om = (float)v.omega;
        if (l == 0) {
            float4 *it = (nu % 2 == 1) ? c.x_f : c.q_f, *ot = (nu % 2 == 1) ? c.q_f : c.x_f;
            bsr_launch<3, 6, BM_ADD>(c, v.nb, v.p_ptr, v.p_col, v.p_val, 1.0f, e, 6, (float *)it, 4);
            for (int s = 0; s < nu; s++) {
                if (s == nu - 1) {
                    k0_launch<double>(c, SM_SMOOTH, om, it, bt, (double *)z);
                } else {
                    k0_launch<float>(c, SM_SMOOTH, om, it, bt, (float *)ot);
                    std::swap(it, ot);
                }
            }
        } else {
            float *it = (nu % 2 == 1) ? v.x : v.y, *ot = (nu % 2 == 1) ? v.y : v.x;
            bsr_launch<6, 6, BM_ADD>(c, v.nb, v.p_ptr, v.p_col, v.p_val, 1.0f, e, 6, it, 6);
            for (int s = 0; s < nu; s++) {
                bsr_launch<6, 6, BM_SMOOTH>(c, v.nb, v.a_ptr, v.a_col, v.a_val, v.a_scale, it, 6, ot, 6, v.b, v.dinv, om);
                std::swap(it, ot);
            }
        }
    }
}

void launch_amg_init(Ctx &c, const dvec4 *b, double scale, double delta2, bool k32)
{
    k_amg_init<<<red_grid(c), ATPB, 0, c.stream>>>(amg_vec(c), b, scale, c.x_d, c.r_d, solve_rtol(c),
                                                   c.opts.cg_maxiter, delta2);
    launch_amg_vcycle(c, c.r_d, c.z_d);
    k_amg_rz<RZ_INIT><<<red_grid(c), ATPB, 0, c.stream>>>(amg_vec(c), c.r_d, c.z_d, c.p_d,
                                                          k32 ? c.p_split : nullptr);
}

void launch_amg_iter(Ctx &c, bool k32)
{
    if (k32)
        launch_spmv_diff(c, c.q_d, true);
    else
        launch_spmv_d(c, c.p_d, c.q_d, true, true);
    const int g = red_grid(c);
    k_amg_update<<<g, ATPB, 0, c.stream>>>(amg_vec(c), c.x_d, c.r_d, c.p_d, c.q_d);
    launch_amg_vcycle(c, c.r_d, c.z_d);
    k_amg_rz<RZ_ITER><<<g, ATPB, 0, c.stream>>>(amg_vec(c), c.r_d, c.z_d, c.p_d);
    launch_cg_p_d(c, k32);
}

void launch_amg_reliable(Ctx &c, const dvec4 *rtrue)
{
    k_amg_reliable<<<red_grid(c), ATPB, 0, c.stream>>>(amg_vec(c), rtrue, c.r_d);
    launch_amg_vcycle(c, c.r_d, c.z_d);
    k_amg_rz<RZ_RELIABLE><<<red_grid(c), ATPB, 0, c.stream>>>(amg_vec(c), c.r_d, c.z_d, c.p_d);
}

// ---- hierarchy on the device -------------------------------------------------------

template <typename T>
static int amg_alloc_copy(T *&d, const T *h, size_t count)
{
    if (count == 0)
        return LPM_OK;
    LPM_CUDA(cudaMalloc((void **)&d, sizeof(T) * count));
    if (h)
        LPM_CUDA(cudaMemcpy(d, h, sizeof(T) * count, cudaMemcpyHostToDevice));
    return LPM_OK;
}

// prolongation, restriction and coarse-operator values are kept in FP16 on
// the device (coarse operators scaled): they only shape the preconditioner,
// and FP16 quarters their traffic against FP64
// FP16 copies of block values divided by scale (round to nearest)
template <typename Vec>
static std::vector<unsigned short> to_half(const Vec &v, float scale)
{
    std::vector<unsigned short> h(v.size());
    const double inv = 1.0 / scale;
#pragma omp parallel for schedule(static)
    for (long long k = 0; k < (long long)v.size(); k++) {
        const __half x = __double2half(v[k] * inv);
        h[k] = *reinterpret_cast<const unsigned short *>(&x);
    }
    return h;
}

// max |v| / 2^14: the largest value maps to 16384, inside FP16's range
template <typename Vec>
static float half_scale(const Vec &v)
{
    double m = 0.0;
    for (size_t k = 0; k < v.size(); k++)
        m = std::max(m, std::fabs((double)v[k]));
    return m > 0.0 ? (float)(m / 16384.0) : 1.0f;
}

template <typename Vec>
static std::vector<float> to_float(const Vec &v)
{
    std::vector<float> f(v.size());
#pragma omp parallel for schedule(static)
    for (long long k = 0; k < (long long)v.size(); k++)
        f[k] = (float)v[k];
    return f;
}

static void amg_free_device(AmgDev &H)
{
    for (AmgDevLevel &v : H.lv) {
        void *ps[] = {v.a_ptr, v.a_col, v.a_val, v.dinv, v.p_ptr, v.p_col, v.p_val,
                      v.pt_ptr, v.pt_col, v.pt_val, v.b, v.x, v.y};
        for (void *p : ps)
            if (p)
                cudaFree(p);
    }
    H.lv.clear();
    void *ps[] = {H.cinv, H.cb, H.cx};
    for (void *p : ps)
        if (p)
            cudaFree(p);
    H.cinv = nullptr;
    H.cb = H.cx = nullptr;
    H.nc = H.cbs = 0;
}

void free_amg(Ctx &c)
{
    if (!c.amg)
        return;
    amg_free_device(*c.amg);
    delete c.amg;
    c.amg = nullptr;
}

static int amg_upload(AmgDev &H, const AmgHierarchy &h)
{
    int rc;
    const int L = (int)h.levels.size();
    H.lv.assign(L, AmgDevLevel());
    for (int l = 0; l < L; l++) {
        const AmgLevel &s = h.levels[l];
        AmgDevLevel &v = H.lv[l];
        v.nb = s.nblock;
        v.bs = s.bs;
        v.nnext = s.P.nbc;
        v.omega = s.omega;
        if ((rc = amg_alloc_copy(v.p_ptr, s.P.ptr.data(), s.P.ptr.size())) ||
            (rc = amg_alloc_copy(v.p_col, s.P.col.data(), s.P.col.size())) ||
            (rc = amg_alloc_copy(v.p_val, to_half(s.P.val, 1.0f).data(), s.P.val.size())) ||
            (rc = amg_alloc_copy(v.pt_ptr, s.Pt.ptr.data(), s.Pt.ptr.size())) ||
            (rc = amg_alloc_copy(v.pt_col, s.Pt.col.data(), s.Pt.col.size())) ||
            (rc = amg_alloc_copy(v.pt_val, to_half(s.Pt.val, 1.0f).data(), s.Pt.val.size())))
            return rc;
        if (l > 0) {
            if ((rc = amg_alloc_copy(v.a_ptr, s.A.ptr.data(), s.A.ptr.size())) ||
                (rc = amg_alloc_copy(v.a_col, s.A.col.data(), s.A.col.size())) ||
                (v.a_scale = half_scale(s.A.val), false) ||
                (rc = amg_alloc_copy(v.a_val, to_half(s.A.val, v.a_scale).data(), s.A.val.size())) ||
                (rc = amg_alloc_copy(v.dinv, to_float(s.Dinv).data(), s.Dinv.size())) ||
                (rc = amg_alloc_copy<float>(v.b, nullptr, 6 * (size_t)s.nblock)) ||
                (rc = amg_alloc_copy<float>(v.x, nullptr, 6 * (size_t)s.nblock)) ||
                (rc = amg_alloc_copy<float>(v.y, nullptr, 6 * (size_t)s.nblock)))
                return rc;
        }
    }
    H.nc = h.coarse_n;
    H.cbs = h.coarse_A.R;
    if ((rc = amg_alloc_copy(H.cinv, h.coarse_inv.data(), h.coarse_inv.size())) ||
        (rc = amg_alloc_copy<float>(H.cb, nullptr, (size_t)H.nc)) ||
        (rc = amg_alloc_copy<float>(H.cx, nullptr, (size_t)H.nc)))
        return rc;
    return LPM_OK;
}

int amg_prepare(Ctx &c)
{
    const int n = c.n;
    if (!c.amg)
        c.amg = new AmgDev();
    AmgDev &H = *c.amg;
    std::vector<uint8_t> mask(n);
    LPM_CUDA(cudaMemcpyAsync(mask.data(), c.mask, n, cudaMemcpyDeviceToHost, c.stream));
    int rc = sync(c);
    if (rc)
        return rc;
    if (H.builds > 0 && !H.stale && mask == H.mask_h)
        return LPM_OK;
    const auto t0 = std::chrono::steady_clock::now();
    // the current stiffness in FP64 on the host
    const bool k32 = c.opts.precision == LPM_PREC_MIXED;
    const size_t nv = 9 * (size_t)c.nblk;
    hvec<double> val(nv);
    if (k32) {
        hvec<float> vf(nv);
        LPM_CUDA(cudaMemcpyAsync(vf.data(), c.Kf, nv * sizeof(float), cudaMemcpyDeviceToHost, c.stream));
        if ((rc = sync(c)))
            return rc;
#pragma omp parallel for schedule(static)
        for (long long k = 0; k < (long long)nv; k++)
            val[k] = (double)vf[k];
    } else {
        LPM_CUDA(cudaMemcpyAsync(val.data(), c.Kd, nv * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
        if ((rc = sync(c)))
            return rc;
    }
    const HostSetup &hs = c.hs;
    AmgInput in;
    in.n = n;
    in.xyz = hs.xyz.data();
    in.mask = mask.data();
    in.rowoff = hs.rowoff.data();
    in.npad = hs.npad.data();
    in.nconn = hs.nconn.data();
    in.cols = hs.cols.data();
    in.val = val.data();
    AmgOptions opt;
    opt.agg_spacing = c.opts.amg_spacing > 0.0 ? c.opts.amg_spacing : 6.0 * hs.radius;
    AmgHierarchy h;
    const int nl = amg_build(in, h, opt);
    if (nl == -2)
        return fail(LPM_ERR_ARG, "multigrid: the lattice does not coarsen with this aggregate spacing");
    if (nl < 0)
        return fail(LPM_ERR_ARG, "multigrid: the coarsest operator is not positive definite (singular stiffness)");
    // the captured PCG graphs hold the old hierarchy's pointers
    if (c.graph_fp64) {
        cudaGraphExecDestroy(c.graph_fp64);
        c.graph_fp64 = nullptr;
    }
    if (c.graph_fp32) {
        cudaGraphExecDestroy(c.graph_fp32);
        c.graph_fp32 = nullptr;
    }
    amg_free_device(H);
    if ((rc = amg_upload(H, h))) {
        amg_free_device(H);
        H.builds = 0;
        return rc;
    }
    H.mask_h.swap(mask);
    H.stale = false;
    H.ref_iters = -1;
    H.builds++;
    H.build_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    if (c.trace)
        std::fprintf(stderr, "lpm: multigrid build %d: %d levels + coarsest %d DOFs, %.1f ms\n", H.builds,
                     (int)H.lv.size(), H.nc, H.build_ms);
    return LPM_OK;
}

}  // namespace lpm
