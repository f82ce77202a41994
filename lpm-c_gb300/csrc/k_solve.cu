// Block-CSR SpMV and the block-Jacobi preconditioned CG that replaces the
// reference's MKL RCI CG (src/solver.c:188-270), in FP64 and in FP32.
//
// SpMV: FP32 uses a half-warp per block row, each lane taking four
// consecutive 3x3 blocks per 64-block chunk: one 128-bit load per stiffness
// component (the row is stored component-major), one int4 of column indices
// and one float4 gather of x per block.  FP64 uses a full warp per row, two
// blocks per lane, double2 loads.  Rows are distributed grid-stride over a
// fixed grid of a multiple of the SM count.
//
// The boundary conditions of setDispBC_stiffnessUpdate3D
// (src/boundary.c:159-281) are applied as a mask: constrained DOFs keep a
// zero residual and a zero search direction, and the product is zeroed there,
// which is the same iteration as CG on the row/column-eliminated matrix.
//
// Reductions are deterministic: per-block partial sums, then the last block
// adds them in a fixed order and updates the CG scalars.
#include "lpm_internal.h"
#include "stream_pipe.h"

namespace lpm {

constexpr int VTPB = 256;

__device__ __forceinline__ double warp_sum(double s)
{
    for (int o = 16; o > 0; o >>= 1)
        s += __shfl_xor_sync(0xffffffffu, s, o);
    return s;
}

// Block partial of NV values -> partials; last block reduces, then calls
// fin(total) on thread 0.  All threads of the grid must call it.
template <int NV, int NT = VTPB, typename Fin>
__device__ void grid_reduce(double (&v)[NV], double *partials, unsigned *counter, Fin fin)
{
    __shared__ double red[NV][NT / 32];
    __shared__ bool last;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < NV; k++) {
        const double s = warp_sum(v[k]);
        if (lane == 0)
            red[k][wid] = s;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < NV; k++) {
            double s = 0.0;
            for (int w = 0; w < NT / 32; w++)
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
        for (unsigned b = threadIdx.x; b < gridDim.x; b += NT)
            s += __ldcg(&partials[(size_t)k * gridDim.x + b]);
        s = warp_sum(s);
        if (lane == 0)
            red[k][wid] = s;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double tot[NV];
#pragma unroll
        for (int k = 0; k < NV; k++) {
            double s = 0.0;
            for (int w = 0; w < NT / 32; w++)
                s += red[k][w];
            tot[k] = s;
        }
        fin(tot);
        *counter = 0u;
    }
}

__device__ __forceinline__ float4 mask4(float4 v, uint8_t m)
{
    return make_float4((m & 1) ? v.x : 0.f, (m & 2) ? v.y : 0.f, (m & 4) ? v.z : 0.f, 0.f);
}
__device__ __forceinline__ dvec4 mask4(dvec4 v, uint8_t m)
{
    return make_dvec4((m & 1) ? v.x : 0.0, (m & 2) ? v.y : 0.0, (m & 4) ? v.z : 0.0, 0.0);
}

struct SpmvArgs {
    int n;
    const long long *rowoff;
    const int *npad, *cols;
    const uint8_t *mask;
    double *partials;
    unsigned *counter;
    CgScalars *sc;
    // batched specimens: skip the whole launch when *stop is set, and the rows
    // of specimens whose solve has stopped (spec_done[row_spec[row]] != 0)
    const int *stop;
    const int *row_spec, *spec_done, *spec_upd;
    const int *act_chunk, *n_act;  // batch: chunks of BATCH_TPB rows holding a running specimen
};

// B consecutive stiffness values of one component: one 64/128-bit (FP32)
// or 128/256-bit (FP64) streaming load.
template <typename V, int B>
struct VPack;
template <>
struct VPack<float, 4> {
    typedef float4 T;
};
template <>
struct VPack<float, 2> {
    typedef float2 T;
};
template <>
struct VPack<double, 4> {
    typedef double4_32a T;
};
template <>
struct VPack<double, 2> {
    typedef double2 T;
};
__device__ __forceinline__ float4 ld_vals(const float4 *p) { return __ldcs(p); }
__device__ __forceinline__ float2 ld_vals(const float2 *p) { return __ldcs(p); }
__device__ __forceinline__ double2 ld_vals(const double2 *p) { return __ldcs(p); }
__device__ __forceinline__ double4_32a ld_vals(const double4_32a *p) { return *p; }
template <int B, typename T, typename A>
__device__ __forceinline__ void unpack(const T &v, A (&o)[B])
{
    o[0] = v.x;
    o[1] = v.y;
    if constexpr (B == 4) {
        o[2] = v.z;
        o[3] = v.w;
    }
}
template <int B>
__device__ __forceinline__ void load_cols(const int *p, int (&c)[B])
{
    if constexpr (B == 4) {
        const int4 v = __ldg(reinterpret_cast<const int4 *>(p));
        c[0] = v.x;
        c[1] = v.y;
        c[2] = v.z;
        c[3] = v.w;
    } else {
        const int2 v = __ldg(reinterpret_cast<const int2 *>(p));
        c[0] = v.x;
        c[1] = v.y;
    }
}
template <typename A>
__device__ __forceinline__ void xyz_of(const float4 &v, A &x, A &y, A &z)
{
    x = (A)v.x;
    y = (A)v.y;
    z = (A)v.z;
}
template <typename A>
__device__ __forceinline__ void xyz_of(const dvec4 &v, A &x, A &y, A &z)
{
    x = (A)v.x;
    y = (A)v.y;
    z = (A)v.z;
}
// read-only gathers of one particle's vector entry
__device__ __forceinline__ float4 ldx(const float4 *p) { return __ldg(p); }
__device__ __forceinline__ dvec4 ldx(const dvec4 *p)
{
    const double2 a = __ldg(reinterpret_cast<const double2 *>(p));
    const double2 b = __ldg(reinterpret_cast<const double2 *>(p) + 1);
    return make_dvec4(a.x, a.y, b.x, b.y);
}
__device__ __forceinline__ void store3(float4 *p, float a, float b, float c) { *p = make_float4(a, b, c, 0.f); }
__device__ __forceinline__ void store3(dvec4 *p, double a, double b, double c) { *p = make_dvec4(a, b, c, 0.0); }

// y = K x with L lanes per block row; each lane takes B consecutive blocks
// of every L*B-block chunk of its row (rows are padded to a multiple of 4
// blocks, so B = 4 or 2 never crosses a row end).  The default L = 16, B = 4
// gives one 128-bit value load per component and one int4 of columns per
// lane for the 61-block rows of the interior; the autotuner picks among the
// variants.  V: stiffness value type (products and sums in V), X: vector
// element type (float4 or dvec4).  MASK zeroes the constrained DOFs of y;
// DOT accumulates x.y in FP64 and sets alpha = rz / (x.y) for the CG.
// BATCH: rows of stopped specimens are skipped (their y is left as it was).
template <typename V, typename X, bool MASK, bool DOT, bool BATCH = false, int L = 16, int B = 4>
__global__ void __launch_bounds__(VTPB) k_spmv(SpmvArgs a, const V *__restrict__ val, const X *__restrict__ x,
                                               X *__restrict__ y)
{
    static_assert(L == 4 || L == 8 || L == 16 || L == 32, "lanes per row");
    static_assert(B == 2 || B == 4, "blocks per lane");
    typedef typename VPack<V, B>::T P;
    if (DOT && a.sc->done)
        return;
    if (BATCH && *a.stop)
        return;
    const int sub = threadIdx.x & (L - 1);
    const unsigned gmask = (L == 32) ? 0xffffffffu : (((1u << L) - 1u) << ((threadIdx.x & 31) & ~(L - 1)));
    const int gw = (blockIdx.x * blockDim.x + threadIdx.x) / L;
    const int nhw = (gridDim.x * blockDim.x) / L;
    double dot = 0.0;
    const int nrows = BATCH ? (*a.n_act) * BATCH_TPB : a.n;
    for (int vrow = gw; vrow < nrows; vrow += nhw) {
        int row = vrow;
        if (BATCH) {
            row = a.act_chunk[vrow / BATCH_TPB] * BATCH_TPB + vrow % BATCH_TPB;
            if (row >= a.n || a.spec_done[a.row_spec[row]])
                continue;
        }
        const long long off = a.rowoff[row];
        const int np = a.npad[row];
        const V *vr = val + 9 * off;
        V y0 = 0, y1 = 0, y2 = 0;
        for (int b0 = B * sub; b0 < np; b0 += B * L) {
            int cc[B];
            load_cols<B>(a.cols + off + b0, cc);
            V v[9][B];
#pragma unroll
            for (int k = 0; k < 9; k++)
                unpack<B>(ld_vals(reinterpret_cast<const P *>(vr + (size_t)k * np + b0)), v[k]);
            V xs[B][3];
#pragma unroll
            for (int j = 0; j < B; j++)
                xyz_of<V>(ldx(x + cc[j]), xs[j][0], xs[j][1], xs[j][2]);
#pragma unroll
            for (int j = 0; j < B; j++) {
                y0 += v[0][j] * xs[j][0] + v[1][j] * xs[j][1] + v[2][j] * xs[j][2];
                y1 += v[3][j] * xs[j][0] + v[4][j] * xs[j][1] + v[5][j] * xs[j][2];
                y2 += v[6][j] * xs[j][0] + v[7][j] * xs[j][1] + v[8][j] * xs[j][2];
            }
        }
#pragma unroll
        for (int o = L / 2; o > 0; o >>= 1) {
            y0 += __shfl_xor_sync(gmask, y0, o);
            y1 += __shfl_xor_sync(gmask, y1, o);
            y2 += __shfl_xor_sync(gmask, y2, o);
        }
        if (sub == 0) {
            if (MASK) {
                const uint8_t m = a.mask[row];
                y0 = (m & 1) ? y0 : V(0);
                y1 = (m & 2) ? y1 : V(0);
                y2 = (m & 4) ? y2 : V(0);
            }
            store3(y + row, y0, y1, y2);
            if (DOT) {
                double px, py, pz;
                xyz_of<double>(x[row], px, py, pz);
                dot += px * (double)y0 + py * (double)y1 + pz * (double)y2;
            }
        }
    }
    if (DOT) {
        double v[1] = {dot};
        CgScalars *sc = a.sc;
        grid_reduce<1>(v, a.partials, a.counter, [sc](const double *t) {
            sc->pq = t[0];
            sc->alpha = (t[0] != 0.0) ? sc->rz / t[0] : 0.0;
        });
    }
}

// ---- difference-form FP32 product ---------------------------------------------
//
// The FP32 product K32 x with x rounded to FP32 is accurate only to about
// 6e-8 |K| |x|.  The stiffness annihilates rigid translations, so on the
// smooth vectors a multigrid-preconditioned CG works with, |K x| is smaller
// than |K| |x| by about the condition number and the rounded product loses
// all accuracy there (measured: the mixed multigrid PCG stagnates at 1M
// particles).  The difference form
//     (K32 x)_i = sum_j K32_ij (x_j - x_i) + R_i x_i,   R_i = sum_j K32_ij,
// is an identity for the FP32 matrix; with x held as two FP32 parts
// (hi = fl32(x), lo = fl32(x - hi)) the differences
// (hi_j - hi_i) + (lo_j - lo_i) are formed in FP32 with an error relative to
// the difference itself, and R_i, zero for the exact tangent (the bond forces
// depend on relative positions only), is the FP64 row sum of the FP32
// values.  The product error becomes about 6e-8 sum_j |K_ij| |x_j - x_i|:
// FP32 arithmetic and an FP32 stiffness stream with the accuracy the CG needs.

// the two FP32 parts of one particle's entry, hi then lo, as one 32-byte
// record (a single sector per neighbour gather)
struct __align__(32) SplitRec {
    float4 hi, lo;
};

__device__ __forceinline__ void split_store(const dvec4 &v, float4 *rec)
{
    const float hx = __double2float_rn(v.x), hy = __double2float_rn(v.y), hz = __double2float_rn(v.z);
    SplitRec s;
    s.hi = make_float4(hx, hy, hz, 0.f);
    s.lo = make_float4(__double2float_rn(v.x - (double)hx), __double2float_rn(v.y - (double)hy),
                       __double2float_rn(v.z - (double)hz), 0.f);
    *reinterpret_cast<SplitRec *>(rec) = s;
}

// Krs[row][k] = sum over the row's blocks of component k of Kf (FP64 sums,
// rounded once); 16 lanes per block row, four blocks per lane per load.
__global__ void __launch_bounds__(VTPB) k_row_sums(int n, const long long *__restrict__ rowoff,
                                                   const int *__restrict__ npad, const float *__restrict__ val,
                                                   float *__restrict__ out)
{
    const int sub = threadIdx.x & 15;
    const unsigned gmask = 0xffffu << ((threadIdx.x & 31) & ~15);
    const int g = (blockIdx.x * blockDim.x + threadIdx.x) >> 4;
    const int ng = (gridDim.x * blockDim.x) >> 4;
    for (int row = g; row < n; row += ng) {
        const long long off = rowoff[row];
        const int np = npad[row];
        const float *vr = val + 9 * off;
        double s[9];
#pragma unroll
        for (int k = 0; k < 9; k++)
            s[k] = 0.0;
        for (int b0 = 4 * sub; b0 < np; b0 += 64) {
#pragma unroll
            for (int k = 0; k < 9; k++) {
                const float4 v = __ldcs(reinterpret_cast<const float4 *>(vr + (size_t)k * np + b0));
                s[k] += ((double)v.x + (double)v.y) + ((double)v.z + (double)v.w);
            }
        }
#pragma unroll
        for (int k = 0; k < 9; k++) {
#pragma unroll
            for (int o = 8; o > 0; o >>= 1)
                s[k] += __shfl_xor_sync(gmask, s[k], o);
        }
        if (sub == 0) {
#pragma unroll
            for (int k = 0; k < 9; k++)
                out[(size_t)row * 9 + k] = (float)s[k];
        }
    }
}

// y = mask(K32 x) in the difference form from x = hi + lo; L lanes per
// block row, four blocks per lane (the layouts of k_spmv's variants, chosen
// by the autotuner).  DOT: p.y with p = x64 (FP64) and alpha = rz / (p.y), as
// k_spmv.
template <bool DOT, int L = 16>
__global__ void __launch_bounds__(VTPB) k_spmv_diff(SpmvArgs a, const float *__restrict__ val,
                                                    const float *__restrict__ rs,
                                                    const SplitRec *__restrict__ split,
                                                    const dvec4 *__restrict__ x64, dvec4 *__restrict__ y)
{
    static_assert(L == 4 || L == 8 || L == 16, "lanes per row");
    if (DOT && a.sc->done)
        return;
    const int sub = threadIdx.x & (L - 1);
    const unsigned gmask = ((1u << L) - 1u) << ((threadIdx.x & 31) & ~(L - 1));
    const int gw = (blockIdx.x * blockDim.x + threadIdx.x) / L;
    const int nhw = (gridDim.x * blockDim.x) / L;
    const int n = a.n;
    double dot = 0.0;
    for (int row = gw; row < n; row += nhw) {
        const long long off = a.rowoff[row];
        const int np = a.npad[row];
        const float *vr = val + 9 * off;
        const SplitRec own = split[row];
        const float4 hi_i = own.hi, lo_i = own.lo;
        float y0 = 0.f, y1 = 0.f, y2 = 0.f;
        for (int b0 = 4 * sub; b0 < np; b0 += 4 * L) {
            int cc[4];
            load_cols<4>(a.cols + off + b0, cc);
            float v[9][4];
#pragma unroll
            for (int k = 0; k < 9; k++)
                unpack<4>(ld_vals(reinterpret_cast<const float4 *>(vr + (size_t)k * np + b0)), v[k]);
            float d[4][3];
#pragma unroll
            for (int j = 0; j < 4; j++) {
                const SplitRec rj = split[cc[j]];
                const float4 h = rj.hi, l = rj.lo;
                d[j][0] = (h.x - hi_i.x) + (l.x - lo_i.x);
                d[j][1] = (h.y - hi_i.y) + (l.y - lo_i.y);
                d[j][2] = (h.z - hi_i.z) + (l.z - lo_i.z);
            }
#pragma unroll
            for (int j = 0; j < 4; j++) {
                y0 += v[0][j] * d[j][0] + v[1][j] * d[j][1] + v[2][j] * d[j][2];
                y1 += v[3][j] * d[j][0] + v[4][j] * d[j][1] + v[5][j] * d[j][2];
                y2 += v[6][j] * d[j][0] + v[7][j] * d[j][1] + v[8][j] * d[j][2];
            }
        }
        // + R_i x_i (R_i is rounding-sized: hi_i suffices), its 9 values
        // (36 contiguous bytes) spread over the lanes
#pragma unroll
        for (int t = 0; t < (9 + L - 1) / L; t++) {
            const int k = sub + t * L;
            if (k < 9) {
                const int c = k % 3;
                const float add = rs[(size_t)row * 9 + k] * (c == 0 ? hi_i.x : (c == 1 ? hi_i.y : hi_i.z));
                if (k < 3)
                    y0 += add;
                else if (k < 6)
                    y1 += add;
                else
                    y2 += add;
            }
        }
#pragma unroll
        for (int o = L / 2; o > 0; o >>= 1) {
            y0 += __shfl_xor_sync(gmask, y0, o);
            y1 += __shfl_xor_sync(gmask, y1, o);
            y2 += __shfl_xor_sync(gmask, y2, o);
        }
        if (sub == 0) {
            const uint8_t m = a.mask[row];
            const double o0 = (m & 1) ? (double)y0 : 0.0, o1 = (m & 2) ? (double)y1 : 0.0,
                         o2 = (m & 4) ? (double)y2 : 0.0;
            y[row] = make_dvec4(o0, o1, o2, 0.0);
            if (DOT) {
                // p = hi + lo (the FP64 p to 2^-48): no second read of p
                dot += ((double)hi_i.x + (double)lo_i.x) * o0 + ((double)hi_i.y + (double)lo_i.y) * o1 +
                       ((double)hi_i.z + (double)lo_i.z) * o2;
            }
        }
    }
    if (DOT) {
        double v[1] = {dot};
        CgScalars *sc = a.sc;
        grid_reduce<1>(v, a.partials, a.counter, [sc](const double *t) {
            sc->pq = t[0];
            sc->alpha = (t[0] != 0.0) ? sc->rz / t[0] : 0.0;
        });
    }
}

// ---- streamed difference-form product ---------------------------------------
// The product of k_spmv_diff<DOT, 16> (the same lanes, blocks and arithmetic
// per row) with the stiffness stream decoupled from the gathers.  Persistent
// CTAs walk tiles of ROWS consecutive rows, whose row offsets, column
// indices and values are contiguous in the block-CSR arrays.  Thread 0
// copies a tile into a ring of shared-memory stages with cp.async.bulk,
// completing on the stage's mbarrier by byte count, up to stages - 1 tiles
// ahead of the computation; every warp computes two rows of the tile from
// shared memory (a half-warp per row) and gathers the split x from L2.  The
// copy engine keeps the DRAM stream deep with no registers held, where the
// register-fed kernel is limited to the loads its resident warps have issued.
// ROWS = 16 (256 threads, one or two CTAs per SM) or 8 (128 threads, five
// CTAs per SM: more rows in computation per SM for the same shared memory).
//
// Every mbarrier wait is bounded (STREAM_WAIT_CYCLES, about a second); one
// that runs out sets LPM_STATUS_DEVICE_WAIT in the status word and ends the
// kernel once the copies it issued have landed (again with bounded waits);
// the CG stops (done = 3) after the kernel's dot product.
template <bool DOT, int ROWS>
__global__ void __launch_bounds__(ROWS * 16, ROWS == 16 ? 1 : 5)
    k_spmv_diff_stream(SpmvArgs a, StreamLayout lay, const float *__restrict__ val, const float *__restrict__ rs,
                       const SplitRec *__restrict__ split, dvec4 *__restrict__ y, int *status)
{
    constexpr int NT = ROWS * 16;
    constexpr unsigned RO_BYTES = (ROWS + 2) * 8;  // the tile's row offsets, r0 .. r0 + ROWS + 1
    extern __shared__ __align__(128) unsigned char stage_mem[];
    __shared__ unsigned long long full[STREAM_MAX_STAGES], empty[STREAM_MAX_STAGES];
    __shared__ volatile int abort_k;
    if (DOT && a.sc->done)
        return;
    const int n = a.n, S = lay.stages;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int sub = lane & 15, rl = 2 * wid + (lane >> 4);  // row of the tile
    const unsigned gmask = 0xffffu << (lane & 16);
    const int ntiles = (n + ROWS - 1) / ROWS;
    const int mine = (int)blockIdx.x < ntiles ? (ntiles - 1 - (int)blockIdx.x) / (int)gridDim.x + 1 : 0;
    if (threadIdx.x == 0) {
        for (int s = 0; s < S; s++) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], NT / 32);
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
    // warp 0 issues the copies; its lanes hold the block range [pb0, pb1) of
    // the tiles jb + lane, loaded 32 tiles at a time
    int issued = 0, jb = -32;
    long long pb0 = 0, pb1 = 0;
    auto issue_next = [&]() -> bool {  // warp 0, warp-uniform
        const int j = issued, s = j % S;
        if (j - jb >= 32) {
            jb += 32;
            if (jb + lane < mine) {
                const int r0 = first_row(jb + lane);
                pb0 = a.rowoff[r0];
                pb1 = a.rowoff[min(r0 + ROWS, n)];
            }
        }
        const long long b0 = __shfl_sync(0xffffffffu, pb0, j - jb);
        const long long b1 = __shfl_sync(0xffffffffu, pb1, j - jb);
        if (j >= S && !warp_mbar_wait(&empty[s], (unsigned)((j / S) - 1) & 1u))
            return false;
        if (lane == 0) {
            unsigned char *st = stage_mem + (size_t)s * lay.stage_bytes;
            const unsigned nb = (unsigned)(b1 - b0);
            mbar_expect_tx(&full[s], RO_BYTES + 40u * nb);
            bulk_g2s(st, a.rowoff + first_row(j), RO_BYTES, &full[s]);
            if (nb) {
                bulk_g2s(st + lay.cols_off, a.cols + b0, 4u * nb, &full[s]);
                bulk_g2s(st + lay.vals_off, val + 9 * b0, 36u * nb, &full[s]);
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
    double dot = 0.0;
    int i = 0;
    for (; i < mine; i++) {
        if (__any_sync(0xffffffffu, abort_k != 0))
            break;
        if (wid == 0 && issued < mine && !issue_next()) {
            fail();
            break;
        }
        const int s = i % S;
        const int row = first_row(i) + rl;
        // the row's own entries, ahead of the stage wait
        SplitRec own = {};
        float rsv = 0.f;
        uint8_t m = 0;
        if (row < n) {
            own = split[row];
            if (sub < 9)
                rsv = rs[(size_t)row * 9 + sub];
            if (sub == 0)
                m = a.mask[row];
        }
        if (!warp_mbar_wait(&full[s], (unsigned)(i / S) & 1u)) {
            fail();
            break;
        }
        if (row < n) {
            const unsigned char *st = stage_mem + (size_t)s * lay.stage_bytes;
            const long long *ro = reinterpret_cast<const long long *>(st);
            const int o = (int)(ro[rl] - ro[0]), np = (int)(ro[rl + 1] - ro[rl]);
            const int *cs = reinterpret_cast<const int *>(st + lay.cols_off) + o;
            const float *vr = reinterpret_cast<const float *>(st + lay.vals_off) + 9 * (size_t)o;
            const float4 hi_i = own.hi, lo_i = own.lo;
            float y0 = 0.f, y1 = 0.f, y2 = 0.f;
            for (int b0 = 4 * sub; b0 < np; b0 += 64) {
                const int4 c4 = *reinterpret_cast<const int4 *>(cs + b0);
                const int cc[4] = {c4.x, c4.y, c4.z, c4.w};
                float d[4][3];
#pragma unroll
                for (int j = 0; j < 4; j++) {
                    const SplitRec rj = split[cc[j]];
                    const float4 h = rj.hi, l = rj.lo;
                    d[j][0] = (h.x - hi_i.x) + (l.x - lo_i.x);
                    d[j][1] = (h.y - hi_i.y) + (l.y - lo_i.y);
                    d[j][2] = (h.z - hi_i.z) + (l.z - lo_i.z);
                }
                float v[9][4];
#pragma unroll
                for (int k = 0; k < 9; k++)
                    unpack<4>(*reinterpret_cast<const float4 *>(vr + (size_t)k * np + b0), v[k]);
#pragma unroll
                for (int j = 0; j < 4; j++) {
                    y0 += v[0][j] * d[j][0] + v[1][j] * d[j][1] + v[2][j] * d[j][2];
                    y1 += v[3][j] * d[j][0] + v[4][j] * d[j][1] + v[5][j] * d[j][2];
                    y2 += v[6][j] * d[j][0] + v[7][j] * d[j][1] + v[8][j] * d[j][2];
                }
            }
            if (sub < 9) {
                const int c = sub % 3;
                const float add = rsv * (c == 0 ? hi_i.x : (c == 1 ? hi_i.y : hi_i.z));
                if (sub < 3)
                    y0 += add;
                else if (sub < 6)
                    y1 += add;
                else
                    y2 += add;
            }
#pragma unroll
            for (int off = 8; off > 0; off >>= 1) {
                y0 += __shfl_xor_sync(gmask, y0, off);
                y1 += __shfl_xor_sync(gmask, y1, off);
                y2 += __shfl_xor_sync(gmask, y2, off);
            }
            if (sub == 0) {
                const double o0 = (m & 1) ? (double)y0 : 0.0, o1 = (m & 2) ? (double)y1 : 0.0,
                             o2 = (m & 4) ? (double)y2 : 0.0;
                y[row] = make_dvec4(o0, o1, o2, 0.0);
                if (DOT)
                    dot += ((double)hi_i.x + (double)lo_i.x) * o0 + ((double)hi_i.y + (double)lo_i.y) * o1 +
                           ((double)hi_i.z + (double)lo_i.z) * o2;
            }
        }
        __syncwarp();
        if (lane == 0)
            mbar_arrive(&empty[s]);
    }
    // after a failed wait: let the copies issued past the last consumed tile land
    if (wid == 0) {
        for (int k = i; k < issued; k++)
            if (!warp_mbar_wait(&full[k % S], (unsigned)(k / S) & 1u))
                break;
    }
    if (DOT) {
        double v[1] = {dot};
        CgScalars *sc = a.sc;
        grid_reduce<1, NT>(v, a.partials, a.counter, [sc](const double *t) {
            sc->pq = t[0];
            sc->alpha = (t[0] != 0.0) ? sc->rz / t[0] : 0.0;
        });
        // stop the CG after a failed wait (every block of this persistent
        // grid read done at its start, and all of them took part in the sum)
        __syncthreads();
        if (threadIdx.x == 0 && abort_k)
            a.sc->done = 3;
    }
}

// two consecutive stiffness values of one component as FP64 (streaming)
__device__ __forceinline__ double2 ld_pair(const float *p)
{
    const float2 v = __ldcs(reinterpret_cast<const float2 *>(p));
    return make_double2((double)v.x, (double)v.y);
}
__device__ __forceinline__ double2 ld_pair(const double *p) { return __ldcs(reinterpret_cast<const double2 *>(p)); }

// Refinement residual r = b - K32 x64 with FP64 products and sums (masked),
// and |r|^2 into norms[slot].  The values are the FP32 stiffness (V = float,
// converted per value) or its exact FP64 copy (V = double: the same
// arithmetic and result without a conversion per value on the FP64 pipe).
// BATCH: only the rows of specimens due for a reliable update (running with a
// request, or recursively converged).
template <bool BATCH = false, typename V = float>
__global__ void __launch_bounds__(VTPB) k_refine_res(SpmvArgs a, const V *__restrict__ val,
                                                     const dvec4 *__restrict__ x,
                                                     const dvec4 *__restrict__ bvec,
                                                     dvec4 *__restrict__ r, double *norms, int slot,
                                                     double bscale)
{
    const int lane = threadIdx.x & 31;
    const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    double acc = 0.0;
    for (int row = gw; row < a.n; row += nw) {
        if (BATCH) {
            const int s = a.row_spec[row];
            const int d = a.spec_done[s];
            if (!((d == 0 && a.spec_upd[s]) || d == 1))
                continue;
        }
        const long long off = a.rowoff[row];
        const int np = a.npad[row];
        const V *vr = val + 9 * off;
        double y0 = 0.0, y1 = 0.0, y2 = 0.0;
        for (int b0 = 2 * lane; b0 < np; b0 += 64) {
            const int2 c2 = __ldg(reinterpret_cast<const int2 *>(a.cols + off + b0));
            double2 v[9];
#pragma unroll
            for (int k = 0; k < 9; k++)
                v[k] = ld_pair(vr + (size_t)k * np + b0);
            const dvec4 xa = x[c2.x], xb = x[c2.y];
            y0 += v[0].x * xa.x + v[1].x * xa.y + v[2].x * xa.z;
            y1 += v[3].x * xa.x + v[4].x * xa.y + v[5].x * xa.z;
            y2 += v[6].x * xa.x + v[7].x * xa.y + v[8].x * xa.z;
            y0 += v[0].y * xb.x + v[1].y * xb.y + v[2].y * xb.z;
            y1 += v[3].y * xb.x + v[4].y * xb.y + v[5].y * xb.z;
            y2 += v[6].y * xb.x + v[7].y * xb.y + v[8].y * xb.z;
        }
        y0 = warp_sum(y0);
        y1 = warp_sum(y1);
        y2 = warp_sum(y2);
        if (lane == 0) {
            const dvec4 bb = bvec[row];
            dvec4 out = make_dvec4(bb.x * bscale - y0, bb.y * bscale - y1, bb.z * bscale - y2, 0.0);
            out = mask4(out, a.mask[row]);
            r[row] = out;
            acc += out.x * out.x + out.y * out.y + out.z * out.z;
        }
    }
    double v[1] = {acc};
    grid_reduce<1>(v, a.partials, a.counter, [norms, slot](const double *t) { norms[slot] = t[0]; });
}

// z = P^{-1} r with the 3x3 block inverses stored [9][n]
template <typename V, typename V4>
__device__ __forceinline__ V4 apply_pinv(const V *P, int n, int i, V4 r)
{
    V4 z;
    z.x = P[(size_t)0 * n + i] * r.x + P[(size_t)1 * n + i] * r.y + P[(size_t)2 * n + i] * r.z;
    z.y = P[(size_t)3 * n + i] * r.x + P[(size_t)4 * n + i] * r.y + P[(size_t)5 * n + i] * r.z;
    z.z = P[(size_t)6 * n + i] * r.x + P[(size_t)7 * n + i] * r.y + P[(size_t)8 * n + i] * r.z;
    z.w = 0;
    return z;
}

struct VecArgs {
    int n;
    const uint8_t *mask;
    double *partials;
    unsigned *counter;
    CgScalars *sc;
};

// x = 0, r = mask(b) (cast), z = P^-1 r, p = z, rz, rr, |b|^2, tolerance.
template <typename V, typename V4>
__global__ void __launch_bounds__(VTPB) k_cg_init(VecArgs a, const dvec4 *b, double scale, const V *P,
                                                  V4 *x, V4 *r, V4 *z, V4 *p, double rtol, int maxit,
                                                  double delta2)
{
    double v[2] = {0.0, 0.0};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.n; i += gridDim.x * blockDim.x) {
        const dvec4 bb = mask4(b[i], a.mask[i]);
        V4 rv;
        rv.x = (V)(bb.x * scale);
        rv.y = (V)(bb.y * scale);
        rv.z = (V)(bb.z * scale);
        rv.w = 0;
        const V4 zv = apply_pinv<V, V4>(P, a.n, i, rv);
        V4 zero;
        zero.x = zero.y = zero.z = zero.w = 0;
        x[i] = zero;
        r[i] = rv;
        z[i] = zv;
        p[i] = zv;
        v[0] += (double)rv.x * zv.x + (double)rv.y * zv.y + (double)rv.z * zv.z;
        v[1] += (double)rv.x * rv.x + (double)rv.y * rv.y + (double)rv.z * rv.z;
    }
    CgScalars *sc = a.sc;
    grid_reduce<2>(v, a.partials, a.counter, [sc, rtol, maxit, delta2](const double *t) {
        sc->rz = t[0];
        sc->rz_old = t[0];
        sc->rr = t[1];
        sc->rr_max = t[1];
        sc->bnorm2 = t[1];
        sc->tol2 = rtol * rtol * t[1];
        sc->upd_delta2 = delta2;
        sc->it = 0;
        sc->maxit = maxit;
        sc->done = (t[1] <= sc->tol2 || !(t[1] == t[1])) ? 1 : 0;
        sc->alpha = 0.0;
        sc->beta = 0.0;
        sc->upd_req = 0;
    });
}

// Reliable update (residual replacement) of the FP32 CG: r = (FP64 true
// residual) * scale, z = P^-1 r, the search direction p is kept, so the
// iteration continues with its Krylov history.
__global__ void __launch_bounds__(VTPB) k_reliable(VecArgs a, const dvec4 *r64, double scale, const float *P,
                                                   float4 *r, float4 *z)
{
    double v[2] = {0.0, 0.0};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.n; i += gridDim.x * blockDim.x) {
        const dvec4 bb = mask4(r64[i], a.mask[i]);
        const float4 rv = make_float4((float)(bb.x * scale), (float)(bb.y * scale), (float)(bb.z * scale), 0.f);
        const float4 zv = apply_pinv<float, float4>(P, a.n, i, rv);
        r[i] = rv;
        z[i] = zv;
        v[0] += (double)rv.x * zv.x + (double)rv.y * zv.y + (double)rv.z * zv.z;
        v[1] += (double)rv.x * rv.x + (double)rv.y * rv.y + (double)rv.z * rv.z;
    }
    CgScalars *sc = a.sc;
    grid_reduce<2>(v, a.partials, a.counter, [sc](const double *t) {
        sc->rz = t[0];
        sc->rr = t[1];
        sc->rr_max = t[1];
        sc->done = !(t[1] == t[1]) ? 3 : 0;
        sc->upd_req = 0;
    });
}

// x += alpha p; r -= alpha q; z = P^-1 r; rz, rr; convergence test.
template <typename V, typename V4>
__global__ void __launch_bounds__(VTPB) k_cg_update(VecArgs a, const V *P, V4 *x, V4 *r, V4 *z,
                                                    const V4 *p, const V4 *q)
{
    CgScalars *sc = a.sc;
    if (sc->done)
        return;
    const V al = (V)sc->alpha;
    double v[2] = {0.0, 0.0};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.n; i += gridDim.x * blockDim.x) {
        V4 xv = x[i], rv = r[i];
        const V4 pv = p[i], qv = q[i];
        xv.x += al * pv.x;
        xv.y += al * pv.y;
        xv.z += al * pv.z;
        rv.x -= al * qv.x;
        rv.y -= al * qv.y;
        rv.z -= al * qv.z;
        const V4 zv = apply_pinv<V, V4>(P, a.n, i, rv);
        x[i] = xv;
        r[i] = rv;
        z[i] = zv;
        v[0] += (double)rv.x * zv.x + (double)rv.y * zv.y + (double)rv.z * zv.z;
        v[1] += (double)rv.x * rv.x + (double)rv.y * rv.y + (double)rv.z * rv.z;
    }
    grid_reduce<2>(v, a.partials, a.counter, [sc](const double *t) {
        sc->rz_old = sc->rz;
        sc->rz = t[0];
        sc->rr = t[1];
        sc->beta = (sc->rz_old != 0.0) ? t[0] / sc->rz_old : 0.0;
        sc->it += 1;
        if (t[1] <= sc->tol2)
            sc->done = 1;
        else if (!(t[1] == t[1]))
            sc->done = 3;
        else if (sc->it >= sc->maxit)
            sc->done = 2;
        else if (t[1] < sc->upd_delta2 * sc->rr_max)
            sc->upd_req = 1;  // raised as done = 4 once p is updated (k_cg_p)
        if (t[1] > sc->rr_max)
            sc->rr_max = t[1];
    });
}

// p = z + beta p; the last block turns a pending reliable-update request into
// done = 4, so the host updates only after p belongs to the new iteration.
// With hi/lo (FP64 vectors only), p is also written as two FP32 parts for
// the difference-form product (split_store).
template <typename V, typename V4>
__global__ void __launch_bounds__(VTPB) k_cg_p(int n, CgScalars *sc, const V4 *z, V4 *p, unsigned *counter,
                                               float4 *split = nullptr)
{
    if (sc->done)
        return;
    const V be = (V)sc->beta;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        V4 pv = p[i];
        const V4 zv = z[i];
        pv.x = zv.x + be * pv.x;
        pv.y = zv.y + be * pv.y;
        pv.z = zv.z + be * pv.z;
        p[i] = pv;
        if constexpr (sizeof(V) == 8) {
            if (split)
                split_store(pv, split + 2 * (size_t)i);
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        if (atomicAdd(counter, 1u) == gridDim.x - 1) {
            if (sc->upd_req) {
                sc->upd_req = 0;
                sc->done = 4;
            }
            *counter = 0u;
        }
    }
}

// Reliable update of the FP64-vector variant: r = true residual (already in
// the scaled units of the iteration), z = P^-1 r; p is kept.
__global__ void __launch_bounds__(VTPB) k_reliable_d(VecArgs a, const dvec4 *rtrue, const double *P, dvec4 *r,
                                                     dvec4 *z)
{
    double v[2] = {0.0, 0.0};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.n; i += gridDim.x * blockDim.x) {
        const dvec4 rv = mask4(rtrue[i], a.mask[i]);
        const dvec4 zv = apply_pinv<double, dvec4>(P, a.n, i, rv);
        r[i] = rv;
        z[i] = zv;
        v[0] += rv.x * zv.x + rv.y * zv.y + rv.z * zv.z;
        v[1] += rv.x * rv.x + rv.y * rv.y + rv.z * rv.z;
    }
    CgScalars *sc = a.sc;
    grid_reduce<2>(v, a.partials, a.counter, [sc](const double *t) {
        sc->rz = t[0];
        sc->rr = t[1];
        sc->rr_max = t[1];
        sc->done = !(t[1] == t[1]) ? 3 : 0;
        sc->upd_req = 0;
    });
}

// x64 += x32 / scale, x32 = 0
__global__ void k_axpy_refine(int n, dvec4 *x, float4 *d, double inv_scale)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        dvec4 xv = x[i];
        const float4 dv = d[i];
        xv.x += (double)dv.x * inv_scale;
        xv.y += (double)dv.y * inv_scale;
        xv.z += (double)dv.z * inv_scale;
        x[i] = xv;
        d[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
}

// y = x * s
__global__ void k_scale_copy(int n, dvec4 *y, const dvec4 *x, double s)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const dvec4 v = x[i];
        y[i] = make_dvec4(v.x * s, v.y * s, v.z * s, 0.0);
    }
}

__global__ void __launch_bounds__(VTPB) k_norm2(int n, const dvec4 *v, double *partials, unsigned *counter,
                                                double *norms, int slot)
{
    double s[1] = {0.0};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const dvec4 a = v[i];
        s[0] += a.x * a.x + a.y * a.y + a.z * a.z;
    }
    grid_reduce<1>(s, partials, counter, [norms, slot](const double *t) { norms[slot] = t[0]; });
}

static int sm_count(const Ctx &c)
{
    if (c.tune.sms > 0)
        return c.tune.sms;
    int sms = 152;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c.device);
    return sms;
}

int red_grid(const Ctx &c) { return sm_count(c) * c.tune.vec_per_sm; }
int spmv_grid(const Ctx &c) { return sm_count(c) * c.tune.spmv_per_sm; }
int spmv_variant_lanes(int v) { return v == 1 ? 8 : (v == 2 ? 32 : (v == 3 ? 4 : 16)); }
int spmv_variant_blocks(int v) { return v == 2 ? 2 : 4; }

// Event pair around SpMV launches; inside a stream capture the records become
// external event nodes, so the last SpMV of each graph launch is timed.
static void record_timing(Ctx &c, cudaEvent_t ev)
{
    if (!c.time_spmv || !c.time_this)
        return;
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    cudaStreamIsCapturing(c.stream, &cs);
    if (cs == cudaStreamCaptureStatusActive)
        cudaEventRecordWithFlags(ev, c.stream, cudaEventRecordExternal);
    else
        cudaEventRecord(ev, c.stream);
}

static SpmvArgs spmv_args(Ctx &c)
{
    SpmvArgs a;
    a.n = c.n;
    a.rowoff = c.rowoff;
    a.npad = c.npad;
    a.cols = c.cols;
    a.mask = c.mask;
    a.partials = c.partials;
    a.counter = c.counter;
    a.sc = c.sc;
    a.stop = nullptr;
    a.row_spec = nullptr;
    a.spec_done = nullptr;
    a.spec_upd = nullptr;
    a.act_chunk = nullptr;
    a.n_act = nullptr;
    return a;
}

static VecArgs vec_args(Ctx &c)
{
    VecArgs a;
    a.n = c.n;
    a.mask = c.mask;
    a.partials = c.partials;
    a.counter = c.counter;
    a.sc = c.sc;
    return a;
}

template <typename V, typename X, bool MASK, bool DOT, bool BATCH>
static void spmv_variant(const Ctx &c, const SpmvArgs &a, const V *val, const X *x, X *y)
{
    const int g = spmv_grid(c);
    switch (c.tune.spmv_variant) {
    case 1:
        k_spmv<V, X, MASK, DOT, BATCH, 8, 4><<<g, VTPB, 0, c.stream>>>(a, val, x, y);
        break;
    case 2:
        k_spmv<V, X, MASK, DOT, BATCH, 32, 2><<<g, VTPB, 0, c.stream>>>(a, val, x, y);
        break;
    case 3:
        k_spmv<V, X, MASK, DOT, BATCH, 4, 4><<<g, VTPB, 0, c.stream>>>(a, val, x, y);
        break;
    default:
        k_spmv<V, X, MASK, DOT, BATCH, 16, 4><<<g, VTPB, 0, c.stream>>>(a, val, x, y);
    }
}

template <typename V, typename X>
static void spmv_launch(Ctx &c, const V *val, const X *x, X *y, bool masked, bool dot)
{
    SpmvArgs a = spmv_args(c);
    record_timing(c, c.ev_a);
    if (masked && dot)
        spmv_variant<V, X, true, true, false>(c, a, val, x, y);
    else if (masked)
        spmv_variant<V, X, true, false, false>(c, a, val, x, y);
    else
        spmv_variant<V, X, false, false, false>(c, a, val, x, y);
    record_timing(c, c.ev_b);
}

void launch_spmv_f(Ctx &c, const float4 *x, float4 *y, bool masked, bool dot)
{
    spmv_launch<float, float4>(c, c.Kf, x, y, masked, dot);
}

void launch_spmv_d(Ctx &c, const dvec4 *x, dvec4 *y, bool masked, bool dot)
{
    spmv_launch<double, dvec4>(c, c.Kd, x, y, masked, dot);
}

void launch_spmv_fx(Ctx &c, const dvec4 *x, dvec4 *y, bool masked, bool dot)
{
    spmv_launch<float, dvec4>(c, c.Kf, x, y, masked, dot);
}

// masked y = K x over every specimen of a batch that is still running
void launch_spmv_batch(Ctx &c, const dvec4 *x, dvec4 *y, bool k32)
{
    SpmvArgs a = spmv_args(c);
    a.stop = c.bcg.all_done;
    a.row_spec = c.bcg.spec_of;
    a.spec_done = c.bcg.done;
    a.act_chunk = c.bcg.act_chunk;
    a.n_act = c.bcg.n_act;
    record_timing(c, c.ev_a);
    if (k32)
        spmv_variant<float, dvec4, true, false, true>(c, a, c.Kf, x, y);
    else
        spmv_variant<double, dvec4, true, false, true>(c, a, c.Kd, x, y);
    record_timing(c, c.ev_b);
}

void launch_refine_residual(Ctx &c, const dvec4 *x, const dvec4 *b, dvec4 *r, double bscale)
{
    if (c.kc_version >= 0 && c.kc_version == c.kf_version)
        k_refine_res<false, double><<<red_grid(c), VTPB, 0, c.stream>>>(spmv_args(c), c.Kc, x, b, r, c.norms, 2,
                                                                        bscale);
    else
        k_refine_res<false, float><<<red_grid(c), VTPB, 0, c.stream>>>(spmv_args(c), c.Kf, x, b, r, c.norms, 2,
                                                                       bscale);
}

// r = b - K x with an FP64 matrix (the FP64 stiffness), |r|^2 into norms[2]
void launch_refine_residual64(Ctx &c, const double *K, const dvec4 *x, const dvec4 *b, dvec4 *r)
{
    k_refine_res<false, double><<<red_grid(c), VTPB, 0, c.stream>>>(spmv_args(c), K, x, b, r, c.norms, 2, 1.0);
}

void launch_refine_batch(Ctx &c, const dvec4 *x, const dvec4 *b, dvec4 *r)
{
    SpmvArgs a = spmv_args(c);
    a.row_spec = c.bcg.spec_of;
    a.spec_done = c.bcg.done;
    a.spec_upd = c.bcg.upd;
    k_refine_res<true, float><<<red_grid(c), VTPB, 0, c.stream>>>(a, c.Kf, x, b, r, c.norms, 3, 1.0);
}

// mixed precision with FP64 CG vectors: FP32 stiffness, FP32 products and row
// sums, FP64 search directions, residuals and dot products
void launch_cg_init_fx(Ctx &c, const dvec4 *b, double scale, double delta2)
{
    k_cg_init<double, dvec4><<<red_grid(c), VTPB, 0, c.stream>>>(
        vec_args(c), b, scale, c.Pinv_d, c.x_d, c.r_d, c.z_d, c.p_d, solve_rtol(c), c.opts.cg_maxiter, delta2);
}

void launch_cg_iter_fx(Ctx &c)
{
    launch_spmv_fx(c, c.p_d, c.q_d, true, true);
    const int g = red_grid(c);
    k_cg_update<double, dvec4><<<g, VTPB, 0, c.stream>>>(vec_args(c), c.Pinv_d, c.x_d, c.r_d, c.z_d,
                                                           c.p_d, c.q_d);
    k_cg_p<double, dvec4><<<g, VTPB, 0, c.stream>>>(c.n, c.sc, c.z_d, c.p_d, c.counter);
}

// reliable update of the FP64-vector variant: r = (true residual), z = P^-1 r
void launch_reliable_d(Ctx &c, const dvec4 *rtrue)
{
    k_reliable_d<<<red_grid(c), VTPB, 0, c.stream>>>(vec_args(c), rtrue, c.Pinv_d, c.r_d, c.z_d);
}

void launch_cg_init_d(Ctx &c, const dvec4 *b, double scale)
{
    k_cg_init<double, dvec4><<<red_grid(c), VTPB, 0, c.stream>>>(
        vec_args(c), b, scale, c.Pinv_d, c.x_d, c.r_d, c.z_d, c.p_d, solve_rtol(c), c.opts.cg_maxiter, 0.0);
}

void launch_cg_init_f(Ctx &c, const dvec4 *r64, double scale, double rtol, double delta2)
{
    k_cg_init<float, float4><<<red_grid(c), VTPB, 0, c.stream>>>(
        vec_args(c), r64, scale, c.Pinv_f, c.x_f, c.r_f, c.z_f, c.p_f, rtol, c.opts.cg_maxiter, delta2);
}

void launch_reliable(Ctx &c, const dvec4 *r64, double scale)
{
    k_reliable<<<red_grid(c), VTPB, 0, c.stream>>>(vec_args(c), r64, scale, c.Pinv_f, c.r_f, c.z_f);
}

void launch_scale_copy(Ctx &c, dvec4 *y, const dvec4 *x, double s)
{
    k_scale_copy<<<red_grid(c), VTPB, 0, c.stream>>>(c.n, y, x, s);
}

void launch_cg_iter_d(Ctx &c)
{
    launch_spmv_d(c, c.p_d, c.q_d, true, true);
    const int g = red_grid(c);
    k_cg_update<double, dvec4><<<g, VTPB, 0, c.stream>>>(vec_args(c), c.Pinv_d, c.x_d, c.r_d, c.z_d,
                                                           c.p_d, c.q_d);
    k_cg_p<double, dvec4><<<g, VTPB, 0, c.stream>>>(c.n, c.sc, c.z_d, c.p_d, c.counter);
}

// p = z + beta p on the FP64 vectors (the multigrid PCG, k_amg.cu); split:
// also the two FP32 parts of p for the difference-form product
void launch_cg_p_d(Ctx &c, bool split)
{
    k_cg_p<double, dvec4><<<red_grid(c), VTPB, 0, c.stream>>>(c.n, c.sc, c.z_d, c.p_d, c.counter,
                                                              split ? c.p_split : nullptr);
}

void launch_row_sums(Ctx &c)
{
    k_row_sums<<<spmv_grid(c), VTPB, 0, c.stream>>>(c.n, c.rowoff, c.npad, c.Kf, c.Krs);
}

// Stage layouts of the streamed product's variants for rows of at most
// max_npad blocks: tiles of 16 rows with one or two CTAs per SM, tiles of 8
// rows with five; a variant gets 0 stages where fewer than two fit in its
// share of shared memory.  Also lifts the kernels' dynamic shared-memory
// limit.
void init_stream_product(Ctx &c, int max_npad)
{
    auto up = [](int v, int a) { return (v + a - 1) / a * a; };
    int optin = 0, per_sm = 0;
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, c.device);
    cudaDeviceGetAttribute(&per_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, c.device);
    const int rows[3] = {16, 16, 8}, ctas[3] = {1, 2, 5};
    for (int k = 0; k < 3; k++) {
        c.stream_cols_off[k] = up((rows[k] + 2) * 8, 128);
        c.stream_vals_off[k] = c.stream_cols_off[k] + up(rows[k] * max_npad * 4, 128);
        c.stream_stage_bytes[k] = c.stream_vals_off[k] + up(rows[k] * max_npad * 36, 128);
        const int avail = std::min(optin, per_sm / ctas[k]) - 2048;  // static memory, per-block reservation
        const int st = avail > 0 ? std::min(STREAM_MAX_STAGES, avail / c.stream_stage_bytes[k]) : 0;
        c.stream_stages[k] = st >= 2 ? st : 0;
    }
    // one limit per kernel instantiation: the largest of the variants using it
    int max16 = 0, max8 = 0;
    for (int k = 0; k < 3; k++) {
        const int bytes = c.stream_stages[k] * c.stream_stage_bytes[k];
        int &m = rows[k] == 16 ? max16 : max8;
        m = std::max(m, bytes);
    }
    if (max16 > 0) {
        cudaFuncSetAttribute(k_spmv_diff_stream<true, 16>, cudaFuncAttributeMaxDynamicSharedMemorySize, max16);
        cudaFuncSetAttribute(k_spmv_diff_stream<false, 16>, cudaFuncAttributeMaxDynamicSharedMemorySize, max16);
    }
    if (max8 > 0) {
        cudaFuncSetAttribute(k_spmv_diff_stream<true, 8>, cudaFuncAttributeMaxDynamicSharedMemorySize, max8);
        cudaFuncSetAttribute(k_spmv_diff_stream<false, 8>, cudaFuncAttributeMaxDynamicSharedMemorySize, max8);
    }
    cudaGetLastError();
}

template <bool DOT>
static void spmv_diff_variant(Ctx &c, const SpmvArgs &a, dvec4 *y)
{
    const SplitRec *sp = reinterpret_cast<const SplitRec *>(c.p_split);
    const int ds = c.tune.diff_stream;
    if (ds >= 1 && ds <= 3 && c.stream_stages[ds - 1] >= 2) {
        const int k = ds - 1;
        const StreamLayout lay = {c.stream_stages[k], c.stream_stage_bytes[k], c.stream_cols_off[k],
                                  c.stream_vals_off[k]};
        const size_t smem = (size_t)lay.stages * lay.stage_bytes;
        if (ds == 3)
            k_spmv_diff_stream<DOT, 8><<<sm_count(c) * 5, 128, smem, c.stream>>>(a, lay, c.Kf, c.Krs, sp, y,
                                                                                c.status);
        else
            k_spmv_diff_stream<DOT, 16><<<sm_count(c) * ds, 256, smem, c.stream>>>(a, lay, c.Kf, c.Krs, sp, y,
                                                                                  c.status);
        return;
    }
    const int g = spmv_grid(c);
    switch (c.tune.spmv_variant) {
    case 1:
        k_spmv_diff<DOT, 8><<<g, VTPB, 0, c.stream>>>(a, c.Kf, c.Krs, sp, c.p_d, y);
        break;
    case 3:
        k_spmv_diff<DOT, 4><<<g, VTPB, 0, c.stream>>>(a, c.Kf, c.Krs, sp, c.p_d, y);
        break;
    default:  // 0, and 2 (whose 32 lanes x 2 blocks has no difference-form counterpart)
        k_spmv_diff<DOT, 16><<<g, VTPB, 0, c.stream>>>(a, c.Kf, c.Krs, sp, c.p_d, y);
    }
}

void launch_spmv_diff(Ctx &c, dvec4 *y, bool dot)
{
    SpmvArgs a = spmv_args(c);
    record_timing(c, c.ev_a);
    if (dot)
        spmv_diff_variant<true>(c, a, y);
    else
        spmv_diff_variant<false>(c, a, y);
    record_timing(c, c.ev_b);
}

void launch_cg_iter_f(Ctx &c)
{
    launch_spmv_f(c, c.p_f, c.q_f, true, true);
    const int g = red_grid(c);
    k_cg_update<float, float4><<<g, VTPB, 0, c.stream>>>(vec_args(c), c.Pinv_f, c.x_f, c.r_f, c.z_f, c.p_f,
                                                         c.q_f);
    k_cg_p<float, float4><<<g, VTPB, 0, c.stream>>>(c.n, c.sc, c.z_f, c.p_f, c.counter);
}

void launch_axpy_refine(Ctx &c, double scale)
{
    k_axpy_refine<<<red_grid(c), VTPB, 0, c.stream>>>(c.n, c.x_d, c.x_f, 1.0 / scale);
}

void launch_norm2(Ctx &c, const dvec4 *v, int slot)
{
    k_norm2<<<red_grid(c), VTPB, 0, c.stream>>>(c.n, v, c.partials, c.counter, c.norms, slot);
}

}  // namespace lpm
