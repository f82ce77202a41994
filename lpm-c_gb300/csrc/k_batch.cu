// Batched specimens: many independent lattices concatenated in one context
// (their stiffness is block-diagonal over specimens), solved together by a
// block-Jacobi PCG whose scalars are per specimen.  Each kernel is one launch
// over all specimens; every specimen keeps its own step size, convergence
// test and iteration count, and a specimen that has stopped is frozen.
//
// Per-specimen sums are deterministic: one thread block per chunk of
// BATCH_TPB consecutive particles; a warp-level segmented scan (specimens are
// contiguous particle ranges) and a fixed-order pass over the warp results
// give one partial per (chunk, specimen) segment; the last block to finish
// adds, for every specimen, its segments in chunk order (one warp per
// specimen, lane-strided, then a fixed shuffle tree).
#include <algorithm>
#include "lpm_internal.h"

namespace lpm {

namespace {

constexpr int TPB = BATCH_TPB;
constexpr int NW = TPB / 32;
constexpr unsigned FULL = 0xffffffffu;

__device__ __forceinline__ double wsum(double s)
{
    for (int o = 16; o > 0; o >>= 1)
        s += __shfl_xor_sync(FULL, s, o);
    return s;
}

__device__ __forceinline__ dvec4 bmask4(dvec4 v, uint8_t m)
{
    return make_dvec4((m & 1) ? v.x : 0.0, (m & 2) ? v.y : 0.0, (m & 4) ? v.z : 0.0, 0.0);
}

__device__ __forceinline__ dvec4 pinv_apply(const double *P, int n, int i, dvec4 r)
{
    return make_dvec4(P[0 * (size_t)n + i] * r.x + P[1 * (size_t)n + i] * r.y + P[2 * (size_t)n + i] * r.z,
                      P[3 * (size_t)n + i] * r.x + P[4 * (size_t)n + i] * r.y + P[5 * (size_t)n + i] * r.z,
                      P[6 * (size_t)n + i] * r.x + P[7 * (size_t)n + i] * r.y + P[8 * (size_t)n + i] * r.z,
                      0.0);
}

// Per-specimen sums, part 1: the block's chunk ch (every thread passes its
// particle's specimen s, -1 beyond n, and NV values) -> one partial per
// (chunk, specimen) segment.  Must be reached by every thread of the block.
template <int NV>
struct SegShared {
    double ev[NV][TPB];
    int es[TPB];
    int en[NW];
    bool last;
};

template <int NV>
__device__ void seg_chunk(const BatchCg &b, SegShared<NV> &sh, int ch, int s, double (&v)[NV])
{
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    // inclusive scan within each run of equal s
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int so = __shfl_up_sync(FULL, s, o);
        double y[NV];
#pragma unroll
        for (int k = 0; k < NV; k++)
            y[k] = __shfl_up_sync(FULL, v[k], o);
        if (lane >= o && so == s) {
#pragma unroll
            for (int k = 0; k < NV; k++)
                v[k] += y[k];
        }
    }
    const int sn = __shfl_down_sync(FULL, s, 1);
    const bool end = (lane == 31) || (sn != s);
    const unsigned bal = __ballot_sync(FULL, end);
    if (end) {
        const int e = wid * 32 + __popc(bal & ((1u << lane) - 1u));
#pragma unroll
        for (int k = 0; k < NV; k++)
            sh.ev[k][e] = v[k];
        sh.es[e] = s;
    }
    if (lane == 0)
        sh.en[wid] = __popc(bal);
    __syncthreads();
    if (threadIdx.x == 0) {
        const int s0 = sh.es[0];  // specimen of the chunk's first particle
        const int base = b.seg_base[ch];
        int cur = -2;
        double acc[NV];
#pragma unroll
        for (int k = 0; k < NV; k++)
            acc[k] = 0.0;
        for (int w = 0; w < NW; w++)
            for (int e = 0; e < sh.en[w]; e++) {
                const int sp = sh.es[w * 32 + e];
                if (sp != cur) {
                    if (cur >= 0) {
#pragma unroll
                        for (int k = 0; k < NV; k++)
                            b.partials[(size_t)k * b.nseg + base + (cur - s0)] = acc[k];
                    }
                    cur = sp;
#pragma unroll
                    for (int k = 0; k < NV; k++)
                        acc[k] = sh.ev[k][w * 32 + e];
                } else {
#pragma unroll
                    for (int k = 0; k < NV; k++)
                        acc[k] += sh.ev[k][w * 32 + e];
                }
            }
        if (cur >= 0) {
#pragma unroll
            for (int k = 0; k < NV; k++)
                b.partials[(size_t)k * b.nseg + base + (cur - s0)] = acc[k];
        }
    }
    __syncthreads();  // the shared entries are reused by the block's next chunk
}

// Part 2, after the block's last chunk: the last block of the grid adds, for
// every specimen with need(sp), its segments in chunk order (one warp per
// specimen) and calls fin(sp, totals) on the warp's lane 0; with TRACK it
// then sets all_done = AND over all specimens of (done != 0).
template <int NV, bool TRACK, typename Need, typename Fin>
__device__ void seg_finish(const BatchCg &b, SegShared<NV> &sh, Need need, Fin fin)
{
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (threadIdx.x == 0) {
        __threadfence();
        sh.last = (atomicAdd(b.counter, 1u) == gridDim.x - 1);
    }
    __syncthreads();
    if (!sh.last)
        return;
    __threadfence();
    int all = 1;
    for (int sp = wid; sp < b.nspec; sp += NW) {
        if (need(sp)) {
            const int cf = b.off[sp] / TPB, cl = (b.off[sp + 1] - 1) / TPB;
            double t[NV];
#pragma unroll
            for (int k = 0; k < NV; k++)
                t[k] = 0.0;
            for (int ch = cf + lane; ch <= cl; ch += 32) {
                const int seg = b.seg_base[ch] + (sp - b.spec_of[ch * TPB]);
#pragma unroll
                for (int k = 0; k < NV; k++)
                    t[k] += __ldcg(&b.partials[(size_t)k * b.nseg + seg]);
            }
#pragma unroll
            for (int k = 0; k < NV; k++)
                t[k] = wsum(t[k]);
            if (lane == 0)
                fin(sp, t);
        }
        if (TRACK && lane == 0)
            all &= (b.done[sp] != 0);
    }
    all = __syncthreads_and(all);
    if (threadIdx.x == 0) {
        if (TRACK)
            *b.all_done = all;
        *b.counter = 0u;
    }
}

// Chunks a kernel covers: all of them, or the compacted list of chunks that
// hold a running specimen.
struct ChunkList {
    const int *list;  // nullptr: all chunks
    int count;
    __device__ __forceinline__ int at(int k) const { return list ? list[k] : k; }
};
__device__ __forceinline__ ChunkList all_chunks(const BatchCg &b) { return ChunkList{nullptr, b.nchunk}; }
__device__ __forceinline__ ChunkList active_chunks(const BatchCg &b) { return ChunkList{b.act_chunk, *b.n_act}; }

// squared |residual| and |reaction| of every specimen (updateRR's norms,
// src/lpmc_project.c:412-413, per specimen)
__global__ void __launch_bounds__(TPB) k_bnorm(BatchCg b, const dvec4 *res, const dvec4 *Pin, const uint8_t *mask,
                                               double *out)
{
    __shared__ SegShared<2> sh;
    const ChunkList L = all_chunks(b);
    for (int k = blockIdx.x; k < L.count; k += gridDim.x) {
        const int ch = L.at(k), i = ch * TPB + threadIdx.x;
        double v[2] = {0.0, 0.0};
        int s = -1;
        if (i < b.n) {
            s = b.spec_of[i];
            const dvec4 r = res[i], p = Pin[i];
            const uint8_t m = mask[i];
            v[0] = r.x * r.x + r.y * r.y + r.z * r.z;
            v[1] = ((m & 1) ? 0.0 : p.x * p.x) + ((m & 2) ? 0.0 : p.y * p.y) + ((m & 4) ? 0.0 : p.z * p.z);
        }
        seg_chunk<2>(b, sh, ch, s, v);
    }
    seg_finish<2, false>(b, sh, [](int) { return true; }, [out](int sp, const double *t) {
        out[2 * sp] = t[0];
        out[2 * sp + 1] = t[1];
    });
}

// x = 0, r = bs = mask(b) / |b_s|, z = P^-1 r, p = z; stopped specimens get
// r = 0 and done = 5
__global__ void __launch_bounds__(TPB) k_bcg_init(BatchCg b, const dvec4 *bv, const uint8_t *mask, const double *P,
                                                  dvec4 *x, dvec4 *r, dvec4 *z, dvec4 *p, dvec4 *bs, double rtol)
{
    __shared__ SegShared<2> sh;
    const ChunkList L = all_chunks(b);
    for (int k = blockIdx.x; k < L.count; k += gridDim.x) {
        const int ch = L.at(k), i = ch * TPB + threadIdx.x;
        double v[2] = {0.0, 0.0};
        int s = -1;
        if (i < b.n) {
            s = b.spec_of[i];
            const double sc = b.active[s] ? b.bscale[s] : 0.0;
            const dvec4 bb = bmask4(bv[i], mask[i]);
            const dvec4 rv = make_dvec4(bb.x * sc, bb.y * sc, bb.z * sc, 0.0);
            const dvec4 zv = pinv_apply(P, b.n, i, rv);
            x[i] = make_dvec4(0.0, 0.0, 0.0, 0.0);
            r[i] = rv;
            bs[i] = rv;
            z[i] = zv;
            p[i] = zv;
            v[0] = rv.x * zv.x + rv.y * zv.y + rv.z * zv.z;
            v[1] = rv.x * rv.x + rv.y * rv.y + rv.z * rv.z;
        }
        seg_chunk<2>(b, sh, ch, s, v);
    }
    seg_finish<2, true>(b, sh, [](int) { return true; }, [b, rtol](int sp, const double *t) {
        b.rz[sp] = t[0];
        b.rz_old[sp] = t[0];
        b.rr[sp] = t[1];
        b.rr_max[sp] = t[1];
        b.tol2[sp] = rtol * rtol * t[1];  // t[1] = 1 for a running specimen (|bs| = 1)
        b.it[sp] = 0;
        b.nrel[sp] = 0;
        b.alpha[sp] = 0.0;
        b.beta[sp] = 0.0;
        b.upd[sp] = 0;
        b.done[sp] = !b.active[sp] ? 5 : ((t[1] <= b.tol2[sp] || !(t[1] == t[1])) ? 1 : 0);
    });
}

// act_chunk = the chunks holding a particle of a running specimen (done == 0);
// n_act was cleared before the launch.  The order of the list is free: the
// per-chunk results land in fixed places.
__global__ void k_bcg_compact(BatchCg b)
{
    const int ch = blockIdx.x * blockDim.x + threadIdx.x;
    if (ch >= b.nchunk)
        return;
    const int first = ch * TPB, last = min(b.n, first + TPB) - 1;
    bool run = false;
    for (int sp = b.spec_of[first]; sp <= b.spec_of[last]; sp++)
        run = run || (b.done[sp] == 0);
    if (run)
        b.act_chunk[atomicAdd(b.n_act, 1)] = ch;
}

// alpha = rz / (p.q) per running specimen
__global__ void __launch_bounds__(TPB) k_bcg_alpha(BatchCg b, const dvec4 *p, const dvec4 *q)
{
    if (*b.all_done)
        return;
    __shared__ SegShared<1> sh;
    const ChunkList L = active_chunks(b);
    for (int k = blockIdx.x; k < L.count; k += gridDim.x) {
        const int ch = L.at(k), i = ch * TPB + threadIdx.x;
        double v[1] = {0.0};
        int s = -1;
        if (i < b.n) {
            s = b.spec_of[i];
            if (b.done[s] == 0) {
                const dvec4 a = p[i], c = q[i];
                v[0] = a.x * c.x + a.y * c.y + a.z * c.z;
            }
        }
        seg_chunk<1>(b, sh, ch, s, v);
    }
    seg_finish<1, false>(b, sh, [b](int sp) { return b.done[sp] == 0; }, [b](int sp, const double *t) {
        b.alpha[sp] = (t[0] != 0.0) ? b.rz[sp] / t[0] : 0.0;
    });
}

// x += alpha p, r -= alpha q, z = P^-1 r; rz, rr, beta and the tests
__global__ void __launch_bounds__(TPB) k_bcg_update(BatchCg b, const double *P, dvec4 *x, dvec4 *r, dvec4 *z,
                                                    const dvec4 *p, const dvec4 *q)
{
    if (*b.all_done)
        return;
    __shared__ SegShared<2> sh;
    const ChunkList L = active_chunks(b);
    for (int k = blockIdx.x; k < L.count; k += gridDim.x) {
        const int ch = L.at(k), i = ch * TPB + threadIdx.x;
        double v[2] = {0.0, 0.0};
        int s = -1;
        if (i < b.n) {
            s = b.spec_of[i];
            if (b.done[s] == 0) {
                const double al = b.alpha[s];
                dvec4 xv = x[i], rv = r[i];
                const dvec4 pv = p[i], qv = q[i];
                xv.x += al * pv.x;
                xv.y += al * pv.y;
                xv.z += al * pv.z;
                rv.x -= al * qv.x;
                rv.y -= al * qv.y;
                rv.z -= al * qv.z;
                const dvec4 zv = pinv_apply(P, b.n, i, rv);
                x[i] = xv;
                r[i] = rv;
                z[i] = zv;
                v[0] = rv.x * zv.x + rv.y * zv.y + rv.z * zv.z;
                v[1] = rv.x * rv.x + rv.y * rv.y + rv.z * rv.z;
            }
        }
        seg_chunk<2>(b, sh, ch, s, v);
    }
    seg_finish<2, true>(b, sh, [b](int sp) { return b.done[sp] == 0; }, [b](int sp, const double *t) {
        b.rz_old[sp] = b.rz[sp];
        b.rz[sp] = t[0];
        b.rr[sp] = t[1];
        b.beta[sp] = (b.rz_old[sp] != 0.0) ? t[0] / b.rz_old[sp] : 0.0;
        b.it[sp] += 1;
        if (t[1] <= b.tol2[sp])
            b.done[sp] = 1;
        else if (!(t[1] == t[1]))
            b.done[sp] = 3;
        else if (b.it[sp] >= b.maxit)
            b.done[sp] = 2;
        else if (t[1] < b.upd_delta2 * b.rr_max[sp])
            b.upd[sp] = 1;
        if (t[1] > b.rr_max[sp])
            b.rr_max[sp] = t[1];
    });
}

// p = z + beta p for running specimens
__global__ void __launch_bounds__(TPB) k_bcg_p(BatchCg b, const dvec4 *z, dvec4 *p)
{
    if (*b.all_done)
        return;
    const ChunkList L = active_chunks(b);
    for (int k = blockIdx.x; k < L.count; k += gridDim.x) {
        const int i = L.at(k) * TPB + threadIdx.x;
        if (i < b.n) {
            const int s = b.spec_of[i];
            if (b.done[s] == 0) {
                const double be = b.beta[s];
                dvec4 pv = p[i];
                const dvec4 zv = z[i];
                pv.x = zv.x + be * pv.x;
                pv.y = zv.y + be * pv.y;
                pv.z = zv.z + be * pv.z;
                p[i] = pv;
            }
        }
    }
}

// Reliable update (FP32 matrix), issued after every chunk of iterations:
// rtrue = bs - K32 x with FP64 products and sums (the refinement-residual
// kernel, on the rows of the specimens concerned).  For each specimen that
// asked for it (its recursive residual fell by the factor inner_rtol since the
// last update) or whose recursive residual met the tolerance: finished
// (done = 6) if the true residual meets the tolerance, else r = rtrue,
// z = P^-1 r, and the iteration continues with the same search direction.
// A specimen stops at done = 2 after refine_maxiter updates.
__device__ __forceinline__ bool due(const BatchCg &b, int s)
{
    const int d = b.done[s];
    return (d == 0 && b.upd[s]) || d == 1;
}

__global__ void __launch_bounds__(TPB) k_bcg_reliable(BatchCg b, const dvec4 *rtrue, const uint8_t *mask,
                                                      const double *P, dvec4 *r, dvec4 *z)
{
    __shared__ SegShared<2> sh;
    const ChunkList L = all_chunks(b);
    for (int k = blockIdx.x; k < L.count; k += gridDim.x) {
        const int ch = L.at(k), i = ch * TPB + threadIdx.x;
        double v[2] = {0.0, 0.0};
        int s = -1;
        if (i < b.n) {
            s = b.spec_of[i];
            if (due(b, s)) {
                const dvec4 rt = bmask4(rtrue[i], mask[i]);
                const dvec4 zv = pinv_apply(P, b.n, i, rt);
                r[i] = rt;
                z[i] = zv;
                v[0] = rt.x * zv.x + rt.y * zv.y + rt.z * zv.z;
                v[1] = rt.x * rt.x + rt.y * rt.y + rt.z * rt.z;
            }
        }
        seg_chunk<2>(b, sh, ch, s, v);
    }
    seg_finish<2, true>(b, sh, [b](int sp) { return due(b, sp); }, [b](int sp, const double *t) {
        b.nrel[sp] += 1;
        b.upd[sp] = 0;
        if (t[1] <= b.tol2[sp]) {
            b.done[sp] = 6;
            return;
        }
        if (!(t[1] == t[1])) {
            b.done[sp] = 3;
            return;
        }
        b.rz[sp] = t[0];
        b.rr[sp] = t[1];
        b.rr_max[sp] = t[1];
        b.done[sp] = (b.it[sp] >= b.maxit || b.nrel[sp] >= b.maxrel) ? 2 : 0;
    });
}

// du = x / bscale (0 for stopped specimens, whose x stayed 0)
__global__ void k_bcg_finish(BatchCg b, const dvec4 *x, dvec4 *du)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= b.n)
        return;
    const int s = b.spec_of[i];
    const double sc = b.active[s] ? b.bscale[s] : 0.0;
    const dvec4 v = x[i];
    du[i] = (sc > 0.0) ? make_dvec4(v.x / sc, v.y / sc, v.z / sc, 0.0) : make_dvec4(0.0, 0.0, 0.0, 0.0);
}

struct DispBCB {
    int type;
    int comp;  // 0 x, 1 y, 2 z, -1 none
    double step;
};

// setDispBC (src/boundary.c:12-45) with a list of nbd entries per specimen
__global__ void k_disp_bc_batch(int n, const int *spec_of, const int *type, dvec4 *xyz, uint8_t *mask,
                                const DispBCB *bcs, int nbd)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    const DispBCB *L = bcs + (size_t)spec_of[i] * nbd;
    dvec4 x = xyz[i];
    uint8_t m = mask[i];
    const int t = type[i];
    for (int k = 0; k < nbd; k++) {
        if (t != L[k].type || L[k].comp < 0)
            continue;
        if (L[k].comp == 0)
            x.x += L[k].step;
        else if (L[k].comp == 1)
            x.y += L[k].step;
        else
            x.z += L[k].step;
        m &= (uint8_t) ~(1u << L[k].comp);
    }
    xyz[i] = x;
    mask[i] = m;
}

}  // namespace

// persistent grid of the batch kernels: 8 blocks of BATCH_TPB threads per SM
// (full occupancy; a block walks several chunks), capped by the chunk count
static int grid_of(const Ctx &c)
{
    const int sms = c.tune.sms > 0 ? c.tune.sms : 152;
    return std::max(1, std::min(8 * sms, c.bcg.nchunk));
}

void launch_bnorm(Ctx &c)
{
    k_bnorm<<<grid_of(c), TPB, 0, c.stream>>>(c.bcg, c.res, c.Pin, c.mask, c.bh.norms_d);
}

void launch_bcg_init(Ctx &c, const dvec4 *b)
{
    k_bcg_init<<<grid_of(c), TPB, 0, c.stream>>>(c.bcg, b, c.mask, c.Pinv_d, c.x_d, c.r_d, c.z_d, c.p_d,
                                                c.bh.bs, c.opts.cg_rtol);
}

void launch_bcg_compact(Ctx &c)
{
    cudaMemsetAsync(c.bcg.n_act, 0, sizeof(int), c.stream);
    k_bcg_compact<<<(c.bcg.nchunk + 255) / 256, 256, 0, c.stream>>>(c.bcg);
}

void launch_bcg_iter(Ctx &c, bool k32)
{
    launch_spmv_batch(c, c.p_d, c.q_d, k32);
    const int g = grid_of(c);
    k_bcg_alpha<<<g, TPB, 0, c.stream>>>(c.bcg, c.p_d, c.q_d);
    k_bcg_update<<<g, TPB, 0, c.stream>>>(c.bcg, c.Pinv_d, c.x_d, c.r_d, c.z_d, c.p_d, c.q_d);
    k_bcg_p<<<g, TPB, 0, c.stream>>>(c.bcg, c.z_d, c.p_d);
}

void launch_bcg_reliable(Ctx &c)
{
    launch_refine_batch(c, c.x_d, c.bh.bs, c.q_d);
    k_bcg_reliable<<<grid_of(c), TPB, 0, c.stream>>>(c.bcg, c.q_d, c.mask, c.Pinv_d, c.r_d, c.z_d);
}

void launch_bcg_finish(Ctx &c)
{
    k_bcg_finish<<<c.bcg.nchunk, TPB, 0, c.stream>>>(c.bcg, c.x_d, c.du);
}

int launch_disp_bc_batch(Ctx &c, int nbd, const lpm_disp_bc *d)
{
    const size_t cnt = (size_t)c.nspec * nbd;
    if (cnt == 0)
        return LPM_OK;
    std::vector<DispBCB> h(cnt);
    for (size_t k = 0; k < cnt; k++) {
        h[k].type = d[k].type;
        h[k].comp = d[k].flag == 'x' ? 0 : (d[k].flag == 'y' ? 1 : (d[k].flag == 'z' ? 2 : -1));
        h[k].step = d[k].step;
    }
    if (c.bh.bc_cap < cnt) {
        if (c.bh.bc_d)
            cudaFree(c.bh.bc_d);
        c.bh.bc_d = nullptr;
        c.bh.bc_cap = 0;
        LPM_CUDA(cudaMalloc(&c.bh.bc_d, cnt * sizeof(DispBCB)));
        c.bh.bc_cap = cnt;
    }
    LPM_CUDA(cudaMemcpyAsync(c.bh.bc_d, h.data(), cnt * sizeof(DispBCB), cudaMemcpyHostToDevice, c.stream));
    k_disp_bc_batch<<<c.bcg.nchunk, TPB, 0, c.stream>>>(c.n, c.bcg.spec_of, c.type, c.xyz, c.mask,
                                                       (const DispBCB *)c.bh.bc_d, nbd);
    // h is pageable host memory and must outlive the copy
    LPM_CUDA(cudaStreamSynchronize(c.stream));
    return LPM_OK;
}

}  // namespace lpm
