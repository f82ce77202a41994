// FP64 bond-force kernels: stretches, elastic force, elastic predictor, J2
// return mapping, crystal-plasticity return mapping, averaged bond force,
// internal force, stress and residual.
//
// This file is compiled with -fmad=false and every expression keeps the
// reference's evaluation order, so for the same inputs the results are
// bit-identical to the reference's FP64 CPU code (sqrt and division are
// IEEE-rounded on both sides).  The crystal-plasticity kernel calls pow,
// cosh and tanh, whose last bits differ from the host C library.
//
// One thread per particle; bond arrays are slot-major [NN][n] so each bond
// slot is a coalesced load across the warp.  The reference's per-particle
// evaluation (src/constitutive.c:466-686) recomputes every neighbour's
// stretches inside each particle's call; the values it computes for a given
// particle depend only on that particle's data, so the same numbers come out
// of three race-free sweeps: return map + new stretches (k_j2 / k_cp), then
// averaged force + internal force + stress + residual (k_final).
#include <cstdio>
#include "lpm_internal.h"

namespace lpm {

constexpr int TPB = 128;

struct ForceArgs {
    int n;
    const dvec4 *xyz, *xyz_temp;
    const int *nbr;
    const int8_t *shell, *rev, *nbv;
    const double *L0, *Kn, *Tv, *oppv;
    double *csx, *csy, *csz;
    double *dL;
    double2 *S, *T;
    double *F;
    const double *F_prev;
    double *ddL;
    double2 *dS, *dT;
    dvec4 *Pin;
    const dvec4 *Pex;
    dvec4 *res;
    const uint8_t *mask;
    double *stress;
    double *partials;
    unsigned *counter;
    double *norms;
    // state
    const double *dLp_c;
    double *dLp_t;
    const double *alpha_c, *beta_c;
    double *alpha_t, *beta_t, *dlambda;
    const double *G, *sy, *H;
    double xi;
    int *status;
    int *pl_flag;
    // damage_broken / damage_w [NN][n]; null while the damage stage is off
    const double *brk, *dw;
};

static ForceArgs make_args(Ctx &c)
{
    ForceArgs a;
    a.n = c.n;
    a.xyz = c.xyz;
    a.xyz_temp = c.xyz_temp;
    a.nbr = c.nbr;
    a.shell = c.shell;
    a.rev = c.rev;
    a.nbv = c.nbv;
    a.L0 = c.L0;
    a.Kn = c.Kn;
    a.Tv = c.Tv;
    a.oppv = c.oppv;
    a.csx = c.csx;
    a.csy = c.csy;
    a.csz = c.csz;
    a.dL = c.dL;
    a.S = c.S;
    a.T = c.T;
    a.F = c.F;
    a.F_prev = c.F_prev;
    a.ddL = c.ddL;
    a.dS = c.dS;
    a.dT = c.dT;
    a.Pin = c.Pin;
    a.Pex = c.Pex;
    a.res = c.res;
    a.mask = c.mask;
    a.stress = c.stress;
    a.partials = c.partials;
    a.counter = c.counter;
    a.norms = c.norms;
    a.dLp_c = c.dLp[0];
    a.dLp_t = c.dLp[2];
    a.alpha_c = c.alpha[0];
    a.beta_c = c.beta[0];
    a.alpha_t = c.alpha[2];
    a.beta_t = c.beta[2];
    a.dlambda = c.dlambda;
    a.G = c.G;
    a.sy = c.sy;
    a.H = c.Hh;
    a.xi = c.xi;
    a.status = c.status;
    a.pl_flag = c.pl_flag;
    a.brk = c.dmg.brk;
    a.dw = c.dmg.dw;
    return a;
}

static inline int grid_for(int n) { return (n + TPB - 1) / TPB; }

__device__ __forceinline__ double bond_length(dvec4 a, dvec4 b, double &dx, double &dy, double &dz)
{
    dx = a.x - b.x;
    dy = a.y - b.y;
    dz = a.z - b.z;
    return sqrt(dx * dx + dy * dy + dz * dz);
}

// Deterministic two-level sum of NV values over the grid: block tree sums into
// partials[k*gridDim + block], the last block to finish adds the partials in
// a fixed order and writes out[k].  Must be reached by every thread.
template <int NV>
__device__ void grid_sum(double (&v)[NV], double *partials, unsigned *counter, double *out)
{
    __shared__ double red[NV][TPB / 32];
    __shared__ bool last;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < NV; k++) {
        double s = v[k];
        for (int o = 16; o > 0; o >>= 1)
            s += __shfl_xor_sync(0xffffffffu, s, o);
        if (lane == 0)
            red[k][wid] = s;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < NV; k++) {
            double s = 0.0;
            for (int w = 0; w < TPB / 32; w++)
                s += red[k][w];
            partials[(size_t)k * gridDim.x + blockIdx.x] = s;
        }
        __threadfence();
        unsigned t = atomicAdd(counter, 1u);
        last = (t == gridDim.x - 1);
    }
    __syncthreads();
    if (!last)
        return;
    __threadfence();
#pragma unroll
    for (int k = 0; k < NV; k++) {
        double s = 0.0;
        for (unsigned b = threadIdx.x; b < gridDim.x; b += TPB)
            s += __ldcg(&partials[(size_t)k * gridDim.x + b]);
        for (int o = 16; o > 0; o >>= 1)
            s += __shfl_xor_sync(0xffffffffu, s, o);
        if (lane == 0)
            red[k][wid] = s;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < NV; k++) {
            double s = 0.0;
            for (int w = 0; w < TPB / 32; w++)
                s += red[k][w];
            out[k] = s;
        }
        *counter = 0u;
    }
}

// updateRR (src/stiffness.c:519-534) for particle i plus the squared norms of
// the residual and of the reaction (Pin on constrained DOFs).
__device__ __forceinline__ void residual_epilogue(const ForceArgs &a, int i, bool valid, double p0,
                                                  double p1, double p2)
{
    double v[2] = {0.0, 0.0};
    if (valid) {
        a.Pin[i] = make_dvec4(p0, p1, p2, 0.0);
        const dvec4 pe = a.Pex[i];
        const uint8_t m = a.mask[i];
        const double m0 = (m & 1) ? 1.0 : 0.0, m1 = (m & 2) ? 1.0 : 0.0, m2 = (m & 4) ? 1.0 : 0.0;
        const double r0 = m0 * (pe.x - p0), r1 = m1 * (pe.y - p1), r2 = m2 * (pe.z - p2);
        a.res[i] = make_dvec4(r0, r1, r2, 0.0);
        v[0] = r0 * r0 + r1 * r1 + r2 * r2;
        v[1] = ((m & 1) ? 0.0 : p0 * p0) + ((m & 2) ? 0.0 : p1 * p1) + ((m & 4) ? 0.0 : p2 * p2);
    }
    grid_sum<2>(v, a.partials, a.counter, a.norms);
}

// computeStress (src/lpm_basic.c:58-98): stress sums of particle i from its
// bond forces; w = (opp_flag / particle_volume) * distance_initial * F.
__device__ __forceinline__ void stress_add(double (&st)[6], double w, double cx, double cy, double cz)
{
    st[0] += w * cx * cx;
    st[1] += w * cy * cy;
    st[2] += w * cz * cz;
    st[3] += w * cy * cz;
    st[4] += w * cx * cz;
    st[5] += w * cx * cy;
}

__device__ __forceinline__ void stress_store(const ForceArgs &a, int i, const double (&st)[6])
{
#pragma unroll
    for (int k = 0; k < 6; k++)
        a.stress[(size_t)k * a.n + i] = st[k];
}

// computedL (src/lpm_basic.c:252-291) / first loop of src/constitutive.c:241-261:
// elastic stretch dL = (|xi - xj| - L0) - dLp, shell sums, unit vectors.
__global__ void k_stretch(ForceArgs a, const double *dLp, int store_cs)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n)
        return;
    const int n = a.n, nbi = a.nbv[i];
    const dvec4 xi = a.xyz[i];
    double S0 = 0, S1 = 0, T0 = 0, T1 = 0;
    for (int j = 0; j < nbi; j++) {
        const size_t b = (size_t)j * n + i;
        const int p = a.nbr[b];
        double dx, dy, dz;
        const double dis = bond_length(xi, a.xyz[p], dx, dy, dz);
        double v = dis - a.L0[b];
        v -= dLp[b];
        if (a.brk)
            v *= a.brk[b];  // damage_broken
        a.dL[b] = v;
        if (a.shell[b] == 0) {
            S0 += v;
            T0 += a.Tv[b] * v;
        } else {
            S1 += v;
            T1 += a.Tv[b] * v;
        }
        if (store_cs) {
            a.csx[b] = dx / dis;
            a.csy[b] = dy / dis;
            a.csz[b] = dz / dis;
        }
    }
    a.S[i] = make_double2(S0, S1);
    a.T[i] = make_double2(T0, T1);
}

// computeBondForceElastic force loop (src/constitutive.c:264-279), plmode 6.
__global__ void k_elastic(ForceArgs a)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const bool valid = i < a.n;
    double p0 = 0.0, p1 = 0.0, p2 = 0.0, st[6] = {0, 0, 0, 0, 0, 0};
    if (valid) {
        const int n = a.n, nbi = a.nbv[i];
        const double2 Si = a.S[i], Ti = a.T[i];
        for (int j = 0; j < nbi; j++) {
            const size_t b = (size_t)j * n + i;
            const int p = a.nbr[b];
            const double2 Sp = a.S[p], Tp = a.T[p];
            const bool s0 = a.shell[b] == 0;
            double f = 2.0 * a.Kn[b] * a.dL[b] + 0.5 * ((s0 ? Ti.x : Ti.y) + (s0 ? Tp.x : Tp.y)) +
                       0.5 * a.Tv[b] * ((s0 ? Si.x : Si.y) + (s0 ? Sp.x : Sp.y));
            if (a.brk)
                f *= a.brk[b];  // damage_broken
            a.F[b] = f;
            const double cx = a.csx[b], cy = a.csy[b], cz = a.csz[b];
            p0 += cx * f;
            p1 += cy * f;
            p2 += cz * f;
            stress_add(st, a.oppv[b] * a.L0[b] * f, cx, cy, cz);
        }
        stress_store(a, i, st);
    }
    residual_epilogue(a, i, valid, p0, p1, p2);
}

// computeBondForceIncrementalUpdating (src/constitutive.c:167-225), plmode 4:
// first sweep, stretch increments from xyz_temp to xyz and their shell sums.
__global__ void k_pred1(ForceArgs a)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n)
        return;
    const int n = a.n, nbi = a.nbv[i];
    const dvec4 x1 = a.xyz[i], x0 = a.xyz_temp[i];
    double S0 = 0, S1 = 0, T0 = 0, T1 = 0;
    for (int j = 0; j < nbi; j++) {
        const size_t b = (size_t)j * n + i;
        const int p = a.nbr[b];
        double dx, dy, dz;
        const double d0 = bond_length(x0, a.xyz_temp[p], dx, dy, dz);
        const double d1 = bond_length(x1, a.xyz[p], dx, dy, dz);
        const double v = (a.brk ? a.brk[b] : 1.0) * (d1 - d0);  // damage_broken
        a.ddL[b] = v;
        if (a.shell[b] == 0) {
            S0 += v;
            T0 += a.Tv[b] * v;
        } else {
            S1 += v;
            T1 += a.Tv[b] * v;
        }
    }
    a.dS[i] = make_double2(S0, S1);
    a.dT[i] = make_double2(T0, T1);
}

// second sweep: F = F_temp + elastic increment, internal force with the
// unit vectors of the previous evaluation (src/constitutive.c:206-221).
__global__ void k_pred2(ForceArgs a)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const bool valid = i < a.n;
    double p0 = 0.0, p1 = 0.0, p2 = 0.0, st[6] = {0, 0, 0, 0, 0, 0};
    if (valid) {
        const int n = a.n, nbi = a.nbv[i];
        const double2 Si = a.dS[i], Ti = a.dT[i];
        for (int j = 0; j < nbi; j++) {
            const size_t b = (size_t)j * n + i;
            const int p = a.nbr[b];
            const double2 Sp = a.dS[p], Tp = a.dT[p];
            const bool s0 = a.shell[b] == 0;
            double f = a.F_prev[b] + 2.0 * a.Kn[b] * a.ddL[b] + 0.5 * ((s0 ? Ti.x : Ti.y) + (s0 ? Tp.x : Tp.y)) +
                       0.5 * a.Tv[b] * ((s0 ? Si.x : Si.y) + (s0 ? Sp.x : Sp.y));
            if (a.brk)
                f *= a.brk[b];  // damage_broken
            a.F[b] = f;
            const double cx = a.csx[b], cy = a.csy[b], cz = a.csz[b];
            p0 += cx * f;
            p1 += cy * f;
            p2 += cz * f;
            stress_add(st, a.oppv[b] * a.L0[b] * f, cx, cy, cz);
        }
        stress_store(a, i, st);
    }
    residual_epilogue(a, i, valid, p0, p1, p2);
}

// J2 radial return (src/constitutive.c:494-621) for particle i followed by the
// re-summed dilatation with the updated plastic stretch (:624-645).
__global__ void __launch_bounds__(TPB) k_j2(ForceArgs a)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n)
        return;
    const int n = a.n, nbi = a.nbv[i];
    const dvec4 xi = a.xyz[i];
    double e[LPM_NN];
    double S0 = 0, S1 = 0, T0 = 0, T1 = 0;
#pragma unroll
    for (int j = 0; j < LPM_NN; j++) {
        e[j] = 0.0;
        if (j < nbi) {
            const size_t b = (size_t)j * n + i;
            double dx, dy, dz;
            const double dis = bond_length(xi, a.xyz[a.nbr[b]], dx, dy, dz);
            e[j] = dis - a.L0[b];
            double v = e[j];
            v -= a.dLp_c[b];
            if (a.brk)
                v *= a.brk[b];  // damage_broken
            if (a.shell[b] == 0) {
                S0 += v;
                T0 += a.Tv[b] * v;
            } else {
                S1 += v;
                T1 += a.Tv[b] * v;
            }
            a.csx[b] = dx / dis;
            a.csy[b] = dy / dis;
            a.csz[b] = dz / dis;
        }
    }
    // trial stress from bond forces with the particle's own shell sums
    double st[6] = {0, 0, 0, 0, 0, 0};
#pragma unroll
    for (int j = 0; j < LPM_NN; j++) {
        if (j < nbi) {
            const size_t b = (size_t)j * n + i;
            double v = e[j];
            v -= a.dLp_c[b];
            if (a.brk)
                v *= a.brk[b];  // damage_broken
            const bool s0 = a.shell[b] == 0;
            double fij = 2.0 * a.Kn[b] * v + (s0 ? T0 : T1) + a.Tv[b] * (s0 ? S0 : S1);
            if (a.dw)
                fij *= a.dw[b];  // damage_w
            stress_add(st, a.oppv[b] * a.L0[b] * fij, a.csx[b], a.csy[b], a.csz[b]);
        }
    }
    const double temp = 1.0 / 3.0 * (st[0] + st[1] + st[2]);
    for (int k = 0; k < 3; k++)
        st[k] -= temp;
    double beta[6];
#pragma unroll
    for (int k = 0; k < 6; k++) {
        beta[k] = a.beta_c[(size_t)k * n + i];
        st[k] -= beta[k];
    }
    double seq = 0.0;
#pragma unroll
    for (int k = 0; k < 6; k++) {
        if (k < 3)
            seq += st[k] * st[k];
        else
            seq += 2.0 * st[k] * st[k];
    }
    seq = sqrt(3.0 / 2.0 * seq);
    double alpha = a.alpha_c[i], dlam = 0.0;
    const double Hh = a.H[i];
    const double yf = seq - (a.sy[i] + (1.0 - a.xi) * Hh * alpha);
    if (yf > 0.0) {
        dlam = yf / (3 * a.G[i] + Hh);
        a.pl_flag[i] = 1;  // pl_flag (src/constitutive.c:594)
    }
    alpha += dlam;
    double dpl[6] = {0, 0, 0, 0, 0, 0};
#pragma unroll
    for (int k = 0; k < 6; k++)
        if (fabs(seq) > 1e-6) {
            dpl[k] = dlam * 1.5 * st[k] / seq;
            beta[k] += 2. / 3. * a.xi * Hh * dpl[k];
        }
    // incremental plastic stretch, new stretches and shell sums
    S0 = 0, S1 = 0, T0 = 0, T1 = 0;
#pragma unroll
    for (int j = 0; j < LPM_NN; j++) {
        const size_t b = (size_t)j * n + i;
        double add = 0.0;
        if (j < nbi) {
            const double cx = a.csx[b], cy = a.csy[b], cz = a.csz[b];
            add = a.L0[b] * (dpl[0] * cx * cx + dpl[1] * cy * cy + dpl[2] * cz * cz + 2 * dpl[3] * cy * cz +
                             2 * dpl[4] * cx * cz + 2 * dpl[5] * cx * cy);
            if (a.brk)
                add *= a.brk[b];  // damage_broken
        }
        const double lp = (a.brk ? a.brk[b] : 1.0) * (a.dLp_c[b] + add);
        a.dLp_t[b] = lp;
        if (j < nbi) {
            double v = e[j];
            v -= lp;
            if (a.brk)
                v *= a.brk[b];  // damage_broken
            a.dL[b] = v;
            if (a.shell[b] == 0) {
                S0 += v;
                T0 += a.Tv[b] * v;
            } else {
                S1 += v;
                T1 += a.Tv[b] * v;
            }
        }
    }
    a.S[i] = make_double2(S0, S1);
    a.T[i] = make_double2(T0, T1);
#pragma unroll
    for (int k = 0; k < 6; k++)
        a.beta_t[(size_t)k * n + i] = beta[k];
    a.alpha_t[i] = alpha;
    a.dlambda[i] = dlam;
}

// Averaged bond force, internal force, stress and residual
// (src/constitutive.c:647-667, src/lpm_basic.c:53-98, src/stiffness.c:519-534).
__global__ void k_final(ForceArgs a)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const bool valid = i < a.n;
    double p0 = 0.0, p1 = 0.0, p2 = 0.0, st[6] = {0, 0, 0, 0, 0, 0};
    if (valid) {
        const int n = a.n, nbi = a.nbv[i];
        const double2 Si = a.S[i], Ti = a.T[i];
        for (int j = 0; j < nbi; j++) {
            const size_t b = (size_t)j * n + i;
            const int p = a.nbr[b];
            const double2 Sp = a.S[p], Tp = a.T[p];
            const bool s0 = a.shell[b] == 0;
            const int rv = a.rev[b];  // always >= 0 for a symmetric bond list
            const double dla = 0.5 * (a.dL[b] + (rv >= 0 ? a.dL[(size_t)rv * n + p] : a.dL[b]));
            double f = 2.0 * a.Kn[b] * dla + 0.5 * ((s0 ? Ti.x : Ti.y) + (s0 ? Tp.x : Tp.y)) +
                       0.5 * a.Tv[b] * ((s0 ? Si.x : Si.y) + (s0 ? Sp.x : Sp.y));
            if (a.dw)
                f *= a.dw[b];  // damage_w
            a.F[b] = f;
            const double cx = a.csx[b], cy = a.csy[b], cz = a.csz[b];
            p0 += cx * f;
            p1 += cy * f;
            p2 += cz * f;
            stress_add(st, a.oppv[b] * a.L0[b] * f, cx, cy, cz);
        }
        stress_store(a, i, st);
    }
    residual_epilogue(a, i, valid, p0, p1, p2);
}

// updateCrack (src/constitutive.c:1399-1434): intact-bond count, damage
// picture, bond forces scaled by w and the internal force re-summed, then
// updateRR and its norms.  Particles left without bonds are not fixed here:
// their internal force is zero, so with no external force their residual is
// zero and the solve leaves them in place, as fix_index does.
__global__ void k_crack(ForceArgs a, int8_t *nbc, double *dvis)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const bool valid = i < a.n;
    double p0 = 0.0, p1 = 0.0, p2 = 0.0;
    if (valid) {
        const int n = a.n, nbi = a.nbv[i];
        int cnt = nbi;
        double vis = 0.0;
        for (int j = 0; j < nbi; j++) {
            const size_t b = (size_t)j * n + i;
            if (a.brk[b] <= 1e-6)
                cnt -= 1;
            vis += a.brk[b];
            const double f = a.F[b] * a.dw[b];
            a.F[b] = f;
            p0 += a.csx[b] * f;
            p1 += a.csy[b] * f;
            p2 += a.csz[b] * f;
        }
        nbc[i] = (int8_t)cnt;
        dvis[i] = 1 - vis / nbi;
    }
    residual_epilogue(a, i, valid, p0, p1, p2);
}

__global__ void k_add_du(int n, dvec4 *xyz, const dvec4 *du)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    dvec4 x = xyz[i];
    const dvec4 d = du[i];
    x.x += d.x;
    x.y += d.y;
    x.z += d.z;
    xyz[i] = x;
}

struct DispBCList {
    int n;
    int type[16];
    int comp[16];
    double step[16];
};

// setDispBC (src/boundary.c:12-45): move constrained coordinates by the step
// and clear their free-DOF bits.
__global__ void k_disp_bc(int n, const int *type, dvec4 *xyz, uint8_t *mask, DispBCList L)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    dvec4 x = xyz[i];
    uint8_t m = mask[i];
    const int t = type[i];
    for (int k = 0; k < L.n; k++) {
        if (t != L.type[k] || L.comp[k] < 0)
            continue;
        if (L.comp[k] == 0)
            x.x += L.step[k];
        else if (L.comp[k] == 1)
            x.y += L.step[k];
        else
            x.z += L.step[k];
        m &= (uint8_t)~(1u << L.comp[k]);
    }
    xyz[i] = x;
    mask[i] = m;
}

struct ForceBCList {
    int n;
    int type[16];
    double f[16][3];
    double cnt[16];
};

// setForceBC (src/boundary.c:48-70)
__global__ void k_force_bc(int n, const int *type, dvec4 *Pex, ForceBCList L)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    dvec4 pe = Pex[i];
    const int t = type[i];
    for (int k = 0; k < L.n; k++) {
        if (t != L.type[k])
            continue;
        pe.x += L.f[k][0] / L.cnt[k];
        pe.y += L.f[k][1] / L.cnt[k];
        pe.z += L.f[k][2] / L.cnt[k];
    }
    Pex[i] = pe;
}

void launch_stretch(Ctx &c, const double *dLp, bool store_cs)
{
    ForceArgs a = make_args(c);
    k_stretch<<<grid_for(c.n), TPB, 0, c.stream>>>(a, dLp, store_cs ? 1 : 0);
}

void launch_crack(Ctx &c)
{
    ForceArgs a = make_args(c);
    k_crack<<<grid_for(c.n), TPB, 0, c.stream>>>(a, c.dmg.nbc, c.dmg.dvis);
}

void launch_elastic_force(Ctx &c)
{
    ForceArgs a = make_args(c);
    k_stretch<<<grid_for(c.n), TPB, 0, c.stream>>>(a, c.dLp[0], 1);
    k_elastic<<<grid_for(c.n), TPB, 0, c.stream>>>(a);
}

void launch_predictor(Ctx &c)
{
    ForceArgs a = make_args(c);
    k_pred1<<<grid_for(c.n), TPB, 0, c.stream>>>(a);
    k_pred2<<<grid_for(c.n), TPB, 0, c.stream>>>(a);
}

void launch_j2(Ctx &c)
{
    ForceArgs a = make_args(c);
    k_j2<<<grid_for(c.n), TPB, 0, c.stream>>>(a);
}

void launch_final_force(Ctx &c)
{
    ForceArgs a = make_args(c);
    k_final<<<grid_for(c.n), TPB, 0, c.stream>>>(a);
}

void launch_residual(Ctx &c) { (void)c; }

void launch_add_du(Ctx &c) { k_add_du<<<grid_for(c.n), TPB, 0, c.stream>>>(c.n, c.xyz, c.du); }

void launch_apply_disp_bc(Ctx &c, int nbd, const lpm_disp_bc *d)
{
    for (int s = 0; s < nbd; s += 16) {
        DispBCList L;
        L.n = nbd - s < 16 ? nbd - s : 16;
        for (int k = 0; k < L.n; k++) {
            const lpm_disp_bc &b = d[s + k];
            L.type[k] = b.type;
            L.comp[k] = b.flag == 'x' ? 0 : (b.flag == 'y' ? 1 : (b.flag == 'z' ? 2 : -1));
            L.step[k] = b.step;
        }
        k_disp_bc<<<grid_for(c.n), TPB, 0, c.stream>>>(c.n, c.type, c.xyz, c.mask, L);
    }
}

void launch_apply_force_bc(Ctx &c, int nbf, const lpm_force_bc *f, const int *counts)
{
    for (int s = 0; s < nbf; s += 16) {
        ForceBCList L;
        L.n = nbf - s < 16 ? nbf - s : 16;
        for (int k = 0; k < L.n; k++) {
            const lpm_force_bc &b = f[s + k];
            L.type[k] = b.type;
            L.f[k][0] = b.step1;
            L.f[k][1] = b.step2;
            L.f[k][2] = b.step3;
            L.cnt[k] = (double)counts[s + k];
        }
        k_force_bc<<<grid_for(c.n), TPB, 0, c.stream>>>(c.n, c.type, c.Pex, L);
    }
}

}  // namespace lpm
