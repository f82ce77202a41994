// Reverse mode of one J2 force evaluation (plmode 0 with isotropic hardening)
// and the vector kernels of the adjoint solve and of the Anderson-accelerated
// Newton loop.
//
// The force evaluation maps (positions u, converged state q = (dLp, alpha),
// material theta = per-particle C11, C12, C44 via Kn/Tv and G = C44, yield
// stress, hardening) to the internal force Pin and the new state
// q' = (dLp', alpha').  For every particle i it is
//   e_ij = |x_i - x_j| - L0_ij,  c_ij = (x_i - x_j)/|x_i - x_j|
//   trial: v_ij = e_ij - dLp_ij,  S_i^s = sum v,  T_i^s = sum Tv v
//          f_ij = 2 Kn v + T_i^s + Tv S_i^s,  sigma_i = sum w_ij f_ij c c (w = oppv L0)
//          s = dev(sigma) - beta,  seq = sqrt(3/2 s:s),  yf = seq - (sy + H alpha)
//          dlam = yf / (3G + H) if yf > 0,  dpl = dlam 3/2 s / seq
//   return: dLp'_ij = dLp_ij + L0 (dpl : c c),  alpha' = alpha + dlam
//   final:  v'_ij = e_ij - dLp'_ij, sums S', T' as above,
//          F_ij = 2 Kn (v'_ij + v'_ji)/2 + (T'_i + T'_j)/2 + Tv (S'_i + S'_j)/2
//          Pin_i = sum_j c_ij F_ij
// (src/constitutive.c:466-686 and the GPU forward in k_force.cu).
//
// k_vjp takes cotangents (Pbar per particle, mu_dLp per bond, mu_alpha per
// particle) and, per particle, differentiates its own part of this map in
// reverse; every quantity that couples two particles is handled from both
// ends through the reverse bond slot, so there are no atomics: per-bond
// results (position cotangent g_ij, Kn and Tv cotangents) are gathered by
// k_vjp_gather.
#include "lpm_internal.h"

namespace lpm {

namespace {

constexpr int ATPB = 128;

struct VjpArgs {
    int n;
    const dvec4 *xyz;
    const int *nbr;
    const int8_t *shell, *rev, *nbv;
    const double *L0, *Kn, *Tv, *oppv;
    const double *dLp_c, *alpha_c, *beta_c;
    const double *G, *sy, *H;
    // forward results at (u, q): final stretches, sums and bond forces
    const double *dL, *F;
    const double2 *S, *T;
    // cotangents
    const dvec4 *Pbar;
    const double *mu_dLp, *mu_alpha;  // may be null (zero)
    // outputs
    double *gx, *gy, *gz;            // [NN][n] position cotangent of bond ij at its owner
    double *knbar, *tvbar;           // [NN][n]
    double *dLp_bar;                 // [NN][n] cotangent of the converged plastic stretch (may be null)
    double *alpha_bar;               // [n] (may be null)
    double *Gbar, *sybar, *Hbar;     // [n] (may be null)
};

__global__ void __launch_bounds__(ATPB) k_vjp(VjpArgs a)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n)
        return;
    const int n = a.n, nbi = a.nbv[i];
    const dvec4 xi = a.xyz[i];
    double e[LPM_NN], cx[LPM_NN], cy[LPM_NN], cz[LPM_NN], dd[LPM_NN], vt[LPM_NN];
    double S0 = 0, S1 = 0, T0 = 0, T1 = 0;
#pragma unroll
    for (int j = 0; j < LPM_NN; j++) {
        e[j] = cx[j] = cy[j] = cz[j] = vt[j] = 0.0;
        dd[j] = 1.0;
        if (j < nbi) {
            const size_t b = (size_t)j * n + i;
            const dvec4 xp = a.xyz[a.nbr[b]];
            const double dx = xi.x - xp.x, dy = xi.y - xp.y, dz = xi.z - xp.z;
            const double dis = sqrt(dx * dx + dy * dy + dz * dz);
            dd[j] = dis;
            e[j] = dis - a.L0[b];
            cx[j] = dx / dis;
            cy[j] = dy / dis;
            cz[j] = dz / dis;
            vt[j] = e[j] - a.dLp_c[b];
            if (a.shell[b] == 0) {
                S0 += vt[j];
                T0 += a.Tv[b] * vt[j];
            } else {
                S1 += vt[j];
                T1 += a.Tv[b] * vt[j];
            }
        }
    }
    // trial stress and return map (recomputed)
    double st[6] = {0, 0, 0, 0, 0, 0}, f[LPM_NN];
#pragma unroll
    for (int j = 0; j < LPM_NN; j++) {
        f[j] = 0.0;
        if (j < nbi) {
            const size_t b = (size_t)j * n + i;
            const bool s0 = a.shell[b] == 0;
            f[j] = 2.0 * a.Kn[b] * vt[j] + (s0 ? T0 : T1) + a.Tv[b] * (s0 ? S0 : S1);
            const double w = a.oppv[b] * a.L0[b] * f[j];
            st[0] += w * cx[j] * cx[j];
            st[1] += w * cy[j] * cy[j];
            st[2] += w * cz[j] * cz[j];
            st[3] += w * cy[j] * cz[j];
            st[4] += w * cx[j] * cz[j];
            st[5] += w * cx[j] * cy[j];
        }
    }
    double s[6];
    const double tr3 = (st[0] + st[1] + st[2]) / 3.0;
#pragma unroll
    for (int k = 0; k < 6; k++)
        s[k] = st[k] - (k < 3 ? tr3 : 0.0) - a.beta_c[(size_t)k * n + i];
    double q2 = 0.0;
#pragma unroll
    for (int k = 0; k < 6; k++)
        q2 += (k < 3 ? 1.0 : 2.0) * s[k] * s[k];
    const double seq = sqrt(1.5 * q2);
    const double Gi = a.G[i], Hi = a.H[i], al_c = a.alpha_c[i];
    const double den = 3.0 * Gi + Hi;
    const double yf = seq - (a.sy[i] + Hi * al_c);
    const bool yielding = yf > 0.0;
    const double dlam = yielding ? yf / den : 0.0;
    const bool hasdir = fabs(seq) > 1e-6;
    double dpl[6];
#pragma unroll
    for (int k = 0; k < 6; k++)
        dpl[k] = hasdir ? dlam * 1.5 * s[k] / seq : 0.0;

    // ---- reverse of Pin_i = sum c F and of the averaged bond force
    const dvec4 Pi = a.Pbar[i];
    const double2 Si = a.S[i];
    double Fs[LPM_NN];
    double Tf0 = 0, Tf1 = 0, Sf0 = 0, Sf1 = 0;
    double gcx[LPM_NN], gcy[LPM_NN], gcz[LPM_NN];  // c-bar per bond
#pragma unroll
    for (int j = 0; j < LPM_NN; j++) {
        Fs[j] = 0.0;
        gcx[j] = gcy[j] = gcz[j] = 0.0;
        if (j < nbi) {
            const size_t b = (size_t)j * n + i;
            const int p = a.nbr[b];
            const size_t br = (size_t)a.rev[b] * n + p;
            const dvec4 Pp = a.Pbar[p];
            const double Fb_ij = cx[j] * Pi.x + cy[j] * Pi.y + cz[j] * Pi.z;
            const double Fb_ji = -(cx[j] * Pp.x + cy[j] * Pp.y + cz[j] * Pp.z);
            const double Fij = a.F[b];
            gcx[j] = Fij * Pi.x;
            gcy[j] = Fij * Pi.y;
            gcz[j] = Fij * Pi.z;
            const double2 Sp = a.S[p];
            const bool s0 = a.shell[b] == 0;
            const double dla = 0.5 * (a.dL[b] + a.dL[br]);
            a.knbar[b] = 2.0 * dla * Fb_ij;
            a.tvbar[b] = 0.5 * ((s0 ? Si.x : Si.y) + (s0 ? Sp.x : Sp.y)) * Fb_ij;
            const double tsum = 0.5 * (Fb_ij + Fb_ji);
            const double ssum = 0.5 * (a.Tv[b] * Fb_ij + a.Tv[br] * Fb_ji);
            if (s0) {
                Tf0 += tsum;
                Sf0 += ssum;
            } else {
                Tf1 += tsum;
                Sf1 += ssum;
            }
            // v'_ij enters F_ij and F_ji through their averaged stretch
            Fs[j] = a.Kn[b] * Fb_ij + a.Kn[br] * Fb_ji;
        }
    }
    // v'-bar, dLp'-bar, and the return map in reverse
    double dplb[6] = {0, 0, 0, 0, 0, 0};
    double eb[LPM_NN], dLpb[LPM_NN];
#pragma unroll
    for (int j = 0; j < LPM_NN; j++) {
        eb[j] = dLpb[j] = 0.0;
        if (j < nbi) {
            const size_t b = (size_t)j * n + i;
            const bool s0 = a.shell[b] == 0;
            const double vnb = Fs[j] + (s0 ? Sf0 : Sf1) + a.Tv[b] * (s0 ? Tf0 : Tf1);
            a.tvbar[b] += a.dL[b] * (s0 ? Tf0 : Tf1);
            const double lpb = (a.mu_dLp ? a.mu_dLp[b] : 0.0) - vnb;  // dLp'-bar
            eb[j] = vnb;
            dLpb[j] = lpb;  // dLp_c-bar (dLp' = dLp_c + ...)
            const double L = a.L0[b] * lpb;
            dplb[0] += L * cx[j] * cx[j];
            dplb[1] += L * cy[j] * cy[j];
            dplb[2] += L * cz[j] * cz[j];
            dplb[3] += L * 2.0 * cy[j] * cz[j];
            dplb[4] += L * 2.0 * cx[j] * cz[j];
            dplb[5] += L * 2.0 * cx[j] * cy[j];
            gcx[j] += L * (2.0 * dpl[0] * cx[j] + 2.0 * dpl[4] * cz[j] + 2.0 * dpl[5] * cy[j]);
            gcy[j] += L * (2.0 * dpl[1] * cy[j] + 2.0 * dpl[3] * cz[j] + 2.0 * dpl[5] * cx[j]);
            gcz[j] += L * (2.0 * dpl[2] * cz[j] + 2.0 * dpl[3] * cy[j] + 2.0 * dpl[4] * cx[j]);
        }
    }
    double alb = a.mu_alpha ? a.mu_alpha[i] : 0.0;  // alpha_c-bar
    double dlamb = alb;                              // alpha' = alpha_c + dlam
    double sb[6] = {0, 0, 0, 0, 0, 0}, seqb = 0.0;
    double Gb = 0.0, Hb = 0.0, syb = 0.0;
    if (hasdir) {
        double ds = 0.0;
#pragma unroll
        for (int k = 0; k < 6; k++) {
            dlamb += dplb[k] * 1.5 * s[k] / seq;
            sb[k] += dlam * 1.5 * dplb[k] / seq;
            ds += dplb[k] * s[k];
        }
        seqb -= dlam * 1.5 * ds / (seq * seq);
    }
    if (yielding) {
        const double yfb = dlamb / den;
        Gb -= 3.0 * dlamb * yf / (den * den);
        Hb -= dlamb * yf / (den * den);
        seqb += yfb;
        syb -= yfb;
        Hb -= yfb * al_c;
        alb -= yfb * Hi;
    }
    if (seq > 0.0) {
#pragma unroll
        for (int k = 0; k < 6; k++)
            sb[k] += seqb * 1.5 * (k < 3 ? 1.0 : 2.0) * s[k] / seq;
    }
    const double sbt = (sb[0] + sb[1] + sb[2]) / 3.0;
    double stb[6];
#pragma unroll
    for (int k = 0; k < 6; k++)
        stb[k] = sb[k] - (k < 3 ? sbt : 0.0);
    // trial stress -> trial bond forces
    double Ttb0 = 0, Ttb1 = 0, Stb0 = 0, Stb1 = 0;
#pragma unroll
    for (int j = 0; j < LPM_NN; j++) {
        if (j < nbi) {
            const size_t b = (size_t)j * n + i;
            const double W = a.oppv[b] * a.L0[b];
            const double fb = W * (stb[0] * cx[j] * cx[j] + stb[1] * cy[j] * cy[j] + stb[2] * cz[j] * cz[j] +
                                   stb[3] * cy[j] * cz[j] + stb[4] * cx[j] * cz[j] + stb[5] * cx[j] * cy[j]);
            const double Wf = W * f[j];
            gcx[j] += Wf * (2.0 * stb[0] * cx[j] + stb[4] * cz[j] + stb[5] * cy[j]);
            gcy[j] += Wf * (2.0 * stb[1] * cy[j] + stb[3] * cz[j] + stb[5] * cx[j]);
            gcz[j] += Wf * (2.0 * stb[2] * cz[j] + stb[3] * cy[j] + stb[4] * cx[j]);
            const bool s0 = a.shell[b] == 0;
            a.knbar[b] += 2.0 * vt[j] * fb;
            a.tvbar[b] += (s0 ? S0 : S1) * fb;
            if (s0) {
                Ttb0 += fb;
                Stb0 += a.Tv[b] * fb;
            } else {
                Ttb1 += fb;
                Stb1 += a.Tv[b] * fb;
            }
            f[j] = fb;  // reuse: f-bar
        }
    }
#pragma unroll
    for (int j = 0; j < LPM_NN; j++) {
        if (j < nbi) {
            const size_t b = (size_t)j * n + i;
            const bool s0 = a.shell[b] == 0;
            const double vtb = 2.0 * a.Kn[b] * f[j] + (s0 ? Stb0 : Stb1) + a.Tv[b] * (s0 ? Ttb0 : Ttb1);
            a.tvbar[b] += vt[j] * (s0 ? Ttb0 : Ttb1);
            eb[j] += vtb;
            dLpb[j] -= vtb;
            if (a.dLp_bar)
                a.dLp_bar[b] = dLpb[j];
            // position cotangent of the bond at its owner: e and c depend on x_i - x_j
            const double cdot = gcx[j] * cx[j] + gcy[j] * cy[j] + gcz[j] * cz[j];
            const double inv = 1.0 / dd[j];
            a.gx[b] = eb[j] * cx[j] + (gcx[j] - cdot * cx[j]) * inv;
            a.gy[b] = eb[j] * cy[j] + (gcy[j] - cdot * cy[j]) * inv;
            a.gz[b] = eb[j] * cz[j] + (gcz[j] - cdot * cz[j]) * inv;
        }
    }
    if (a.alpha_bar)
        a.alpha_bar[i] = alb;
    if (a.Gbar) {
        a.Gbar[i] = Gb;
        a.Hbar[i] = Hb;
        a.sybar[i] = syb;
    }
}

struct GatherArgs {
    int n, lattice;
    double radius;
    const int *nbr;
    const int8_t *shell, *rev, *nbv;
    const double *gx, *gy, *gz, *knbar, *tvbar;
    const double *Gbar, *sybar, *Hbar;  // may be null
    const double *E, *nu;               // material (for the C(E, nu) chain rule; may be null)
    dvec4 *xbar;                         // out: position cotangent
    const uint8_t *mask;                 // non-null: zero the prescribed DOFs of xbar
    double *gC;                          // [3][n] accumulated C11, C12, C44 cotangents (may be null)
    double *gE, *gnu, *gsy, *gH;         // accumulated material cotangents (may be null)
};

// x-bar_i = sum_j (g_ij - g_ji); material cotangents per particle
__global__ void k_vjp_gather(GatherArgs a)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n)
        return;
    const int n = a.n, nbi = a.nbv[i];
    double x0 = 0, x1 = 0, x2 = 0, kb[3] = {0, 0, 0};
    const bool sc = a.lattice == 2;
    for (int j = 0; j < nbi; j++) {
        const size_t b = (size_t)j * n + i;
        const int p = a.nbr[b];
        const size_t br = (size_t)a.rev[b] * n + p;
        x0 += a.gx[b] - a.gx[br];
        x1 += a.gy[b] - a.gy[br];
        x2 += a.gz[b] - a.gz[br];
        const int sh = a.shell[b];
        // SC: Kn_ij = (knt_i + knt_j)/2 (src/stiffness.c:192-200); FCC: Kn_ij = knt_i
        kb[sh] += sc ? 0.5 * (a.knbar[b] + a.knbar[br]) : a.knbar[b];
        kb[2] += sc ? 0.5 * (a.tvbar[b] + a.tvbar[br]) : a.tvbar[b];
    }
    if (a.mask) {
        const uint8_t m = a.mask[i];
        x0 = (m & 1) ? x0 : 0.0;
        x1 = (m & 2) ? x1 : 0.0;
        x2 = (m & 4) ? x2 : 0.0;
    }
    a.xbar[i] = make_dvec4(x0, x1, x2, 0.0);
    if (!a.gsy)
        return;
    // knt = radius * M * (C11, C12, C44): SC rows (1,-1,-1), (0,0,1), (0,1/18,-1/18);
    // FCC rows (0,0,r2), (r2/4,-r2/4,-r2/4), (0,r2/24,-r2/24) (src/stiffness.c:179-185, 210-216)
    const double r2 = sqrt(2.0);
    const double msc[9] = {1, -1, -1, 0, 0, 1, 0, 1.0 / 18.0, -1.0 / 18.0};
    const double mfcc[9] = {0, 0, r2, r2 / 4.0, -r2 / 4.0, -r2 / 4.0, 0, r2 / 24.0, -r2 / 24.0};
    const double *M = sc ? msc : mfcc;
    double cb[3];
    for (int k = 0; k < 3; k++)
        cb[k] = a.radius * (M[k] * kb[0] + M[3 + k] * kb[1] + M[6 + k] * kb[2]);
    cb[2] += a.Gbar[i];  // G = C44 in the return map
    a.gsy[i] += a.sybar[i];
    a.gH[i] += a.Hbar[i];
    if (a.gC)
        for (int k = 0; k < 3; k++)
            a.gC[(size_t)k * n + i] += cb[k];
    if (!a.gE)
        return;
    const double E = a.E[i], v = a.nu[i];
    const double D = (1.0 + v) * (1.0 - 2.0 * v);
    const double dD = -1.0 - 4.0 * v;
    const double dC11E = (1.0 - v) / D, dC12E = v / D, dC44E = 0.5 / (1.0 + v);
    const double dC11v = E * (-D - (1.0 - v) * dD) / (D * D);
    const double dC12v = E * (D - v * dD) / (D * D);
    const double dC44v = -0.5 * E / ((1.0 + v) * (1.0 + v));
    a.gE[i] += cb[0] * dC11E + cb[1] * dC12E + cb[2] * dC44E;
    a.gnu[i] += cb[0] * dC11v + cb[1] * dC12v + cb[2] * dC44v;
}

constexpr int RTPB = 256;

__device__ __forceinline__ double rsum(double s)
{
    for (int o = 16; o > 0; o >>= 1)
        s += __shfl_xor_sync(0xffffffffu, s, o);
    return s;
}

// deterministic grid sum of NV per-thread values: block partials, then the
// last block adds them in block order and writes out[0..NV-1]
template <int NV>
__device__ void adj_grid_sum(double (&v)[NV], double *partials, unsigned *counter, double *out)
{
    __shared__ double red[NV][RTPB / 32];
    __shared__ bool last;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < NV; k++) {
        const double s = rsum(v[k]);
        if (lane == 0)
            red[k][wid] = s;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int k = 0; k < NV; k++) {
            double s = 0.0;
            for (int w = 0; w < RTPB / 32; w++)
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
        for (unsigned b = threadIdx.x; b < gridDim.x; b += RTPB)
            s += __ldcg(&partials[(size_t)k * gridDim.x + b]);
        s = rsum(s);
        __syncthreads();
        if (lane == 0)
            red[k][wid] = s;
        __syncthreads();
        if (threadIdx.x == 0) {
            double t = 0.0;
            for (int w = 0; w < RTPB / 32; w++)
                t += red[k][w];
            out[k] = t;
        }
    }
    if (threadIdx.x == 0)
        *counter = 0u;
}

__global__ void __launch_bounds__(RTPB) k_dot(int n, const dvec4 *x, const dvec4 *y, double *partials,
                                              unsigned *counter, double *out)
{
    double v[1] = {0.0};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const dvec4 a = x[i], b = y[i];
        v[0] += a.x * b.x + a.y * b.y + a.z * b.z;
    }
    adj_grid_sum<1>(v, partials, counter, out);
}

// out[k] = <A_k, w> for k < K (K <= 16), one pass over w
struct MultiDot {
    const dvec4 *A[16];
    int K;
};
__global__ void __launch_bounds__(RTPB) k_multidot(int n, MultiDot md, const dvec4 *w, double *partials,
                                                   unsigned *counter, double *out)
{
    double v[16];
#pragma unroll
    for (int k = 0; k < 16; k++)
        v[k] = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const dvec4 b = w[i];
#pragma unroll
        for (int k = 0; k < 16; k++)
            if (k < md.K) {
                const dvec4 a = md.A[k][i];
                v[k] += a.x * b.x + a.y * b.y + a.z * b.z;
            }
    }
    adj_grid_sum<16>(v, partials, counter, out);
}

// y = a x + b y
__global__ void k_axpby(int n, double alpha, const dvec4 *x, double beta, dvec4 *y)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const dvec4 a = x[i], b = y[i];
        y[i] = make_dvec4(alpha * a.x + beta * b.x, alpha * a.y + beta * b.y, alpha * a.z + beta * b.z, 0.0);
    }
}

// reaction of writeReaction (src/data_handler.c:309-335): -sum over particles
// of type t of the internal force component comp
__global__ void __launch_bounds__(RTPB) k_reaction(int n, const int *type, int t, int comp, const dvec4 *Pin,
                                                   double *partials, unsigned *counter, double *out)
{
    double v[1] = {0.0};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        if (type[i] == t) {
            const dvec4 p = Pin[i];
            v[0] -= comp == 0 ? p.x : (comp == 1 ? p.y : p.z);
        }
    adj_grid_sum<1>(v, partials, counter, out);
}

// Pbar = w on the reaction DOFs (type t, component comp), 0 elsewhere; plus
// lam on the free DOFs when lam is non-null
__global__ void k_reaction_seed(int n, const int *type, int t, int comp, double w, const dvec4 *lam,
                                dvec4 *Pbar)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    dvec4 v = lam ? lam[i] : make_dvec4(0.0, 0.0, 0.0, 0.0);
    if (type[i] == t) {
        if (comp == 0)
            v.x += w;
        else if (comp == 1)
            v.y += w;
        else
            v.z += w;
    }
    Pbar[i] = v;
}

}  // namespace

// ---- launchers ---------------------------------------------------------------

static int agrid(int n) { return (n + ATPB - 1) / ATPB; }

void adj_vjp(Ctx &c, const dvec4 *Pbar, const double *mu_dLp, const double *mu_alpha, double *dLp_bar,
             double *alpha_bar, bool theta, AdjBuffers &w)
{
    VjpArgs a;
    a.n = c.n;
    a.xyz = c.xyz;
    a.nbr = c.nbr;
    a.shell = c.shell;
    a.rev = c.rev;
    a.nbv = c.nbv;
    a.L0 = c.L0;
    a.Kn = c.Kn;
    a.Tv = c.Tv;
    a.oppv = c.oppv;
    a.dLp_c = c.dLp[1];
    a.alpha_c = c.alpha[1];
    a.beta_c = c.beta[1];
    a.G = c.G;
    a.sy = c.sy;
    a.H = c.Hh;
    a.dL = c.dL;
    a.F = c.F;
    a.S = c.S;
    a.T = c.T;
    a.Pbar = Pbar;
    a.mu_dLp = mu_dLp;
    a.mu_alpha = mu_alpha;
    a.gx = w.gx;
    a.gy = w.gy;
    a.gz = w.gz;
    a.knbar = w.knbar;
    a.tvbar = w.tvbar;
    a.dLp_bar = dLp_bar;
    a.alpha_bar = alpha_bar;
    a.Gbar = theta ? w.Gbar : nullptr;
    a.sybar = theta ? w.sybar : nullptr;
    a.Hbar = theta ? w.Hbar : nullptr;
    k_vjp<<<agrid(c.n), ATPB, 0, c.stream>>>(a);
}

void adj_gather(Ctx &c, dvec4 *xbar, bool masked, bool theta, AdjBuffers &w)
{
    GatherArgs g;
    g.n = c.n;
    g.lattice = c.hs.lattice;
    g.radius = c.hs.radius;
    g.nbr = c.nbr;
    g.shell = c.shell;
    g.rev = c.rev;
    g.nbv = c.nbv;
    g.gx = w.gx;
    g.gy = w.gy;
    g.gz = w.gz;
    g.knbar = w.knbar;
    g.tvbar = w.tvbar;
    g.Gbar = w.Gbar;
    g.sybar = w.sybar;
    g.Hbar = w.Hbar;
    g.E = w.E;
    g.nu = w.nu;
    g.xbar = xbar;
    g.mask = masked ? c.mask : nullptr;
    g.gC = theta ? w.gC : nullptr;
    g.gE = (theta && w.E) ? w.gE : nullptr;
    g.gnu = (theta && w.E) ? w.gnu : nullptr;
    g.gsy = theta ? w.gsy : nullptr;
    g.gH = theta ? w.gH : nullptr;
    k_vjp_gather<<<agrid(c.n), ATPB, 0, c.stream>>>(g);
}

void adj_dot(Ctx &c, const dvec4 *x, const dvec4 *y, double *out)
{
    k_dot<<<red_grid(c), RTPB, 0, c.stream>>>(c.n, x, y, c.partials, c.counter, out);
}

void adj_multidot(Ctx &c, int K, const dvec4 *const *A, const dvec4 *w, double *out)
{
    MultiDot md;
    md.K = K;
    for (int k = 0; k < 16; k++)
        md.A[k] = k < K ? A[k] : w;
    const int sms = c.tune.sms > 0 ? c.tune.sms : 152;
    // 16 partials per block must fit the reduction buffer (sized for 16 blocks per SM x 4)
    k_multidot<<<2 * sms, RTPB, 0, c.stream>>>(c.n, md, w, c.partials, c.counter, out);
}

void adj_axpby(Ctx &c, double alpha, const dvec4 *x, double beta, dvec4 *y)
{
    k_axpby<<<red_grid(c), RTPB, 0, c.stream>>>(c.n, alpha, x, beta, y);
}

void adj_reaction(Ctx &c, int type, int comp, double *out)
{
    k_reaction<<<red_grid(c), RTPB, 0, c.stream>>>(c.n, c.type, type, comp, c.Pin, c.partials, c.counter, out);
}

void adj_reaction_seed(Ctx &c, int type, int comp, double w, const dvec4 *lam, dvec4 *Pbar)
{
    k_reaction_seed<<<agrid(c.n), ATPB, 0, c.stream>>>(c.n, c.type, type, comp, w, lam, Pbar);
}

}  // namespace lpm
