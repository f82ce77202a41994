// Damage stage of the reference's main (src/constitutive.c:149-164,
// :1399-1862): nonlocal ductile damage for J2, brittle bond breaking for
// elastic bonds, and the stress weights of the intact bonds.
//
// Compiled with -fmad=false and written in the reference's evaluation order.
// The nonlocal sum visits the particles within 3 L cell by cell instead of in
// ascending index, and exp is CUDA's, so damage_nonlocal agrees with the
// reference to rounding rather than bit for bit; every other quantity here is
// a comparison, a copy or a product the reference also forms.
//
// Bond arrays are slot-major [NN][n]: bond b = j * n + i is slot j of
// particle i.  Damage kernels that find bonds append them to a list with an
// atomic counter; the host sorts the list into the reference's (i, j) scan
// order before logging or choosing bonds, so the outcome does not depend on
// the order the threads ran in.
#include "lpm_internal.h"

namespace lpm {

constexpr int DTPB = 128;
constexpr double DMG_EPS = 1e-6;  // EPS, include/lpm.h:42

static inline int dgrid(long long n) { return (int)((n + DTPB - 1) / DTPB); }

// updateDuctileDamagePwiseNonlocal (src/constitutive.c:1796-1820): for a
// particle at or below the threshold, damage_nonlocal += (sum_j Ddot_j
// phi(r_ij) V) / (sum_j phi(r_ij) V) over the particles j within 3 L at the
// initial positions (i itself included), Ddot_j = dlambda_j (1 + A
// triaxiality_j) when positive, phi(r) = exp(-r^2 / 2 L^2) / (L sqrt(2 pi)).
// J2_triaxiality is never assigned in the reference, so it is 0 here too.
// Particles above the threshold are clamped to 1.
__global__ void __launch_bounds__(DTPB) k_dmg_nonlocal(int n, const dvec4 *__restrict__ x0,
                                                       const int *__restrict__ cstart,
                                                       const int *__restrict__ corder, int g0, int g1, int g2,
                                                       double lo0, double lo1, double lo2, double cs, double L,
                                                       double thr, double cA, double vol,
                                                       const double *__restrict__ dlambda, double *dnl)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    const double d0 = dnl[i];
    if (d0 > thr) {
        if (d0 > 1.0)
            dnl[i] = 1.0;
        return;
    }
    const dvec4 xi = x0[i];
    const int cx = min(g0 - 1, (int)((xi.x - lo0) / cs)), cy = min(g1 - 1, (int)((xi.y - lo1) / cs)),
              cz = min(g2 - 1, (int)((xi.z - lo2) / cs));
    const double rc = 3 * L;
    const double PI_ = 3.14159265358979323846;  // include/lpm.h:34
    double Ddot = 0.0, A = 0.0;
    for (int dz = -1; dz <= 1; dz++) {
        const int z = cz + dz;
        if (z < 0 || z >= g2)
            continue;
        for (int dy = -1; dy <= 1; dy++) {
            const int y = cy + dy;
            if (y < 0 || y >= g1)
                continue;
            for (int dx = -1; dx <= 1; dx++) {
                const int x = cx + dx;
                if (x < 0 || x >= g0)
                    continue;
                const size_t c = ((size_t)z * g1 + y) * g0 + x;
                for (int q = cstart[c]; q < cstart[c + 1]; q++) {
                    const int j = corder[q];
                    const dvec4 xj = x0[j];
                    const double ex = xj.x - xi.x, ey = xj.y - xi.y, ez = xj.z - xi.z;
                    const double dis = sqrt(ex * ex + ey * ey + ez * ez);
                    if (dis < rc) {
                        double DdotLocal = 0;
                        const double triax = 0.0;
                        const double damage_f = (1.0 + cA * triax);
                        if (damage_f > 0.0)
                            DdotLocal = dlambda[j] * (1.0 + cA * triax);
                        const double phi = 1.0 / L / sqrt(2 * PI_) * exp(-0.5 * dis * dis / L / L);
                        Ddot += DdotLocal * phi * vol;
                        A += phi * vol;
                    }
                }
            }
        }
    }
    if (Ddot > 0.0)
        dnl[i] = d0 + 1.0 / A * Ddot;
}

// src/constitutive.c:1822-1841: every intact bond touching a particle past
// the threshold breaks (D = 1); the broken bonds go to the list.
__global__ void k_dmg_ductile_break(int n, const int *__restrict__ nbr, const int8_t *__restrict__ nbv,
                                    const double *__restrict__ dnl, double thr, double *brk, double *D,
                                    int *list, int *count)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    const int nbi = nbv[i];
    const bool hot = dnl[i] > thr;
    for (int j = 0; j < nbi; j++) {
        const size_t b = (size_t)j * n + i;
        if (hot || dnl[nbr[b]] > thr) {
            if (fabs(brk[b]) > DMG_EPS) {
                brk[b] = 0.0;
                D[b] = 1.0;
                list[atomicAdd(count, 1)] = (int)b;
            }
        }
    }
}

// src/constitutive.c:1843-1854: intact bonds carry D = max of the two
// particles' nonlocal damage; w = 1 - D for every bond.
__global__ void k_dmg_ductile_w(int n, const int *__restrict__ nbr, const int8_t *__restrict__ nbv,
                                const double *__restrict__ dnl, const double *__restrict__ brk, double *D,
                                double *w)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    const int nbi = nbv[i];
    const double di = dnl[i];
    for (int j = 0; j < nbi; j++) {
        const size_t b = (size_t)j * n + i;
        if (fabs(brk[b]) > DMG_EPS) {
            const double dp = dnl[nbr[b]];
            D[b] = di > dp ? di : dp;
        }
        w[b] = 1.0 - D[b];
    }
}

// updateBrittleDamage (src/constitutive.c:1452-1469): bonds whose elastic
// stretch over the initial length reaches the critical strain (broken bonds
// have zero stretch) go to the list with their strain.
__global__ void k_dmg_brittle_cand(int n, const int8_t *__restrict__ nbv, const double *__restrict__ dL,
                                   const double *__restrict__ L0, double crit, int *list, double *lval, int *count)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    const int nbi = nbv[i];
    for (int j = 0; j < nbi; j++) {
        const size_t b = (size_t)j * n + i;
        const double ave_bstrain = dL[b] / L0[b];
        if (ave_bstrain >= crit) {
            const int k = atomicAdd(count, 1);
            list[k] = (int)b;
            lval[k] = ave_bstrain;
        }
    }
}

// src/constitutive.c:1476-1520: the chosen bonds break.
__global__ void k_dmg_break_list(const int *__restrict__ bonds, int k, double *brk, double *D, double *w)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= k)
        return;
    const int b = bonds[t];
    D[b] = 1.0;
    w[b] = 0.0;
    brk[b] = 0.0;
}

// opp_flag / particle_volume of every bond as the force and stress routines
// compute it (src/constitutive.c:532-551, src/lpm_basic.c:70-90): 0.5 while
// the particle keeps all its bonds, else 0.5 if the bond's opposite bond
// exists and is intact, 1.0 otherwise.
__global__ void k_dmg_oppv(int n, const int8_t *__restrict__ nbv, const int8_t *__restrict__ nbc,
                           const int8_t *__restrict__ opp, const double *__restrict__ brk, double vol,
                           double *oppv)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    const int nbi = nbv[i];
    const bool full = nbc[i] == LPM_NN;
    for (int j = 0; j < nbi; j++) {
        const size_t b = (size_t)j * n + i;
        double o = 1.0;
        if (full) {
            o = 0.5;
        } else {
            const int m = opp[b];
            if (m >= 0)
                o = brk[(size_t)m * n + i] <= DMG_EPS ? 1.0 : 0.5;
        }
        oppv[b] = o / vol;
    }
}

void launch_dmg_nonlocal(Ctx &c)
{
    const Ctx::Damage &d = c.dmg;
    k_dmg_nonlocal<<<dgrid(c.n), DTPB, 0, c.stream>>>(c.n, c.xyz0, d.cstart, d.corder, d.g[0], d.g[1], d.g[2],
                                                      d.lo[0], d.lo[1], d.lo[2], d.cs, d.opts.length,
                                                      d.opts.threshold, d.opts.triax_coeff, c.hs.vol, c.dlambda,
                                                      d.dnl[0]);
}

void launch_dmg_ductile_break(Ctx &c)
{
    Ctx::Damage &d = c.dmg;
    cudaMemsetAsync(d.count, 0, sizeof(int), c.stream);
    k_dmg_ductile_break<<<dgrid(c.n), DTPB, 0, c.stream>>>(c.n, c.nbr, c.nbv, d.dnl[0], d.opts.threshold, d.brk,
                                                           d.D[0], d.list, d.count);
}

void launch_dmg_ductile_w(Ctx &c)
{
    Ctx::Damage &d = c.dmg;
    k_dmg_ductile_w<<<dgrid(c.n), DTPB, 0, c.stream>>>(c.n, c.nbr, c.nbv, d.dnl[0], d.brk, d.D[0], d.dw);
}

void launch_dmg_brittle_cand(Ctx &c)
{
    Ctx::Damage &d = c.dmg;
    cudaMemsetAsync(d.count, 0, sizeof(int), c.stream);
    k_dmg_brittle_cand<<<dgrid(c.n), DTPB, 0, c.stream>>>(c.n, c.nbv, c.dL, c.L0, d.opts.critical_bstrain, d.list,
                                                          d.lval, d.count);
}

void launch_dmg_break_list(Ctx &c, const int *bonds, int k)
{
    Ctx::Damage &d = c.dmg;
    if (k > 0)
        k_dmg_break_list<<<dgrid(k), DTPB, 0, c.stream>>>(bonds, k, d.brk, d.D[0], d.dw);
}

void launch_dmg_oppv(Ctx &c)
{
    const Ctx::Damage &d = c.dmg;
    k_dmg_oppv<<<dgrid(c.n), DTPB, 0, c.stream>>>(c.n, c.nbv, d.nbc, d.opp, d.brk, c.hs.vol, c.oppv);
}

}  // namespace lpm
