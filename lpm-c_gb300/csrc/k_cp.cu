// Crystal-plasticity return mapping (Miehe's algorithm, plmode 1) and the
// slip-system coupling matrix Cab, FP64, one thread per particle.
//
// Restates computeBondForceCPMiehe (src/constitutive.c:866-1318) and
// computeCab (src/constitutive.c:1864-1917).  The reference solves the
// nslip x nslip Newton system with LAPACKE_dgesv on a matrix whose inactive
// rows and columns are identity; partial pivoting never selects an inactive
// row and elimination never touches it, so the same arithmetic is done here
// on the compacted active block (at most 24 x 24, usually a few entries).
// Compiled with -fmad=false like the other force kernels.
#include "lpm_internal.h"

namespace lpm {

constexpr int CTPB = 64;

struct CpArgs {
    int n, ns;
    const dvec4 *xyz;
    const int *nbr;
    const int8_t *shell, *nbv;
    const double *L0, *Kn, *Tv, *oppv;
    double *csx, *csy, *csz;
    double *dL;
    double2 *S, *T;
    const double *dLp_c;
    double *dLp_t;
    const double *gy_c, *As_c, *A_c;
    double *gy_t, *As_t, *A_t;
    const double *Cab;
    const double *sch;  // [ns][6]
    int *jact;
    double tau0, taus, h0, p, q, eta, maxloop, dtime;
    int *status;
    int *pl_flag;
    // damage_broken / damage_w [NN][n]; null while the damage stage is off
    const double *brk, *dw;
};

__device__ __forceinline__ double proj6(const double *sc, double cx, double cy, double cz)
{
    return cx * cx * sc[0] + cy * cy * sc[1] + cz * cz * sc[2] + cy * cz * sc[3] + cx * cz * sc[4] +
           cx * cy * sc[5];
}

// DMG: the damage stage is on (a.brk, a.dw set); the undamaged instantiation
// carries no trace of it.
template <bool DMG>
__global__ void __launch_bounds__(CTPB) k_cp(CpArgs a)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n)
        return;
    const int n = a.n, ns = a.ns, nbi = a.nbv[i];
    const dvec4 xi = a.xyz[i];
    double e[LPM_NN], dL[LPM_NN], xdL[LPM_NN], ddlp[LPM_NN];
    double S[2] = {0, 0}, T[2] = {0, 0};
    // trial stretches (src/constitutive.c:911-936)
    for (int j = 0; j < LPM_NN; j++) {
        ddlp[j] = 0.0;
        if (j < nbi) {
            const size_t b = (size_t)j * n + i;
            const dvec4 xp = a.xyz[a.nbr[b]];
            const double dx = xi.x - xp.x, dy = xi.y - xp.y, dz = xi.z - xp.z;
            const double dis = sqrt(dx * dx + dy * dy + dz * dz);
            e[j] = dis - a.L0[b];
            double v = e[j];
            v -= a.dLp_c[b];
            if (DMG)
                v *= a.brk[b];  // damage_broken
            dL[j] = v;
            xdL[j] = v;
            S[a.shell[b]] += v;
            T[a.shell[b]] += a.Tv[b] * v;
            a.csx[b] = dx / dis;
            a.csy[b] = dy / dis;
            a.csz[b] = dz / dis;
        }
    }
    double gamma[LPM_NSLIP], r[LPM_NSLIP], rr[LPM_NSLIP], xgy[LPM_NSLIP], RSS[LPM_NSLIP], yfn[LPM_NSLIP];
    double D[LPM_NSLIP * LPM_NSLIP];
    int act[LPM_NSLIP];
    unsigned J = 0u;
    double gy0[LPM_NSLIP];
    for (int m = 0; m < ns; m++) {
        gy0[m] = a.gy_c[(size_t)m * n + i];
        xgy[m] = gy0[m];
        gamma[m] = 0.0;
    }
    const double A0 = a.A_c[i];
    double xA = A0;
    auto stress_of = [&](const double *dls, const double *Ss, const double *Ts, double st[6]) {
        for (int k = 0; k < 6; k++)
            st[k] = 0.0;
        for (int j = 0; j < nbi; j++) {
            const size_t b = (size_t)j * n + i;
            const int s = a.shell[b];
            double fij = 2.0 * a.Kn[b] * dls[j] + Ts[s] + a.Tv[b] * Ss[s];
            if (DMG)
                fij *= a.dw[b];  // damage_w
            const double w = a.oppv[b] * a.L0[b] * fij;
            const double cx = a.csx[b], cy = a.csy[b], cz = a.csz[b];
            st[0] += w * cx * cx;
            st[1] += w * cy * cy;
            st[2] += w * cz * cz;
            st[3] += w * cy * cz;
            st[4] += w * cx * cz;
            st[5] += w * cx * cy;
        }
    };
    double st[6];
    stress_of(xdL, S, T, st);
    double tmax = 0.0;
    for (int m = 0; m < ns; m++) {
        const double *sc = a.sch + 6 * m;
        RSS[m] = st[0] * sc[0] + st[1] * sc[1] + st[2] * sc[2] + st[3] * sc[3] + st[4] * sc[4] + st[5] * sc[5];
        yfn[m] = RSS[m] - gy0[m];
        if (yfn[m] > tmax)
            tmax = yfn[m];
    }
    if (!(tmax <= 1e-6)) {
        a.pl_flag[i] = 1;  // pl_flag (src/constitutive.c:1026)
        // active-set loop (src/constitutive.c:1024-1305)
        int nouter = 0;
        const double dts = a.taus - a.tau0;
        for (;;) {
            nouter++;
            double nr = 1.0;
            int na = 0;
            for (int m = 0; m < ns; m++) {
                gamma[m] = r[m] = rr[m] = 0.0;
                if (J & (1u << m))
                    act[na++] = m;
            }
            int ninner = 0;
            do {
                ninner++;
                double dpl[6] = {0, 0, 0, 0, 0, 0};
                for (int s = 0; s < ns; s++) {
                    const double jg = ((J >> s) & 1u ? 1.0 : 0.0) * gamma[s];
                    for (int k = 0; k < 6; k++)
                        dpl[k] += jg * a.sch[6 * s + k];
                }
                double xS[2] = {0, 0}, xT[2] = {0, 0};
                for (int j = 0; j < nbi; j++) {
                    const size_t b = (size_t)j * n + i;
                    const double cx = a.csx[b], cy = a.csy[b], cz = a.csz[b];
                    double v = a.L0[b] * (dpl[0] * cx * cx + dpl[1] * cy * cy + dpl[2] * cz * cz +
                                          dpl[3] * cy * cz + dpl[4] * cx * cz + dpl[5] * cx * cy);
                    if (DMG)
                        v *= a.brk[b];  // damage_broken
                    ddlp[j] = v;
                    xdL[j] = dL[j] - v;
                    xS[a.shell[b]] += xdL[j];
                    xT[a.shell[b]] += a.Tv[b] * xdL[j];
                }
                stress_of(xdL, xS, xT, st);
                double dA = 0.0;
                for (int s = 0; s < ns; s++)
                    dA += gamma[s];
                xA = A0 + dA;
                const double ch = cosh(a.h0 * xA / dts);
                const double hh = a.h0 / (ch * ch);
                const double hp = -2.0 * a.h0 * a.h0 / dts * tanh(a.h0 * xA / dts) * hh;
                for (int al = 0; al < ns; al++) {
                    double t1 = 0.0;
                    for (int b2 = 0; b2 < ns; b2++) {
                        const double hab = (al == b2) ? hh : a.q * hh;
                        t1 += ((J >> b2) & 1u ? 1.0 : 0.0) * hab * gamma[b2];
                    }
                    xgy[al] = gy0[al] + ((J >> al) & 1u ? 1.0 : 0.0) * t1;
                }
                for (int m = 0; m < ns; m++) {
                    const double *sc = a.sch + 6 * m;
                    const double t1 = pow(1. + gamma[m] * a.eta / a.dtime, 1. / a.p);
                    RSS[m] = st[0] * sc[0] + st[1] * sc[1] + st[2] * sc[2] + st[3] * sc[3] + st[4] * sc[4] +
                             st[5] * sc[5];
                    r[m] = ((J >> m) & 1u ? 1.0 : 0.0) * (RSS[m] - xgy[m] * t1);
                }
                // Jacobian on the active block
                for (int ia = 0; ia < na; ia++) {
                    const int m = act[ia];
                    const double t1 = xgy[m] * (a.eta / a.p / a.dtime *
                                                pow(1. + a.eta * gamma[m] / a.dtime, (1. - a.p) / a.p));
                    const double pw = pow(1. + a.eta * gamma[m] / a.dtime, (1. / a.p));
                    for (int ib = 0; ib < na; ib++) {
                        const int q = act[ib];
                        double hs = 0.0;
                        for (int d = 0; d < ns; d++) {
                            double hd;
                            if (m == d && q == d)
                                hd = hh + hp * gamma[d];
                            else if (m == d && q != d)
                                hd = hp * gamma[d];
                            else if (m != d && q == d)
                                hd = a.q * (hh + hp * gamma[d]);
                            else
                                hd = a.q * hp * gamma[d];
                            hs += ((J >> d) & 1u ? 1.0 : 0.0) * hd;
                        }
                        const double t2 = hs * pw;
                        const double cab = a.Cab[((size_t)m * ns + q) * n + i];
                        D[ia * na + ib] = (m == q) ? cab + t1 + t2 : cab + t2;
                    }
                    rr[ia] = r[m];
                }
                // LU with partial pivoting (first maximal |pivot|) and solve
                bool singular = false;
                int piv[LPM_NSLIP];
                for (int k = 0; k < na; k++) {
                    int pv = k;
                    double best = fabs(D[k * na + k]);
                    for (int ii = k + 1; ii < na; ii++) {
                        const double v = fabs(D[ii * na + k]);
                        if (v > best) {
                            best = v;
                            pv = ii;
                        }
                    }
                    piv[k] = pv;
                    if (D[pv * na + k] == 0.0) {
                        singular = true;
                        continue;
                    }
                    if (pv != k)
                        for (int cc = 0; cc < na; cc++) {
                            const double t = D[k * na + cc];
                            D[k * na + cc] = D[pv * na + cc];
                            D[pv * na + cc] = t;
                        }
                    const double dd = D[k * na + k];
                    for (int ii = k + 1; ii < na; ii++) {
                        const double l = D[ii * na + k] / dd;
                        D[ii * na + k] = l;
                        if (l != 0.0)
                            for (int cc = k + 1; cc < na; cc++)
                                D[ii * na + cc] -= l * D[k * na + cc];
                    }
                }
                if (singular) {
                    atomicOr(a.status, LPM_STATUS_CP_SINGULAR);
                    break;
                }
                for (int k = 0; k < na; k++)
                    if (piv[k] != k) {
                        const double t = rr[k];
                        rr[k] = rr[piv[k]];
                        rr[piv[k]] = t;
                    }
                for (int ii = 1; ii < na; ii++) {
                    double s = rr[ii];
                    for (int cc = 0; cc < ii; cc++)
                        s -= D[ii * na + cc] * rr[cc];
                    rr[ii] = s;
                }
                for (int ii = na - 1; ii >= 0; ii--) {
                    double s = rr[ii];
                    for (int cc = ii + 1; cc < na; cc++)
                        s -= D[ii * na + cc] * rr[cc];
                    rr[ii] = s / D[ii * na + ii];
                }
                for (int ia = 0; ia < na; ia++)
                    gamma[act[ia]] += 1.0 * rr[ia];
                double s2 = 0.0;
                for (int m = 0; m < ns; m++)
                    s2 += r[m] * r[m];
                nr = sqrt(s2);
            } while (nr > 1e-4 && ninner < 20);
            // drop the most negative-yield active system with non-positive slip
            int mi = -1;
            double my = 0.0;
            for (int m = 0; m < ns; m++) {
                yfn[m] = RSS[m] - xgy[m];
                if (((J >> m) & 1u) && gamma[m] <= 0.0 && yfn[m] < my) {
                    my = yfn[m];
                    mi = m;
                }
            }
            if (mi != -1) {
                J &= ~(1u << mi);
                continue;
            }
            // add the most loaded inactive system
            int ma = -1;
            double mxy = 0.0;
            for (int m = 0; m < ns; m++)
                if (!((J >> m) & 1u) && yfn[m] > 0.0 && yfn[m] > mxy) {
                    mxy = yfn[m];
                    ma = m;
                }
            if (ma != -1) {
                J |= (1u << ma);
                if (nouter < a.maxloop)
                    continue;
            }
            break;
        }
    } else {
        for (int j = 0; j < LPM_NN; j++)
            ddlp[j] = 0.0;
    }
    // state of slot 2 (src/constitutive.c:1307-1380) and re-summed dilatation
    S[0] = S[1] = T[0] = T[1] = 0.0;
    for (int j = 0; j < LPM_NN; j++) {
        const size_t b = (size_t)j * n + i;
        const double lp = (DMG ? a.brk[b] : 1.0) * (a.dLp_c[b] + (j < nbi ? ddlp[j] : 0.0));
        a.dLp_t[b] = lp;
        if (j < nbi) {
            double v = e[j];
            v -= lp;
            if (DMG)
                v *= a.brk[b];  // damage_broken
            a.dL[b] = v;
            S[a.shell[b]] += v;
            T[a.shell[b]] += a.Tv[b] * v;
        }
    }
    a.S[i] = make_double2(S[0], S[1]);
    a.T[i] = make_double2(T[0], T[1]);
    for (int s = 0; s < ns; s++) {
        const double das = ((J >> s) & 1u ? 1.0 : 0.0) * gamma[s];
        a.gy_t[(size_t)s * n + i] = xgy[s];
        a.As_t[(size_t)s * n + i] = a.As_c[(size_t)s * n + i] + das;
    }
    a.A_t[i] = xA;
    a.jact[i] = (int)J;
}

// computeCab (src/constitutive.c:1864-1917) on the current geometry:
// Cab[m][q] = sum_j -(opp/V) L_j dF_j/dgamma_q P_m(j).
__global__ void __launch_bounds__(CTPB) k_cab(int n, int ns, const int8_t *nbv, const int8_t *shell,
                                              const double *L0, const double *Kn, const double *Tv,
                                              const double *oppv, const double *csx, const double *csy,
                                              const double *csz, const double *sch, double *Cab)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    const int nbi = nbv[i];
    for (int m = 0; m < ns; m++)
        for (int q = 0; q < ns; q++) {
            double ls[2] = {0, 0};
            for (int j = 0; j < nbi; j++) {
                const size_t b = (size_t)j * n + i;
                ls[shell[b]] += Tv[b] * L0[b] * proj6(sch + 6 * q, csx[b], csy[b], csz[b]);
            }
            double c = 0.;
            for (int j = 0; j < nbi; j++) {
                const size_t b = (size_t)j * n + i;
                const double dfdg = -2.0 * Kn[b] * L0[b] * proj6(sch + 6 * q, csx[b], csy[b], csz[b]) -
                                    2.0 * ls[shell[b]];
                c += -oppv[b] * L0[b] * dfdg * proj6(sch + 6 * m, csx[b], csy[b], csz[b]);
            }
            Cab[((size_t)m * ns + q) * n + i] = c;
        }
}

void launch_cp(Ctx &c)
{
    CpArgs a;
    a.n = c.n;
    a.ns = c.nslip;
    a.xyz = c.xyz;
    a.nbr = c.nbr;
    a.shell = c.shell;
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
    a.dLp_c = c.dLp[0];
    a.dLp_t = c.dLp[2];
    a.gy_c = c.gy[0];
    a.As_c = c.As[0];
    a.A_c = c.A[0];
    a.gy_t = c.gy[2];
    a.As_t = c.As[2];
    a.A_t = c.A[2];
    a.Cab = c.Cab;
    a.sch = c.sch;
    a.jact = c.jact;
    a.pl_flag = c.pl_flag;
    a.tau0 = c.cp[0];
    a.taus = c.cp[1];
    a.h0 = c.cp[2];
    a.p = c.cp[3];
    a.q = c.cp[4];
    a.eta = c.cp[5];
    a.maxloop = c.cp[6];
    a.dtime = c.cp[7];
    a.status = c.status;
    a.brk = c.dmg.brk;
    a.dw = c.dmg.dw;
    if (a.brk)
        k_cp<true><<<(c.n + CTPB - 1) / CTPB, CTPB, 0, c.stream>>>(a);
    else
        k_cp<false><<<(c.n + CTPB - 1) / CTPB, CTPB, 0, c.stream>>>(a);
}

void launch_cab(Ctx &c)
{
    k_cab<<<(c.n + CTPB - 1) / CTPB, CTPB, 0, c.stream>>>(c.n, c.nslip, c.nbv, c.shell, c.L0, c.Kn, c.Tv,
                                                          c.oppv, c.csx, c.csy, c.csz, c.sch, c.Cab);
}

}  // namespace lpm
