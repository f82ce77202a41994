// Stiffness assembly: the elastic tangent of the internal force, computed
// analytically bond by bond and scattered into the fixed block-CSR by slot
// lookup (no atomics), plus the block-Jacobi preconditioner.
//
// The reference builds the same matrix by forward finite differences of
// computeBondForceElastic (src/stiffness.c:384-516): K_ik = dPin_i/dx_k, then
// stores the upper triangle with off-diagonal blocks averaged,
// 0.5 (K_ik + K_ki^T).  With the elastic bond force
//   F_ij = 2 Kn dL_ij + (T_i^s + T_n^s)/2 + Tv (S_i^s + S_n^s)/2,
//   Pin_i = sum_j c_ij F_ij,  c_ij = (x_i - x_n)/|x_i - x_n|,
// S_p^s = sum of shell-s stretches of p, T_p^s = sum of Tv-weighted ones,
// the derivative has, per bond j of particle i (partner n, shell s):
//   k = i : (F_ij/d)(I - c c^T) + 2Kn c c^T + c (x) a_j
//   k = n : -(Fbar_ij/d)(I - c c^T) - 2Kn c c^T + c (x) b_j - a_j (x) c
//   k = q, q a shell-s neighbour of n : -(Tv_nq + Tv_ij)/2 c (x) c_nq
// with a_j = (W_i^s + Tv_ij U_i^s)/2, b_j = (W_n^s + Tv_ij U_n^s)/2,
// U_p^s = sum of shell-s unit vectors, W_p^s = Tv-weighted sum.  Using
// Fbar_ij = (F_ij + F_ji)/2 in the off-diagonal geometric term is exactly the
// reference's symmetrisation; the other terms are already symmetric.
//
// With the damage stage on, a broken bond has zero stretch and force
// (damage_broken multiplies both, src/constitutive.c:254,271), so it drops out
// of the shell sums S, T, U, W, of its own terms and of the two-hop terms
// through it.  A pair contributes only when the bond and its reverse are both
// intact; that is the reference's matrix whenever the two break together.
#include "lpm_internal.h"

namespace lpm {

constexpr int STPB = 128;

// stretches, unit vectors and shell sums at the current configuration with
// the converged plastic stretch (computedL, src/lpm_basic.c:252-291), plus
// the unit-vector sums U and W of each shell.
__global__ void k_tgeom(int n, const dvec4 *xyz, const int *nbr, const int8_t *shell,
                        const int8_t *nbv, const double *L0, const double *Tv, const double *dLp,
                        const double *brk, double *dL, double *csx, double *csy, double *csz, double2 *S,
                        double2 *T, double *U, double *W)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    const int nbi = nbv[i];
    const dvec4 xi = xyz[i];
    double s[2] = {0, 0}, t[2] = {0, 0}, u[6] = {0, 0, 0, 0, 0, 0}, w[6] = {0, 0, 0, 0, 0, 0};
    for (int j = 0; j < nbi; j++) {
        const size_t b = (size_t)j * n + i;
        const dvec4 xp = xyz[nbr[b]];
        const double dx = xi.x - xp.x, dy = xi.y - xp.y, dz = xi.z - xp.z;
        const double dis = sqrt(dx * dx + dy * dy + dz * dz);
        double v = dis - L0[b];
        v -= dLp[b];
        if (brk)
            v *= brk[b];  // damage_broken
        dL[b] = v;
        const int sh = shell[b];
        s[sh] += v;
        t[sh] += Tv[b] * v;
        const double cx = dx / dis, cy = dy / dis, cz = dz / dis;
        csx[b] = cx;
        csy[b] = cy;
        csz[b] = cz;
        if (brk && brk[b] == 0.0)
            continue;
        u[3 * sh] += cx;
        u[3 * sh + 1] += cy;
        u[3 * sh + 2] += cz;
        w[3 * sh] += Tv[b] * cx;
        w[3 * sh + 1] += Tv[b] * cy;
        w[3 * sh + 2] += Tv[b] * cz;
    }
    S[i] = make_double2(s[0], s[1]);
    T[i] = make_double2(t[0], t[1]);
    for (int k = 0; k < 6; k++) {
        U[(size_t)k * n + i] = u[k];
        W[(size_t)k * n + i] = w[k];
    }
}

struct AsmArgs {
    int n;
    const dvec4 *xyz;
    const int *nbr;
    const int8_t *shell, *rev, *nbv, *nconn;
    const double *Kn, *Tv, *dL, *csx, *csy, *csz, *U, *W;
    const double2 *S, *T;
    const long long *rowoff;
    const int *npad, *cols;
    const double *brk;  // damage_broken [NN][n], null while the damage stage is off
};

__device__ __forceinline__ int find_slot(const int *c, int cnt, int key)
{
    int lo = 0, hi = cnt - 1;
    while (lo <= hi) {
        const int mid = (lo + hi) >> 1;
        const int v = c[mid];
        if (v == key)
            return mid;
        if (v < key)
            lo = mid + 1;
        else
            hi = mid - 1;
    }
    return -1;
}

template <typename V>
__device__ __forceinline__ void add_block(V *row, int np, int slot, const double (&blk)[9])
{
#pragma unroll
    for (int k = 0; k < 9; k++)
        row[(size_t)k * np + slot] += (V)blk[k];
}

// One thread per block row i.  All contributions of the row are added in a
// fixed order (deterministic); other rows are never written.
template <typename V>
__global__ void __launch_bounds__(STPB) k_assemble(AsmArgs a, V *val)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n)
        return;
    const int n = a.n, nbi = a.nbv[i], nc = a.nconn[i], np = a.npad[i];
    const long long off = a.rowoff[i];
    const int *cols = a.cols + off;
    V *row = val + 9 * off;
    for (int k = 0; k < 9 * np; k++)
        row[k] = (V)0;
    const dvec4 xi = a.xyz[i];
    const double2 Si = a.S[i], Ti = a.T[i];
    double self[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    for (int j = 0; j < nbi; j++) {
        const size_t b = (size_t)j * n + i;
        const int p = a.nbr[b];
        const int s = a.shell[b];
        const dvec4 xp = a.xyz[p];
        const double dx = xi.x - xp.x, dy = xi.y - xp.y, dz = xi.z - xp.z;
        const double d = sqrt(dx * dx + dy * dy + dz * dz);
        const double c[3] = {a.csx[b], a.csy[b], a.csz[b]};
        const double kn = a.Kn[b], tv = a.Tv[b];
        const double2 Sp = a.S[p], Tp = a.T[p];
        const double Tsum = (s == 0 ? Ti.x + Tp.x : Ti.y + Tp.y);
        const double Ssum = (s == 0 ? Si.x + Sp.x : Si.y + Sp.y);
        const int rv = a.rev[b];
        if (a.brk && a.brk[b] * (rv >= 0 ? a.brk[(size_t)rv * n + p] : 1.0) == 0.0)
            continue;  // broken pair
        const double dlij = a.dL[b], dlji = rv >= 0 ? a.dL[(size_t)rv * n + p] : dlij;
        const double fel = 2.0 * kn * dlij + 0.5 * Tsum + 0.5 * tv * Ssum;
        const double fbar = kn * (dlij + dlji) + 0.5 * Tsum + 0.5 * tv * Ssum;
        double av[3], bv[3];
        for (int k = 0; k < 3; k++) {
            av[k] = 0.5 * (a.W[(size_t)(3 * s + k) * n + i] + tv * a.U[(size_t)(3 * s + k) * n + i]);
            bv[k] = 0.5 * (a.W[(size_t)(3 * s + k) * n + p] + tv * a.U[(size_t)(3 * s + k) * n + p]);
        }
        double blk[9];
        for (int r = 0; r < 3; r++)
            for (int q = 0; q < 3; q++) {
                const double proj = (r == q ? 1.0 : 0.0) - c[r] * c[q];
                self[3 * r + q] += fel / d * proj + 2.0 * kn * c[r] * c[q] + c[r] * av[q];
                blk[3 * r + q] = -fbar / d * proj - 2.0 * kn * c[r] * c[q] + c[r] * bv[q] - av[r] * c[q];
            }
        const int sn = find_slot(cols, nc, p);
        if (sn >= 0)
            add_block(row, np, sn, blk);
        // two-hop terms through n's same-shell bonds
        const int nbp = a.nbv[p];
        for (int m = 0; m < nbp; m++) {
            const size_t bm = (size_t)m * n + p;
            if (a.shell[bm] != s || (a.brk && a.brk[bm] == 0.0))
                continue;
            const int q = a.nbr[bm];
            const double cq[3] = {a.csx[bm], a.csy[bm], a.csz[bm]};
            const double f = -0.5 * (a.Tv[bm] + tv);
            if (q == i) {
                for (int r = 0; r < 3; r++)
                    for (int t = 0; t < 3; t++)
                        self[3 * r + t] += f * c[r] * cq[t];
                continue;
            }
            const int sq = find_slot(cols, nc, q);
            if (sq < 0)
                continue;
            for (int r = 0; r < 3; r++)
                for (int t = 0; t < 3; t++)
                    blk[3 * r + t] = f * c[r] * cq[t];
            add_block(row, np, sq, blk);
        }
    }
    const int ss = find_slot(cols, nc, i);
    if (ss >= 0)
        add_block(row, np, ss, self);
}

// Block-Jacobi: inverse of each 3x3 diagonal block with the constrained
// DOFs' rows and columns replaced by the identity (setDispBC_stiffnessUpdate3D,
// src/boundary.c:159-281, decouples them; their solution is zero).
template <typename V, typename P>
__global__ void k_jacobi(int n, const long long *rowoff, const int *npad, const int *cols,
                         const int8_t *nconn, const V *val, const uint8_t *mask, P *Pinv)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    const long long off = rowoff[i];
    const int np = npad[i];
    const int ss = find_slot(cols + off, nconn[i], i);
    double m[9];
    const uint8_t fm = mask[i];
    for (int r = 0; r < 3; r++)
        for (int c = 0; c < 3; c++) {
            const bool fr = (fm >> r) & 1u, fc = (fm >> c) & 1u;
            double v = ss >= 0 ? (double)val[9 * off + (size_t)(3 * r + c) * np + ss] : 0.0;
            if (!fr || !fc)
                v = (r == c) ? 1.0 : 0.0;
            m[3 * r + c] = v;
        }
    // symmetric part (the stored blocks are symmetric up to rounding)
    const double a00 = m[0], a11 = m[4], a22 = m[8];
    const double a01 = 0.5 * (m[1] + m[3]), a02 = 0.5 * (m[2] + m[6]), a12 = 0.5 * (m[5] + m[7]);
    const double c00 = a11 * a22 - a12 * a12, c01 = a02 * a12 - a01 * a22, c02 = a01 * a12 - a02 * a11;
    const double c11 = a00 * a22 - a02 * a02, c12 = a01 * a02 - a00 * a12, c22 = a00 * a11 - a01 * a01;
    double det = a00 * c00 + a01 * c01 + a02 * c02;
    if (!(fabs(det) > 0.0))
        det = 1.0;
    const double inv = 1.0 / det;
    const double out[9] = {c00 * inv, c01 * inv, c02 * inv, c01 * inv, c11 * inv, c12 * inv,
                           c02 * inv, c12 * inv, c22 * inv};
    for (int k = 0; k < 9; k++)
        Pinv[(size_t)k * n + i] = (P)out[k];
}

void launch_tangent_geometry(Ctx &c)
{
    k_tgeom<<<(c.n + STPB - 1) / STPB, STPB, 0, c.stream>>>(c.n, c.xyz, c.nbr, c.shell, c.nbv, c.L0, c.Tv,
                                                            c.dLp[0], c.dmg.brk, c.dL, c.csx, c.csy, c.csz,
                                                            c.S, c.T, c.U, c.W);
}

void launch_assemble(Ctx &c, bool fp32)
{
    AsmArgs a;
    a.n = c.n;
    a.xyz = c.xyz;
    a.nbr = c.nbr;
    a.shell = c.shell;
    a.rev = c.rev;
    a.nbv = c.nbv;
    a.nconn = c.nconn_d;
    a.Kn = c.Kn;
    a.Tv = c.Tv;
    a.dL = c.dL;
    a.csx = c.csx;
    a.csy = c.csy;
    a.csz = c.csz;
    a.U = c.U;
    a.W = c.W;
    a.S = c.S;
    a.T = c.T;
    a.rowoff = c.rowoff;
    a.npad = c.npad;
    a.cols = c.cols;
    a.brk = c.dmg.brk;
    const int g = (c.n + STPB - 1) / STPB;
    if (fp32)
        k_assemble<float><<<g, STPB, 0, c.stream>>>(a, c.Kf);
    else
        k_assemble<double><<<g, STPB, 0, c.stream>>>(a, c.Kd);
}

// [9][n] -> [n][9]: the smoother reads one row's inverse as 36 contiguous bytes
__global__ void k_rows_of(int n, const float *__restrict__ in, float *__restrict__ out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    for (int k = 0; k < 9; k++)
        out[(size_t)i * 9 + k] = in[(size_t)k * n + i];
}

void launch_block_jacobi(Ctx &c, bool fp32)
{
    const int g = (c.n + STPB - 1) / STPB;
    if (fp32) {
        // FP32 inverse for FP32 CG vectors, FP64 inverse of the same FP32 blocks
        // for the FP64-vector variant
        k_jacobi<float, float><<<g, STPB, 0, c.stream>>>(c.n, c.rowoff, c.npad, c.cols, c.nconn_d, c.Kf,
                                                         c.mask, c.Pinv_f);
        k_jacobi<float, double><<<g, STPB, 0, c.stream>>>(c.n, c.rowoff, c.npad, c.cols, c.nconn_d, c.Kf,
                                                          c.mask, c.Pinv_d);
    } else {
        k_jacobi<double, double><<<g, STPB, 0, c.stream>>>(c.n, c.rowoff, c.npad, c.cols, c.nconn_d, c.Kd,
                                                           c.mask, c.Pinv_d);
        // the multigrid's level-0 smoother works in FP32
        if (c.opts.preconditioner == LPM_PRECOND_AMG && c.nspec == 0)
            k_jacobi<double, float><<<g, STPB, 0, c.stream>>>(c.n, c.rowoff, c.npad, c.cols, c.nconn_d, c.Kd,
                                                              c.mask, c.Pinv_f);
    }
    if (c.opts.preconditioner == LPM_PRECOND_AMG && c.nspec == 0)
        k_rows_of<<<g, STPB, 0, c.stream>>>(c.n, c.Pinv_f, c.Pinv_rf);
}

}  // namespace lpm
