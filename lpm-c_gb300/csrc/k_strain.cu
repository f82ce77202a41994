// computeStrain (src/lpm_basic.c:127-249): the particle strain tensor by
// weighted least squares over the bonds (weight 0.1 for the first shell, 0.9
// for the second), fitting e : (n (x) n) to the bond strains dL / L0 with
// n = (x0_j - x0_i) / L0.  One thread per particle builds the 6 x 6 normal
// system from the fourth- and second-order direction moments and solves it
// by LU with partial pivoting (first maximal |pivot|), the reference's
// dgesv call.  Compiled without FMA contraction and in the reference's
// evaluation order, so the result is bit-identical for the same inputs.
#include "lpm_internal.h"

namespace lpm {

namespace {

constexpr int STR_TPB = 128;

__global__ void __launch_bounds__(STR_TPB) k_strain(int n, const dvec4 *__restrict__ x0, const int *__restrict__ nbr,
                                                    const int8_t *__restrict__ shell, const int8_t *__restrict__ nbv,
                                                    const double *__restrict__ L0, const double *__restrict__ dL,
                                                    double *strain)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    double r4[3][3][3][3], r2[3][3];
    for (int k = 0; k < 3; k++)
        for (int q = 0; q < 3; q++) {
            r2[k][q] = 0.0;
            for (int m = 0; m < 3; m++)
                for (int l = 0; l < 3; l++)
                    r4[k][q][m][l] = 0.0;
        }
    const dvec4 xi = x0[i];
    const double Xi[3] = {xi.x, xi.y, xi.z};
    const int nbi = nbv[i];
    for (int j = 0; j < nbi; j++) {
        const size_t b = (size_t)j * n + i;
        const int sh = shell[b];
        if (sh != 0 && sh != 1)
            continue;
        const double w = sh == 0 ? 0.1 : 0.9;
        const dvec4 xp = x0[nbr[b]];
        const double Xp[3] = {xp.x, xp.y, xp.z};
        const double d = L0[b];
        for (int k = 0; k < 3; k++)
            for (int q = 0; q < 3; q++)
                for (int m = 0; m < 3; m++)
                    for (int l = 0; l < 3; l++)
                        r4[k][q][m][l] += w * (Xp[k] - Xi[k]) / d * (Xp[q] - Xi[q]) / d * (Xp[m] - Xi[m]) / d *
                                          (Xp[l] - Xi[l]) / d;
        const double s = dL[b];
        for (int k = 0; k < 3; k++)
            for (int q = 0; q < 3; q++)
                r2[k][q] += w * s / d * (Xp[k] - Xi[k]) / d * (Xp[q] - Xi[q]) / d;
    }
    double A[36], rb[6];
    int ii = 0;
    for (int j = 0; j < 3; j++)
        for (int k = 0; k < 3; k++)
            for (int m = 0; m < 3; m++)
                for (int l = 0; l < 3; l++)
                    if (m <= l && j <= k)
                        A[ii++] = r4[m][l][j][k];
    ii = 0;
    for (int j = 0; j < 3; j++)
        for (int k = 0; k < 3; k++)
            if (j <= k)
                rb[ii++] = r2[j][k];
    // LU with partial pivoting, then the two triangular solves
    int piv[6];
    bool singular = false;
    for (int k = 0; k < 6; k++) {
        int p = k;
        double best = fabs(A[k * 6 + k]);
        for (int r = k + 1; r < 6; r++) {
            const double v = fabs(A[r * 6 + k]);
            if (v > best) {
                best = v;
                p = r;
            }
        }
        piv[k] = p;
        if (A[p * 6 + k] == 0.0) {
            singular = true;
            continue;
        }
        if (p != k)
            for (int c = 0; c < 6; c++) {
                const double t = A[k * 6 + c];
                A[k * 6 + c] = A[p * 6 + c];
                A[p * 6 + c] = t;
            }
        const double dk = A[k * 6 + k];
        for (int r = k + 1; r < 6; r++) {
            const double lr = A[r * 6 + k] / dk;
            A[r * 6 + k] = lr;
            if (lr != 0.0)
                for (int c = k + 1; c < 6; c++)
                    A[r * 6 + c] -= lr * A[k * 6 + c];
        }
    }
    if (singular) {
        // the reference leaves particle 0 as it was and stores the untouched
        // right-hand side for the others (src/lpm_basic.c:220-228)
        if (i == 0)
            return;
    } else {
        for (int k = 0; k < 6; k++)
            if (piv[k] != k) {
                const double t = rb[k];
                rb[k] = rb[piv[k]];
                rb[piv[k]] = t;
            }
        for (int r = 1; r < 6; r++) {
            double s = rb[r];
            for (int c = 0; c < r; c++)
                s -= A[r * 6 + c] * rb[c];
            rb[r] = s;
        }
        for (int r = 5; r >= 0; r--) {
            double s = rb[r];
            for (int c = r + 1; c < 6; c++)
                s -= A[r * 6 + c] * rb[c];
            rb[r] = s / A[r * 6 + r];
        }
    }
    // e11, e12, e13, e22, e23, e33 -> s11 s22 s33 s23 s13 s12 order
    strain[(size_t)0 * n + i] = rb[0];
    strain[(size_t)5 * n + i] = rb[1];
    strain[(size_t)4 * n + i] = rb[2];
    strain[(size_t)1 * n + i] = rb[3];
    strain[(size_t)3 * n + i] = rb[4];
    strain[(size_t)2 * n + i] = rb[5];
}

}  // namespace

void launch_strain(Ctx &c)
{
    k_strain<<<(c.n + STR_TPB - 1) / STR_TPB, STR_TPB, 0, c.stream>>>(c.n, c.xyz0, c.nbr, c.shell, c.nbv, c.L0, c.dL,
                                                                      c.strain);
}

}  // namespace lpm
