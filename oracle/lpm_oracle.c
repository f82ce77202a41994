/*
 * lpm_oracle.c - CPU restatement of the LPM-C quasi-static solve path.
 * TEST INFRASTRUCTURE ONLY (the checker); see lpm_oracle.h for the list of
 * reference functions restated here and how parity is kept.
 *
 * Structure: the reference evaluates bond forces particle by particle, each
 * call recomputing the stretches of the particle and all its neighbours
 * (src/constitutive.c:495-515).  The values each call computes for a given
 * particle depend only on that particle's own data, so the same results are
 * produced here by three race-free sweeps over all particles (own stretches
 * and return map; re-summed dilatation; averaged bond force and internal
 * force), in the reference's operation order.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <stdio.h>
#ifdef _OPENMP
#include <omp.h>
#endif
#include "lpm_oracle.h"
#include "mkl_shim/mkl.h"
#include "cg_rci.h"

#define NDIM 3
#define EPSP 1e-6      /* include/lpm.h:42 EPS */
#define TOLITER_ 1e-4  /* include/lpm.h:41 */
#define MAXSMALL_ 20   /* include/lpm.h:38 */
#define MAXSLIP 24

struct lpm_oracle {
    int n, nn, nn1, nn2, lattice, nafem, plmode, nslip;
    double radius, vol, cut1, cut2, xi;
    double box[6];
    /* particles */
    double *xyz, *xyz0, *xyz_temp;
    int *type, *nb;
    /* bonds [n][nn] */
    int *nbr, *shell, *nbr1, *nbr2, *rev;
    double *L0, *cs0x, *cs0y, *cs0z, *dist, *Kn, *Tv, *opp;
    /* AFEM connectivity and upper CSR */
    int *conn, *nconn, *kp0, *kp1;
    int nnz, *IK, *JK;
    double *K;
    /* material per particle */
    double *knt; /* [n][3] KnTve */
    double *G, *sy, *H;
    /* state, 3 slots each */
    double *dLp[3], *alpha[3], *beta[3];
    double *cp_gy[3], *cp_A[3], *cp_As[3];
    double *dlambda;
    /* per-iteration work */
    double *dL, *Ssum, *Tsum, *csx, *csy, *csz, *F, *F_temp, *ddLp;
    double *ddL, *ddS, *ddT;
    double *Pin, *Pex, *Pex_temp, *residual, *reaction, *disp, *stress;
    int *mask, nreact;
    /* crystal plasticity */
    double cp_tau0, cp_taus, cp_h0, cp_p, cp_q, cp_eta, cp_maxloop, dtime;
    double sch[MAXSLIP][6];
    double *Cab, *cp_RSS, *cp_dA, *cp_dgy, *cp_dAs;
    int *Jact;
    int error;
    /* damage (src/constitutive.c:1399-1862): per bond damage_broken (brk),
     * damage_w (dw), damage_D (dD, slots 0 and 1); per particle
     * damage_nonlocal (dnl, slots 0 and 1), damage_visual (dvis), the current
     * bond count nb (nbc; o->nb holds nb_initial) and fix_index (fix, per
     * DOF); the damage parameters and the broken-bond log (pairs i, j). */
    double *brk, *dw, *dD[2], *dnl[2], *dvis;
    int *nbc, *fix;
    double dmg_L, dmg_thr, dmg_cA, dmg_crit;
    int dmg_nbreak;
    int *blog, nblog, blog_cap;
};

static void *xcalloc(size_t n, size_t s)
{
    void *p = calloc(n ? n : 1, s);
    if (!p) {
        fprintf(stderr, "lpm_oracle: out of memory\n");
        abort();
    }
    return p;
}
#define DALLOC(n) ((double *)xcalloc((size_t)(n), sizeof(double)))
#define IALLOC(n) ((int *)xcalloc((size_t)(n), sizeof(int)))

void lo_set_threads(int n)
{
#ifdef _OPENMP
    omp_set_num_threads(n);
#else
    (void)n;
#endif
}

lpm_oracle *lo_create(void) { return (lpm_oracle *)xcalloc(1, sizeof(lpm_oracle)); }

void lo_free(lpm_oracle *o)
{
    if (!o)
        return;
    void *ptrs[] = {o->xyz, o->xyz0, o->xyz_temp, o->type, o->nb, o->nbr, o->shell, o->nbr1,
                    o->nbr2, o->rev, o->L0, o->cs0x, o->cs0y, o->cs0z, o->dist, o->Kn, o->Tv,
                    o->opp, o->conn, o->nconn, o->kp0, o->kp1, o->IK, o->JK, o->K, o->knt,
                    o->G, o->sy, o->H, o->dlambda, o->dL, o->Ssum, o->Tsum, o->csx, o->csy,
                    o->csz, o->F, o->F_temp, o->ddLp, o->ddL, o->ddS, o->ddT, o->Pin, o->Pex,
                    o->Pex_temp, o->residual, o->reaction, o->disp, o->stress, o->mask, o->Cab,
                    o->cp_RSS, o->cp_dA, o->cp_dgy, o->cp_dAs, o->Jact, o->brk, o->dw, o->dD[0],
                    o->dD[1], o->dnl[0], o->dnl[1], o->dvis, o->nbc, o->fix, o->blog};
    for (size_t k = 0; k < sizeof(ptrs) / sizeof(ptrs[0]); k++)
        free(ptrs[k]);
    for (int s = 0; s < 3; s++) {
        free(o->dLp[s]);
        free(o->alpha[s]);
        free(o->beta[s]);
        free(o->cp_gy[s]);
        free(o->cp_A[s]);
        free(o->cp_As[s]);
    }
    free(o);
}

/* ---------------------------------------------------------------------- */
/* Lattice generation: createCuboid, src/initialization.c:241-324 (SC) and
 * :326-459 (FCC), with the identity orientation (all Euler angles 0, so the
 * dgemv rotation of :287-313 returns each point unchanged). */
static int gen_lattice(lpm_oracle *o, double **out)
{
    double *b = o->box;
    double bx = b[1] - b[0], by = b[3] - b[2], bz = b[5] - b[4];
    double a = sqrt(bx * bx + by * by + bz * bz);
    double bt[6] = {-a, a, -a, a, -a, a};
    size_t cap = 0, cnt = 0;
    double *xyz = NULL;
#define PUSH(X, Y, Z)                                                                      \
    do {                                                                                   \
        double px = (X), py = (Y), pz = (Z);                                               \
        if (px >= b[0] && px <= b[1] && py >= b[2] && py <= b[3] && pz >= b[4] && pz <= b[5]) { \
            if (cnt == cap) {                                                              \
                cap = cap ? 2 * cap : 4096;                                                \
                xyz = (double *)realloc(xyz, cap * 3 * sizeof(double));                    \
            }                                                                              \
            xyz[3 * cnt] = px;                                                             \
            xyz[3 * cnt + 1] = py;                                                         \
            xyz[3 * cnt + 2] = pz;                                                         \
            cnt++;                                                                         \
        }                                                                                  \
    } while (0)
    if (o->lattice == 2) {
        double hx = 2 * o->radius, hy = hx, hz = hx;
        int pfr = 1 + (int)floor((bt[1] - bt[0]) / hx);
        int rows = 1 + (int)floor((bt[3] - bt[2]) / hy);
        int layers = 1 + (int)floor((bt[5] - bt[4]) / hz);
        for (int k = 1; k <= layers; k++) {
            double z = bt[4] + hz * (k - 1);
            for (int j = 1; j <= rows; j++) {
                double y = bt[2] + hy * (j - 1);
                for (int i = 1; i <= pfr; i++)
                    PUSH(b[0] + hx * (i - 1), y, z);
            }
        }
    } else if (o->lattice == 3) {
        double hx = 4 * o->radius / sqrt(2.0), hy = hx, hz = hx;
        int pfr = 1 + (int)floor((bt[1] - bt[0]) / hx);
        int rows = 1 + (int)floor((bt[3] - bt[2]) / (hy / 2.0));
        int layers = 1 + (int)floor((bt[5] - bt[4]) / (hz / 2.0));
        for (int k = 1; k <= layers; k++) {
            double z = bt[4] + hz / 2.0 * (k - 1);
            for (int j = 1; j <= rows; j++) {
                double y = bt[2] + hy / 2.0 * (j - 1);
                int full = ((k % 2 == 1) == (j % 2 == 1));
                if (full)
                    for (int i = 1; i <= pfr; i++)
                        PUSH(bt[0] + hx * (i - 1), y, z);
                else
                    for (int i = 1; i <= pfr - 1; i++)
                        PUSH(bt[0] + hx * (i - 1) + hx / 2.0, y, z);
            }
        }
    } else {
        return -1;
    }
#undef PUSH
    *out = xyz;
    return (int)cnt;
}

static void lattice_params(lpm_oracle *o)
{
    double r = o->radius;
    o->nn = 18;
    o->nafem = 60;
    o->cut1 = 2.0 * r;
    o->cut2 = 2.0 * sqrt(2.0) * r;
    if (o->lattice == 2) {
        o->nn1 = 6;
        o->nn2 = 12;
        o->vol = pow(2 * r, 3);
    } else {
        o->nn1 = 12;
        o->nn2 = 6;
        o->vol = 4.0 * sqrt(2.0) * pow(r, 3);
    }
}

/* searchNormalNeighbor, src/neighbor.c:9-46.  A cell grid replaces the
 * all-pairs loop; candidates are tested with the reference's expressions
 * and kept in ascending j, so the lists are identical. */
static void search_neighbors(lpm_oracle *o)
{
    int n = o->n, nn = o->nn;
    double c1 = 1.01 * o->cut1, c2 = 1.01 * o->cut2;
    double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
    for (int i = 0; i < n; i++)
        for (int d = 0; d < 3; d++) {
            double v = o->xyz[3 * i + d];
            lo[d] = v < lo[d] ? v : lo[d];
            hi[d] = v > hi[d] ? v : hi[d];
        }
    double h = c2 * 1.0001;
    int g[3];
    for (int d = 0; d < 3; d++) {
        g[d] = (int)((hi[d] - lo[d]) / h) + 1;
    }
    size_t ncell = (size_t)g[0] * g[1] * g[2];
    int *head = IALLOC(ncell + 1), *cell_of = IALLOC(n), *order = IALLOC(n);
    for (int i = 0; i < n; i++) {
        int c[3];
        for (int d = 0; d < 3; d++) {
            c[d] = (int)((o->xyz[3 * i + d] - lo[d]) / h);
            if (c[d] >= g[d])
                c[d] = g[d] - 1;
        }
        cell_of[i] = (c[2] * g[1] + c[1]) * g[0] + c[0];
        head[cell_of[i] + 1]++;
    }
    for (size_t c = 0; c < ncell; c++)
        head[c + 1] += head[c];
    int *fill = IALLOC(ncell);
    for (int i = 0; i < n; i++)
        order[head[cell_of[i]] + fill[cell_of[i]]++] = i;
    free(fill);
#pragma omp parallel for schedule(dynamic, 256)
    for (int i = 0; i < n; i++) {
        int cand[64], nc = 0;
        int ci = cell_of[i];
        int cx = ci % g[0], cy = (ci / g[0]) % g[1], cz = ci / (g[0] * g[1]);
        for (int dz = -1; dz <= 1; dz++)
            for (int dy = -1; dy <= 1; dy++)
                for (int dx = -1; dx <= 1; dx++) {
                    int x = cx + dx, y = cy + dy, z = cz + dz;
                    if (x < 0 || y < 0 || z < 0 || x >= g[0] || y >= g[1] || z >= g[2])
                        continue;
                    size_t c = ((size_t)z * g[1] + y) * g[0] + x;
                    for (int q = head[c]; q < head[c + 1]; q++) {
                        int j = order[q];
                        double ddx = o->xyz[3 * j] - o->xyz[3 * i];
                        double ddy = o->xyz[3 * j + 1] - o->xyz[3 * i + 1];
                        double ddz = o->xyz[3 * j + 2] - o->xyz[3 * i + 2];
                        double dis = sqrt(ddx * ddx + ddy * ddy + ddz * ddz);
                        int keep = ((dis < c1) && (j != i)) || ((dis > c1) && (dis < c2));
                        if (keep && nc < 64)
                            cand[nc++] = j;
                    }
                }
        /* ascending j, as the reference's j loop */
        for (int a = 1; a < nc; a++) {
            int v = cand[a], b = a - 1;
            while (b >= 0 && cand[b] > v) {
                cand[b + 1] = cand[b];
                b--;
            }
            cand[b + 1] = v;
        }
        int i1 = 0, i2 = 0, i3 = 0;
        for (int q = 0; q < nc && i3 < nn; q++) {
            int j = cand[q];
            double dis = sqrt((o->xyz[3 * j] - o->xyz[3 * i]) * (o->xyz[3 * j] - o->xyz[3 * i]) +
                              (o->xyz[3 * j + 1] - o->xyz[3 * i + 1]) * (o->xyz[3 * j + 1] - o->xyz[3 * i + 1]) +
                              (o->xyz[3 * j + 2] - o->xyz[3 * i + 2]) * (o->xyz[3 * j + 2] - o->xyz[3 * i + 2]));
            size_t b = (size_t)i * nn + i3;
            int s;
            if ((dis < c1) && (j != i)) {
                s = 0;
                if (i1 < o->nn1)
                    o->nbr1[(size_t)i * o->nn1 + i1++] = j;
            } else {
                s = 1;
                if (i2 < o->nn2)
                    o->nbr2[(size_t)i * o->nn2 + i2++] = j;
            }
            o->cs0x[b] = (o->xyz[3 * i] - o->xyz[3 * j]) / dis;
            o->cs0y[b] = (o->xyz[3 * i + 1] - o->xyz[3 * j + 1]) / dis;
            o->cs0z[b] = (o->xyz[3 * i + 2] - o->xyz[3 * j + 2]) / dis;
            o->L0[b] = dis;
            o->shell[b] = s;
            o->nbr[b] = j;
            i3++;
        }
        o->nb[i] = i3;
    }
    free(head);
    free(cell_of);
    free(order);
}

static int icmp(const void *a, const void *b)
{
    int x = *(const int *)a, y = *(const int *)b;
    return (x > y) - (x < y);
}

/* searchAFEMNeighbor, src/neighbor.c:49-141: conn = sorted unique union of
 * same-shell neighbours and their same-shell neighbours; K_pointer. */
static void search_afem(lpm_oracle *o)
{
    int n = o->n, nn = o->nn, w = o->nafem + 1;
#pragma omp parallel for schedule(dynamic, 256)
    for (int i = 0; i < n; i++) {
        int col[18 * 19], nc = 0, i1 = 0, i2 = 0;
        for (int j = 0; j < o->nb[i]; j++) {
            int s = o->shell[(size_t)i * nn + j];
            if (s == 0) {
                int p = o->nbr1[(size_t)i * o->nn1 + i1++];
                col[nc++] = p;
                for (int k = 0; k < o->nn1; k++) {
                    int q = o->nbr1[(size_t)p * o->nn1 + k];
                    if (q != -1)
                        col[nc++] = q;
                }
            } else {
                int p = o->nbr2[(size_t)i * o->nn2 + i2++];
                col[nc++] = p;
                for (int k = 0; k < o->nn2; k++) {
                    int q = o->nbr2[(size_t)p * o->nn2 + k];
                    if (q != -1)
                        col[nc++] = q;
                }
            }
        }
        qsort(col, nc, sizeof(int), icmp);
        int m = 0;
        for (int k = 0; k < nc; k++)
            if (m == 0 || col[k] != col[m - 1])
                col[m++] = col[k];
        if (m > w)
            m = w;
        for (int k = 0; k < m; k++)
            o->conn[(size_t)i * w + k] = col[k];
        o->nconn[i] = m;
    }
    o->kp1[0] = 0;
    for (int i = 0; i < n; i++) {
        int c = 0;
        for (int k = 0; k < o->nconn[i]; k++)
            if (o->conn[(size_t)i * w + k] >= i)
                c++;
        o->kp0[i] = c;
        o->kp1[i + 1] = o->kp1[i] + 9 * c - 3;
    }
    o->nnz = o->kp1[n];
}

/* reverse bond slot and the opposite-bond weight of the stress sums
 * (src/constitutive.c:541-559: 0.5 when the opposite bond exists and is
 * intact, else 1.0; damage_broken is 1 for every bond here). */
static void bond_tables(lpm_oracle *o)
{
    int n = o->n, nn = o->nn;
#pragma omp parallel for
    for (int i = 0; i < n; i++) {
        for (int j = 0; j < nn; j++) {
            size_t b = (size_t)i * nn + j;
            o->rev[b] = -1;
            o->opp[b] = 1.0;
            if (j >= o->nb[i])
                continue;
            int p = o->nbr[b];
            for (int q = 0; q < nn; q++)
                if (o->nbr[(size_t)p * nn + q] == i)
                    o->rev[b] = q;
            if (o->nb[i] == nn) {
                o->opp[b] = 0.5;
            } else {
                for (int m = 0; m < o->nb[i]; m++) {
                    size_t c = (size_t)i * nn + m;
                    if (fabs(o->cs0x[c] + o->cs0x[b]) < EPSP && fabs(o->cs0y[c] + o->cs0y[b]) < EPSP &&
                        fabs(o->cs0z[c] + o->cs0z[b]) < EPSP) {
                        o->opp[b] = 0.5;
                        break;
                    }
                }
            }
        }
    }
}

static void alloc_state(lpm_oracle *o)
{
    int n = o->n, nn = o->nn;
    size_t nb = (size_t)n * nn;
    o->xyz0 = DALLOC(3 * n);
    o->xyz_temp = DALLOC(3 * n);
    o->type = IALLOC(n);
    o->nb = IALLOC(n);
    o->nbr = IALLOC(nb);
    o->shell = IALLOC(nb);
    o->nbr1 = IALLOC((size_t)n * o->nn1);
    o->nbr2 = IALLOC((size_t)n * o->nn2);
    for (size_t k = 0; k < nb; k++)
        o->nbr[k] = o->shell[k] = -1;
    for (size_t k = 0; k < (size_t)n * o->nn1; k++)
        o->nbr1[k] = -1;
    for (size_t k = 0; k < (size_t)n * o->nn2; k++)
        o->nbr2[k] = -1;
    o->rev = IALLOC(nb);
    o->L0 = DALLOC(nb);
    o->cs0x = DALLOC(nb);
    o->cs0y = DALLOC(nb);
    o->cs0z = DALLOC(nb);
    o->dist = DALLOC(nb);
    o->Kn = DALLOC(nb);
    o->Tv = DALLOC(nb);
    o->opp = DALLOC(nb);
    o->conn = IALLOC((size_t)n * (o->nafem + 1));
    for (size_t k = 0; k < (size_t)n * (o->nafem + 1); k++)
        o->conn[k] = -1;
    o->nconn = IALLOC(n);
    o->kp0 = IALLOC(n + 1);
    o->kp1 = IALLOC(n + 1);
    o->knt = DALLOC(3 * n);
    o->G = DALLOC(n);
    o->sy = DALLOC(n);
    o->H = DALLOC(n);
    for (int s = 0; s < 3; s++) {
        o->dLp[s] = DALLOC(nb);
        o->alpha[s] = DALLOC(n);
        o->beta[s] = DALLOC(6 * n);
    }
    o->dlambda = DALLOC(n);
    o->dL = DALLOC(nb);
    o->Ssum = DALLOC(2 * n);
    o->Tsum = DALLOC(2 * n);
    o->csx = DALLOC(nb);
    o->csy = DALLOC(nb);
    o->csz = DALLOC(nb);
    o->F = DALLOC(nb);
    o->F_temp = DALLOC(nb);
    o->ddLp = DALLOC(nb);
    o->ddL = DALLOC(nb);
    o->ddS = DALLOC(2 * n);
    o->ddT = DALLOC(2 * n);
    o->Pin = DALLOC(3 * n);
    o->Pex = DALLOC(3 * n);
    o->Pex_temp = DALLOC(3 * n);
    o->residual = DALLOC(3 * n);
    o->reaction = DALLOC(3 * n);
    o->disp = DALLOC(3 * n);
    o->stress = DALLOC(6 * n);
    o->mask = IALLOC(3 * n);
    for (int k = 0; k < 3 * n; k++)
        o->mask[k] = 1;
    /* damage state as initMatrices leaves it (src/initialization.c:1120-1194):
     * intact bonds, no damage, nothing fixed; parameters as the reference's
     * main sets them (src/lpmc_project.c:239-244) */
    o->brk = DALLOC(nb);
    o->dw = DALLOC(nb);
    for (size_t k = 0; k < nb; k++)
        o->brk[k] = o->dw[k] = 1.0;
    o->dD[0] = DALLOC(nb);
    o->dD[1] = DALLOC(nb);
    o->dnl[0] = DALLOC(n);
    o->dnl[1] = DALLOC(n);
    o->dvis = DALLOC(n);
    o->nbc = IALLOC(n);
    o->fix = IALLOC(3 * n);
    for (int k = 0; k < 3 * n; k++)
        o->fix[k] = 1;
    o->dmg_L = 0.5;
    o->dmg_thr = 0.9;
    o->dmg_cA = 0.0;
    o->dmg_crit = 1.0e-2;
    o->dmg_nbreak = 20;
}

static int finish_setup(lpm_oracle *o)
{
    lattice_params(o);
    alloc_state(o);
    memcpy(o->xyz0, o->xyz, sizeof(double) * 3 * o->n);
    search_neighbors(o);
    memcpy(o->nbc, o->nb, sizeof(int) * o->n);
    search_afem(o);
    bond_tables(o);
    lo_csr_pattern(o);
    return o->n;
}

int lo_setup_lattice(lpm_oracle *o, int lattice, double radius, const double *box)
{
    o->lattice = lattice;
    o->radius = radius;
    memcpy(o->box, box, sizeof(o->box));
    double *xyz = NULL;
    int n = gen_lattice(o, &xyz);
    if (n <= 0)
        return -1;
    o->n = n;
    o->xyz = xyz;
    return finish_setup(o);
}

int lo_setup_particles(lpm_oracle *o, int lattice, double radius, int n, const double *xyz)
{
    o->lattice = lattice;
    o->radius = radius;
    o->n = n;
    o->xyz = DALLOC(3 * n);
    memcpy(o->xyz, xyz, sizeof(double) * 3 * n);
    return finish_setup(o);
}

void lo_set_types(lpm_oracle *o, const int *type) { memcpy(o->type, type, sizeof(int) * o->n); }

/* calcKnTv, src/stiffness.c:145-204 (SC, bond values averaged over the two
 * end particles) and :207-235 (FCC, the particle's own values); KnTve is
 * radius * mapping * [C11, C12, C44] computed per particle. */
void lo_set_material(lpm_oracle *o, const double *c11, const double *c12, const double *c44,
                     const double *sy, const double *H, double xi, int plmode)
{
    static const double msc[9] = {1, -1, -1, 0, 0, 1, 0, 1.0 / 18.0, -1.0 / 18.0};
    double mfcc[9] = {0, 0, sqrt(2.0), sqrt(2.0) / 4.0, -sqrt(2.0) / 4.0, -sqrt(2.0) / 4.0,
                      0, sqrt(2.0) / 24.0, -sqrt(2.0) / 24.0};
    const double *m = o->lattice == 2 ? msc : mfcc;
    int n = o->n, nn = o->nn;
    for (int i = 0; i < n; i++) {
        double ce[3] = {c11[i], c12[i], c44[i]};
        cblas_dgemm(CblasRowMajor, CblasNoTrans, CblasNoTrans, 3, 1, 3, o->radius, m, 3, ce, 1, 0.0,
                    o->knt + 3 * i, 1);
        o->G[i] = c44[i];
        o->sy[i] = sy ? sy[i] : 0.0;
        o->H[i] = H ? H[i] : 0.0;
    }
    for (int i = 0; i < n; i++)
        for (int j = 0; j < o->nb[i]; j++) {
            size_t b = (size_t)i * nn + j;
            int p = o->nbr[b], s = o->shell[b];
            if (o->lattice == 2) {
                o->Kn[b] = 0.5 * (o->knt[3 * i + s] + o->knt[3 * p + s]);
                o->Tv[b] = 0.5 * (o->knt[3 * i + 2] + o->knt[3 * p + 2]);
            } else {
                o->Kn[b] = o->knt[3 * i + s];
                o->Tv[b] = o->knt[3 * i + 2];
            }
        }
    o->xi = xi;
    o->plmode = plmode;
}

/* one particle's stretches and shell sums, src/lpm_basic.c:252-291 and
 * src/constitutive.c:501-514 (dLp from slot `plastic`) */
static void stretch_one(lpm_oracle *o, int i, const double *plastic, double *dL, double *S,
                        double *T, int store_cs)
{
    int nn = o->nn;
    S[0] = 0, T[0] = 0;
    S[1] = 0, T[1] = 0;
    for (int j = 0; j < o->nb[i]; j++) {
        size_t b = (size_t)i * nn + j;
        int p = o->nbr[b];
        double dx = o->xyz[3 * i] - o->xyz[3 * p];
        double dy = o->xyz[3 * i + 1] - o->xyz[3 * p + 1];
        double dz = o->xyz[3 * i + 2] - o->xyz[3 * p + 2];
        double dis = sqrt(dx * dx + dy * dy + dz * dz);
        double v = dis - o->L0[b];
        v -= plastic[b];
        v *= o->brk[b]; /* damage_broken */
        dL[j] = v;
        S[o->shell[b]] += v;
        T[o->shell[b]] += o->Tv[b] * v;
        if (store_cs) {
            o->csx[b] = dx / dis;
            o->csy[b] = dy / dis;
            o->csz[b] = dz / dis;
        }
    }
}

void lo_computedL(lpm_oracle *o)
{
    int n = o->n, nn = o->nn;
#pragma omp parallel for
    for (int i = 0; i < n; i++) {
        stretch_one(o, i, o->dLp[0], o->dL + (size_t)i * nn, o->Ssum + 2 * i, o->Tsum + 2 * i, 1);
        for (int j = 0; j < o->nb[i]; j++) {
            size_t b = (size_t)i * nn + j;
            int p = o->nbr[b];
            double dx = o->xyz[3 * i] - o->xyz[3 * p], dy = o->xyz[3 * i + 1] - o->xyz[3 * p + 1],
                   dz = o->xyz[3 * i + 2] - o->xyz[3 * p + 2];
            o->dist[b] = sqrt(dx * dx + dy * dy + dz * dz);
        }
    }
}

/* computeBondForceElastic(ii), src/constitutive.c:228-283, including its
 * writes to the shared per-particle arrays of ii and its neighbours. */
static void force_elastic_one(lpm_oracle *o, int ii)
{
    int nn = o->nn;
    int list[19], nl = 1;
    list[0] = ii;
    for (int k = 0; k < nn; k++)
        if (o->brk[(size_t)ii * nn + k] > EPSP && o->nbr[(size_t)ii * nn + k] != -1)
            list[nl++] = o->nbr[(size_t)ii * nn + k];
    for (int k = 0; k < nl; k++) {
        int i = list[k];
        stretch_one(o, i, o->dLp[0], o->dL + (size_t)i * nn, o->Ssum + 2 * i, o->Tsum + 2 * i, 1);
    }
    int i = ii;
    o->Pin[3 * i] = 0.0, o->Pin[3 * i + 1] = 0.0, o->Pin[3 * i + 2] = 0.0;
    for (int j = 0; j < o->nb[i]; j++) {
        size_t b = (size_t)i * nn + j;
        int p = o->nbr[b], s = o->shell[b];
        double f = 2.0 * o->Kn[b] * o->dL[b] + 0.5 * (o->Tsum[2 * i + s] + o->Tsum[2 * p + s]) +
                   0.5 * o->Tv[b] * (o->Ssum[2 * i + s] + o->Ssum[2 * p + s]);
        f *= o->brk[b]; /* damage_broken */
        o->F[b] = f;
        o->Pin[3 * i] += o->csx[b] * f;
        o->Pin[3 * i + 1] += o->csy[b] * f;
        o->Pin[3 * i + 2] += o->csz[b] * f;
    }
}

/* upper CSR structure written by calcStiffness3DFiniteDifference,
 * src/stiffness.c:486-515 (JK, IK 1-based). */
void lo_csr_pattern(lpm_oracle *o)
{
    int n = o->n, w = o->nafem + 1;
    free(o->IK);
    free(o->JK);
    free(o->K);
    o->IK = IALLOC(3 * n + 1);
    o->JK = IALLOC(o->nnz);
    o->K = DALLOC(o->nnz);
    for (int i = 0; i < n; i++) {
        int base = o->kp1[i], k0 = o->kp0[i], num1 = 0;
        for (int jid = 0; jid < o->nconn[i]; jid++) {
            int jj = o->conn[(size_t)i * w + jid];
            if (jj == i) {
                o->JK[base] = 3 * (jj + 1) - 2;
                o->JK[base + 1] = 3 * (jj + 1) - 1;
                o->JK[base + 2] = 3 * (jj + 1);
                o->JK[base + 3 * k0] = 3 * (jj + 1) - 1;
                o->JK[base + 3 * k0 + 1] = 3 * (jj + 1);
                o->JK[base + 6 * k0 - 1] = 3 * (jj + 1);
            } else if (jj > i) {
                num1++;
                o->JK[base + 3 * num1] = 3 * (jj + 1) - 2;
                o->JK[base + 3 * num1 + 1] = 3 * (jj + 1) - 1;
                o->JK[base + 3 * num1 + 2] = 3 * (jj + 1);
                o->JK[base + 3 * k0 + 3 * num1 - 1] = 3 * (jj + 1) - 2;
                o->JK[base + 3 * k0 + 3 * num1] = 3 * (jj + 1) - 1;
                o->JK[base + 3 * k0 + 3 * num1 + 1] = 3 * (jj + 1);
                o->JK[base + 6 * k0 + 3 * num1 - 3] = 3 * (jj + 1) - 2;
                o->JK[base + 6 * k0 + 3 * num1 - 2] = 3 * (jj + 1) - 1;
                o->JK[base + 6 * k0 + 3 * num1 - 1] = 3 * (jj + 1);
            }
        }
        o->IK[3 * i] = base + 1;
        o->IK[3 * i + 1] = base + 3 * k0 + 1;
        o->IK[3 * i + 2] = base + 6 * k0;
    }
    o->IK[3 * n] = o->kp1[n] + 1;
}

/* slot of column block `col` in the upper part of block row `row`:
 * returns num (1-based among conn > row), as src/stiffness.c:605-613. */
static int upper_num(const lpm_oracle *o, int row, int col)
{
    int w = o->nafem + 1, num = 0;
    for (int k = 0; k < o->nconn[row]; k++) {
        int c = o->conn[(size_t)row * w + k];
        if (c <= row)
            continue;
        num++;
        if (c == col)
            return num;
    }
    return -1;
}

static void scatter_block(lpm_oracle *o, int i, int jj, double Kl[3][3])
{
    double *K = o->K;
    if (jj == i) {
        int base = o->kp1[i], k0 = o->kp0[i];
        K[base] += Kl[0][0];
        K[base + 1] += Kl[0][1];
        K[base + 2] += Kl[0][2];
        K[base + 3 * k0] += Kl[1][1];
        K[base + 3 * k0 + 1] += Kl[1][2];
        K[base + 6 * k0 - 1] += Kl[2][2];
    } else if (jj > i) {
        int base = o->kp1[i], k0 = o->kp0[i], num1 = upper_num(o, i, jj);
        K[base + 3 * num1] += 0.5 * Kl[0][0];
        K[base + 3 * num1 + 1] += 0.5 * Kl[0][1];
        K[base + 3 * num1 + 2] += 0.5 * Kl[0][2];
        K[base + 3 * k0 + 3 * num1 - 1] += 0.5 * Kl[1][0];
        K[base + 3 * k0 + 3 * num1] += 0.5 * Kl[1][1];
        K[base + 3 * k0 + 3 * num1 + 1] += 0.5 * Kl[1][2];
        K[base + 6 * k0 + 3 * num1 - 3] += 0.5 * Kl[2][0];
        K[base + 6 * k0 + 3 * num1 - 2] += 0.5 * Kl[2][1];
        K[base + 6 * k0 + 3 * num1 - 1] += 0.5 * Kl[2][2];
    } else {
        int base = o->kp1[jj], k0 = o->kp0[jj], num2 = upper_num(o, jj, i);
        K[base + 3 * num2] += 0.5 * Kl[0][0];
        K[base + 3 * num2 + 1] += 0.5 * Kl[1][0];
        K[base + 3 * num2 + 2] += 0.5 * Kl[2][0];
        K[base + 3 * k0 + 3 * num2 - 1] += 0.5 * Kl[0][1];
        K[base + 3 * k0 + 3 * num2] += 0.5 * Kl[1][1];
        K[base + 3 * k0 + 3 * num2 + 1] += 0.5 * Kl[2][1];
        K[base + 6 * k0 + 3 * num2 - 3] += 0.5 * Kl[0][2];
        K[base + 6 * k0 + 3 * num2 - 2] += 0.5 * Kl[1][2];
        K[base + 6 * k0 + 3 * num2 - 1] += 0.5 * Kl[2][2];
    }
}

/* calcStiffness3DFiniteDifference(6), src/stiffness.c:384-516, for block
 * rows i0..i1-1, serially and in order (side effects included). */
void lo_fd_stiffness_range(lpm_oracle *o, int i0, int i1)
{
    if (i0 < 0)
        i0 = 0;
    if (i1 > o->n)
        i1 = o->n;
    int w = o->nafem + 1;
    double h = EPSP * o->radius;
    double *Kloc = DALLOC(3 * w * 3);
    for (int i = i0; i < i1; i++) {
        int nc = o->nconn[i];
        force_elastic_one(o, i);
        double f0[3] = {o->Pin[3 * i], o->Pin[3 * i + 1], o->Pin[3 * i + 2]};
        for (int jid = 0; jid < nc; jid++) {
            int p = o->conn[(size_t)i * w + jid];
            for (int r = 0; r < 3; r++) {
                double xt = o->xyz[3 * p + r];
                o->xyz[3 * p + r] = xt + h;
                force_elastic_one(o, i);
                o->xyz[3 * p + r] = xt;
                for (int s = 0; s < 3; s++)
                    Kloc[3 * nc * r + 3 * jid + s] = (o->Pin[3 * i + s] - f0[s]) / EPSP / o->radius;
            }
        }
        for (int jid = 0; jid < nc; jid++) {
            int jj = o->conn[(size_t)i * w + jid];
            double Kl[3][3];
            for (int r = 0; r < 3; r++)
                for (int s = 0; s < 3; s++)
                    Kl[r][s] = Kloc[3 * nc * s + 3 * jid + r];
            scatter_block(o, i, jj, Kl);
        }
    }
    free(Kloc);
}

/* Timing helper for the CPU baseline: calcStiffness3DFiniteDifference's
 * OpenMP loop over block rows (src/stiffness.c:388-516) on `threads` threads
 * (the reference's main runs it on nt_force = 3, src/lpmc_project.c:57,391)
 * for `count` rows spread evenly over the lattice.  Like the reference's
 * parallel loop, the row bodies write the shared per-particle arrays and the
 * matrix without synchronisation, so the state is not used afterwards.
 * Returns the wall time in seconds. */
double lo_fd_stiffness_timing(lpm_oracle *o, int count, int threads)
{
    if (count > o->n)
        count = o->n;
    if (count < 1)
        return 0.0;
    int w = o->nafem + 1;
    double h = EPSP * o->radius;
    long long stride = o->n / count;
    double t0 = omp_get_wtime();
#pragma omp parallel num_threads(threads)
    {
        double *Kloc = DALLOC(3 * w * 3);
#pragma omp for schedule(dynamic, 16)
        for (int k = 0; k < count; k++) {
            int i = (int)(k * stride);
            int nc = o->nconn[i];
            force_elastic_one(o, i);
            double f0[3] = {o->Pin[3 * i], o->Pin[3 * i + 1], o->Pin[3 * i + 2]};
            for (int jid = 0; jid < nc; jid++) {
                int p = o->conn[(size_t)i * w + jid];
                for (int r = 0; r < 3; r++) {
                    double xt = o->xyz[3 * p + r];
                    o->xyz[3 * p + r] = xt + h;
                    force_elastic_one(o, i);
                    o->xyz[3 * p + r] = xt;
                    for (int s2 = 0; s2 < 3; s2++)
                        Kloc[3 * nc * r + 3 * jid + s2] = (o->Pin[3 * i + s2] - f0[s2]) / EPSP / o->radius;
                }
            }
            for (int jid = 0; jid < nc; jid++) {
                int jj = o->conn[(size_t)i * w + jid];
                double Kl[3][3];
                for (int r = 0; r < 3; r++)
                    for (int s2 = 0; s2 < 3; s2++)
                        Kl[r][s2] = Kloc[3 * nc * s2 + 3 * jid + r];
                scatter_block(o, i, jj, Kl);
            }
        }
        free(Kloc);
    }
    return omp_get_wtime() - t0;
}

void lo_fd_stiffness(lpm_oracle *o)
{
    memset(o->K, 0, sizeof(double) * o->nnz);
    lo_fd_stiffness_range(o, 0, o->n);
}

/* setDispBC, src/boundary.c:12-45 */
void lo_set_disp_bc(lpm_oracle *o, int nbd, const lo_disp_bc *d)
{
    for (int i = 0; i < o->n; i++)
        for (int k = 0; k < nbd; k++)
            if (o->type[i] == d[k].type) {
                int c = d[k].flag == 'x' ? 0 : (d[k].flag == 'y' ? 1 : (d[k].flag == 'z' ? 2 : -1));
                if (c < 0)
                    continue;
                o->xyz[3 * i + c] += d[k].step;
                o->mask[3 * i + c] = 0;
            }
    int c = 0;
    for (int k = 0; k < 3 * o->n; k++)
        c += (o->mask[k] != 1);
    o->nreact = c;
}

/* setForceBC, src/boundary.c:48-70 */
void lo_set_force_bc(lpm_oracle *o, int nbf, const lo_force_bc *f)
{
    for (int k = 0; k < nbf; k++) {
        int cnt = 0;
        for (int i = 0; i < o->n; i++)
            cnt += (o->type[i] == f[k].type);
        for (int i = 0; i < o->n; i++)
            if (o->type[i] == f[k].type) {
                o->Pex[3 * i] += f[k].step1 / cnt;
                o->Pex[3 * i + 1] += f[k].step2 / cnt;
                o->Pex[3 * i + 2] += f[k].step3 / cnt;
            }
    }
}

/* setDispBC_stiffnessUpdate3D, src/boundary.c:159-281 */
void lo_bc_stiffness_update(lpm_oracle *o)
{
    int n = o->n, w = o->nafem + 1;
    double *K = o->K;
    double *diag = DALLOC(3 * n);
    for (int i = 0; i < n; i++) {
        diag[3 * i] = K[o->kp1[i]];
        diag[3 * i + 1] = K[o->kp1[i] + 3 * o->kp0[i]];
        diag[3 * i + 2] = K[o->kp1[i] + 6 * o->kp0[i] - 1];
    }
    double nd = cblas_dnrm2(3 * n, diag, 1);
    free(diag);
    for (int i = 0; i < n; i++) {
        for (int d = 0; d < 3; d++) {
            if (o->mask[3 * i + d] != 0 && o->fix[3 * i + d] != 0)
                continue;
            for (int jc = 0; jc < o->nconn[i]; jc++) {
                int c = o->conn[(size_t)i * w + jc];
                if (c > i)
                    continue;
                if (c == i) {
                    int b = o->kp1[i], k0 = o->kp0[i];
                    if (d == 0) {
                        for (int kk = b + 1; kk <= b + 3 * k0 - 1; kk++)
                            K[kk] = 0.0;
                        K[b] = nd;
                    } else if (d == 1) {
                        K[b + 1] = 0.0;
                        for (int kk = b + 3 * k0 + 1; kk <= b + 6 * k0 - 2; kk++)
                            K[kk] = 0.0;
                        K[b + 3 * k0] = nd;
                    } else {
                        K[b + 2] = 0.0;
                        K[b + 3 * k0 + 1] = 0.0;
                        for (int kk = b + 6 * k0 - 1; kk <= o->kp1[i + 1] - 1; kk++)
                            K[kk] = 0.0;
                        K[b + 6 * k0 - 1] = nd;
                    }
                } else {
                    int num2 = upper_num(o, c, i);
                    int b = o->kp1[c], k0 = o->kp0[c];
                    if (d == 0) {
                        K[b + 3 * num2] = 0.0;
                        K[b + 3 * k0 + 3 * num2 - 1] = 0.0;
                        K[b + 6 * k0 + 3 * num2 - 3] = 0.0;
                    } else if (d == 1) {
                        K[b + 3 * num2 + 1] = 0.0;
                        K[b + 3 * k0 + 3 * num2] = 0.0;
                        K[b + 6 * k0 + 3 * num2 - 2] = 0.0;
                    } else {
                        K[b + 3 * num2 + 2] = 0.0;
                        K[b + 3 * k0 + 3 * num2 + 1] = 0.0;
                        K[b + 6 * k0 + 3 * num2 - 1] = 0.0;
                    }
                }
            }
            o->residual[3 * i + d] = 0.0;
        }
    }
}

/* solverCG, src/solver.c:188-270: RCI CG (shared core) with the symmetric
 * upper-CSR product, x0 = 0, then xyz += disp.  Returns the iteration count,
 * or -1 on a solver failure (the reference prints and still moves xyz). */
int lo_solver_cg(lpm_oracle *o, double rtol_sq, double atol_sq)
{
    int n = 3 * o->n, rci = 0, ipar[128], it = 0;
    double dpar[128];
    double *tmp = DALLOC(4 * (size_t)n);
    sparse_matrix_t A;
    struct matrix_descr descr = {SPARSE_MATRIX_TYPE_SYMMETRIC, SPARSE_FILL_MODE_UPPER, SPARSE_DIAG_NON_UNIT};
    mkl_sparse_d_create_csr(&A, SPARSE_INDEX_BASE_ONE, n, n, o->IK, o->IK + 1, o->JK, o->K);
    memset(o->disp, 0, sizeof(double) * n);
    dcg_init(&n, o->disp, o->residual, &rci, ipar, dpar, tmp);
    ipar[4] = n;
    ipar[8] = 1;
    ipar[9] = 0;
    dpar[0] = rtol_sq;
    dpar[1] = atol_sq;
    dcg_check(&n, o->disp, o->residual, &rci, ipar, dpar, tmp);
    int fail = (rci != 0);
    while (!fail) {
        dcg(&n, o->disp, o->residual, &rci, ipar, dpar, tmp);
        if (rci == 0)
            break;
        if (rci == 1) {
            mkl_sparse_d_mv(SPARSE_OPERATION_NON_TRANSPOSE, 1.0, A, descr, tmp, 0.0, tmp + n);
            continue;
        }
        fail = 1;
    }
    dcg_get(&n, o->disp, o->residual, &rci, ipar, dpar, tmp, &it);
    mkl_sparse_destroy(A);
    free(tmp);
    for (int i = 0; i < o->n; i++)
        for (int d = 0; d < 3; d++)
            o->xyz[3 * i + d] += o->disp[3 * i + d];
    return fail ? -1 : it;
}

/* Timing helper for the CPU baseline: nit iterations of the reference's CG
 * (src/solver.c:188-270) on the current upper CSR and residual, with the
 * symmetric product spread over all OpenMP threads (per-thread accumulation,
 * as a threaded sparse BLAS would).  Returns the iterations run. */
int lo_cg_iterations(lpm_oracle *o, int nit)
{
    int n = 3 * o->n, nt = 1;
#ifdef _OPENMP
    nt = omp_get_max_threads();
#endif
    double *x = DALLOC(n), *r = DALLOC(n), *p = DALLOC(n), *q = DALLOC(n);
    double *acc = DALLOC((size_t)nt * n);
    memcpy(r, o->residual, sizeof(double) * n);
    memcpy(p, r, sizeof(double) * n);
    double rr = lpm_rci_dot(n, r, r);
    int it = 0;
    for (; it < nit; it++) {
#pragma omp parallel
        {
            int t = 0;
#ifdef _OPENMP
            t = omp_get_thread_num();
#endif
            double *a = acc + (size_t)t * n;
            memset(a, 0, sizeof(double) * n);
#pragma omp for schedule(static)
            for (int i = 0; i < n; i++)
                for (int k = o->IK[i] - 1; k < o->IK[i + 1] - 1; k++) {
                    int j = o->JK[k] - 1;
                    a[i] += o->K[k] * p[j];
                    if (j != i)
                        a[j] += o->K[k] * p[i];
                }
#pragma omp for schedule(static)
            for (int i = 0; i < n; i++) {
                double s = 0.0;
                for (int u = 0; u < nt; u++)
                    s += acc[(size_t)u * n + i];
                q[i] = s;
            }
        }
        double pq = 0.0, rr2 = 0.0;
#pragma omp parallel for reduction(+ : pq)
        for (int i = 0; i < n; i++)
            pq += p[i] * q[i];
        double al = pq != 0.0 ? rr / pq : 0.0;
#pragma omp parallel for reduction(+ : rr2)
        for (int i = 0; i < n; i++) {
            x[i] += al * p[i];
            r[i] -= al * q[i];
            rr2 += r[i] * r[i];
        }
        double be = rr != 0.0 ? rr2 / rr : 0.0;
        rr = rr2;
#pragma omp parallel for
        for (int i = 0; i < n; i++)
            p[i] = r[i] + be * p[i];
    }
    free(x);
    free(r);
    free(p);
    free(q);
    free(acc);
    return it;
}

/* opp_flag of bond b of particle i as the force and stress routines compute
 * it (src/constitutive.c:532-551, src/lpm_basic.c:70-90): 0.5 when i keeps
 * all its bonds, else 0.5 if the bond has an opposite bond that is intact,
 * 1.0 otherwise.  Equal to the setup table o->opp while no bond is broken. */
static double opp_now(const lpm_oracle *o, int i, size_t b)
{
    int nn = o->nn;
    if (o->nbc[i] == nn)
        return 0.5;
    for (int m = 0; m < o->nb[i]; m++) {
        size_t c = (size_t)i * nn + m;
        if (fabs(o->cs0x[c] + o->cs0x[b]) < EPSP && fabs(o->cs0y[c] + o->cs0y[b]) < EPSP &&
            fabs(o->cs0z[c] + o->cs0z[b]) < EPSP)
            return o->brk[c] <= EPSP ? 1.0 : 0.5;
    }
    return 1.0;
}

/* computeStress, src/lpm_basic.c:53-109 (stress tensor only) */
static void stress_all(lpm_oracle *o)
{
    int n = o->n, nn = o->nn;
#pragma omp parallel for
    for (int i = 0; i < n; i++) {
        double *st = o->stress + 6 * i;
        for (int k = 0; k < 6; k++)
            st[k] = 0.0;
        for (int j = 0; j < o->nb[i]; j++) {
            size_t b = (size_t)i * nn + j;
            double w = opp_now(o, i, b) / o->vol * o->L0[b] * o->F[b];
            st[0] += w * o->csx[b] * o->csx[b];
            st[1] += w * o->csy[b] * o->csy[b];
            st[2] += w * o->csz[b] * o->csz[b];
            st[3] += w * o->csy[b] * o->csz[b];
            st[4] += w * o->csx[b] * o->csz[b];
            st[5] += w * o->csx[b] * o->csy[b];
        }
    }
}

/* computeBondForceIncrementalUpdating, src/constitutive.c:167-225 (plmode 4):
 * F = F_temp + elastic increment from xyz_temp -> xyz, with the stored
 * (previous) unit vectors. */
static void force_predictor(lpm_oracle *o)
{
    int n = o->n, nn = o->nn;
#pragma omp parallel for
    for (int i = 0; i < n; i++) {
        o->ddS[2 * i] = 0, o->ddT[2 * i] = 0;
        o->ddS[2 * i + 1] = 0, o->ddT[2 * i + 1] = 0;
        for (int j = 0; j < o->nb[i]; j++) {
            size_t b = (size_t)i * nn + j;
            int p = o->nbr[b];
            const double *a0 = o->xyz_temp + 3 * i, *b0 = o->xyz_temp + 3 * p;
            const double *a1 = o->xyz + 3 * i, *b1 = o->xyz + 3 * p;
            double d0 = sqrt((a0[0] - b0[0]) * (a0[0] - b0[0]) + (a0[1] - b0[1]) * (a0[1] - b0[1]) +
                             (a0[2] - b0[2]) * (a0[2] - b0[2]));
            double d1 = sqrt((a1[0] - b1[0]) * (a1[0] - b1[0]) + (a1[1] - b1[1]) * (a1[1] - b1[1]) +
                             (a1[2] - b1[2]) * (a1[2] - b1[2]));
            double v = o->brk[b] * (d1 - d0);
            o->ddL[b] = v;
            o->ddS[2 * i + o->shell[b]] += v;
            o->ddT[2 * i + o->shell[b]] += o->Tv[b] * v;
        }
    }
#pragma omp parallel for
    for (int i = 0; i < n; i++) {
        o->Pin[3 * i] = 0.0, o->Pin[3 * i + 1] = 0.0, o->Pin[3 * i + 2] = 0.0;
        for (int j = 0; j < o->nb[i]; j++) {
            size_t b = (size_t)i * nn + j;
            int p = o->nbr[b], s = o->shell[b];
            double f = o->F_temp[b] + 2.0 * o->Kn[b] * o->ddL[b] + 0.5 * (o->ddT[2 * i + s] + o->ddT[2 * p + s]) +
                       0.5 * o->Tv[b] * (o->ddS[2 * i + s] + o->ddS[2 * p + s]);
            f *= o->brk[b]; /* damage_broken */
            o->F[b] = f;
            o->Pin[3 * i] += o->csx[b] * f;
            o->Pin[3 * i + 1] += o->csy[b] * f;
            o->Pin[3 * i + 2] += o->csz[b] * f;
        }
    }
}

/* stress sums of one particle from bond forces computed with its own shell
 * sums (src/constitutive.c:526-568) */
static void trial_stress(const lpm_oracle *o, int i, const double *dL, const double *S,
                         const double *T, const double *cx, const double *cy, const double *cz,
                         double st[6])
{
    int nn = o->nn;
    for (int k = 0; k < 6; k++)
        st[k] = 0.0;
    for (int j = 0; j < o->nb[i]; j++) {
        size_t b = (size_t)i * nn + j;
        int s = o->shell[b];
        double fij = 2.0 * o->Kn[b] * dL[j] + T[s] + o->Tv[b] * S[s];
        fij *= o->dw[b]; /* damage_w */
        double w = opp_now(o, i, b) / o->vol * o->L0[b] * fij;
        st[0] += w * cx[j] * cx[j];
        st[1] += w * cy[j] * cy[j];
        st[2] += w * cz[j] * cz[j];
        st[3] += w * cy[j] * cz[j];
        st[4] += w * cx[j] * cz[j];
        st[5] += w * cx[j] * cy[j];
    }
}

static void unit_vectors(const lpm_oracle *o, int i, double *cx, double *cy, double *cz)
{
    int nn = o->nn;
    for (int j = 0; j < o->nb[i]; j++) {
        int p = o->nbr[(size_t)i * nn + j];
        double dx = o->xyz[3 * i] - o->xyz[3 * p], dy = o->xyz[3 * i + 1] - o->xyz[3 * p + 1],
               dz = o->xyz[3 * i + 2] - o->xyz[3 * p + 2];
        double dis = sqrt(dx * dx + dy * dy + dz * dz);
        cx[j] = dx / dis;
        cy[j] = dy / dis;
        cz[j] = dz / dis;
    }
}

/* J2 radial return for particle i, src/constitutive.c:517-621: writes the
 * new plastic stretch (slot 2), alpha, beta, dlambda. */
static void j2_return_one(lpm_oracle *o, int i)
{
    int nn = o->nn;
    double dL[18], S[2], T[2], cx[18], cy[18], cz[18], st[6], dpl[6] = {0};
    stretch_one(o, i, o->dLp[0], dL, S, T, 0);
    unit_vectors(o, i, cx, cy, cz);
    trial_stress(o, i, dL, S, T, cx, cy, cz, st);
    double temp = 1.0 / 3.0 * (st[0] + st[1] + st[2]);
    for (int k = 0; k < 3; k++)
        st[k] -= temp;
    const double *beta0 = o->beta[0] + 6 * i;
    double beta[6];
    for (int k = 0; k < 6; k++) {
        st[k] -= beta0[k];
        beta[k] = beta0[k];
    }
    double seq = 0.0;
    for (int k = 0; k < 6; k++) {
        if (k < 3)
            seq += st[k] * st[k];
        else
            seq += 2.0 * st[k] * st[k];
    }
    seq = sqrt(3.0 / 2.0 * seq);
    double alpha = o->alpha[0][i], dlam = 0.0;
    double yf = seq - (o->sy[i] + (1.0 - o->xi) * o->H[i] * alpha);
    if (yf > 0.0)
        dlam = yf / (3 * o->G[i] + o->H[i]);
    alpha += dlam;
    for (int k = 0; k < 6; k++)
        if (fabs(seq) > EPSP) {
            dpl[k] = dlam * 1.5 * st[k] / seq;
            beta[k] += 2. / 3. * o->xi * o->H[i] * dpl[k];
        }
    for (int j = 0; j < nn; j++) {
        size_t b = (size_t)i * nn + j;
        double add = 0.0;
        if (j < o->nb[i]) {
            add = o->L0[b] * (dpl[0] * cx[j] * cx[j] + dpl[1] * cy[j] * cy[j] + dpl[2] * cz[j] * cz[j] +
                              2 * dpl[3] * cy[j] * cz[j] + 2 * dpl[4] * cx[j] * cz[j] +
                              2 * dpl[5] * cx[j] * cy[j]);
            add *= o->brk[b]; /* damage_broken */
            o->ddLp[b] = add;
        }
        o->dLp[2][b] = o->brk[b] * (o->dLp[0][b] + add);
    }
    for (int k = 0; k < 6; k++)
        o->beta[2][6 * i + k] = beta[k];
    o->alpha[2][i] = alpha;
    o->dlambda[i] = dlam;
}

/* ---------------------------------------------------------------------- */
/* crystal plasticity (plmode 1) */

/* slipSysDefine3D for lattice 3, src/initialization.c:565-637: the 24 signed
 * {111}<110> systems in the reference's plane/direction order. */
static void fcc_slip_systems(lpm_oracle *o)
{
    static const int pl[4][3] = {{1, 1, 1}, {-1, 1, 1}, {1, -1, 1}, {-1, -1, 1}};
    static const int dir[4][6][3] = {
        {{1, -1, 0}, {-1, 1, 0}, {-1, 0, 1}, {1, 0, -1}, {0, 1, -1}, {0, -1, 1}},
        {{1, 0, 1}, {-1, 0, -1}, {-1, -1, 0}, {1, 1, 0}, {0, 1, -1}, {0, -1, 1}},
        {{-1, 0, 1}, {1, 0, -1}, {0, -1, -1}, {0, 1, 1}, {1, 1, 0}, {-1, -1, 0}},
        {{-1, 1, 0}, {1, -1, 0}, {1, 0, 1}, {-1, 0, -1}, {0, -1, -1}, {0, 1, 1}}};
    double a3 = 1 / sqrt(3), a2 = 1 / sqrt(2);
    int m = 0;
    for (int p = 0; p < 4; p++)
        for (int d = 0; d < 6; d++, m++) {
            double nv[3], sv[3];
            for (int k = 0; k < 3; k++) {
                nv[k] = pl[p][k] * a3;
                sv[k] = dir[p][d][k] * a2;
            }
            o->sch[m][0] = nv[0] * sv[0];
            o->sch[m][1] = nv[1] * sv[1];
            o->sch[m][2] = nv[2] * sv[2];
            o->sch[m][3] = nv[1] * sv[2] + nv[2] * sv[1];
            o->sch[m][4] = nv[0] * sv[2] + nv[2] * sv[0];
            o->sch[m][5] = nv[0] * sv[1] + nv[1] * sv[0];
        }
    o->nslip = 24;
}

void lo_set_cp(lpm_oracle *o, const double *cp)
{
    o->cp_tau0 = cp[0];
    o->cp_taus = cp[1];
    o->cp_h0 = cp[2];
    o->cp_p = cp[3];
    o->cp_q = cp[4];
    o->cp_eta = cp[5];
    o->cp_maxloop = cp[6];
    o->dtime = cp[7];
}

static double proj(const double *sc, double cx, double cy, double cz)
{
    return cx * cx * sc[0] + cy * cy * sc[1] + cz * cz * sc[2] + cy * cz * sc[3] + cx * cz * sc[4] +
           cx * cy * sc[5];
}

/* computeCab, src/constitutive.c:1864-1917 (uses the initial geometry). */
static void compute_cab(lpm_oracle *o)
{
    int n = o->n, nn = o->nn, ns = o->nslip;
#pragma omp parallel for
    for (int i = 0; i < n; i++) {
        for (int m = 0; m < ns; m++)
            for (int q = 0; q < ns; q++) {
                double ls[2] = {0, 0};
                for (int j = 0; j < o->nb[i]; j++) {
                    size_t b = (size_t)i * nn + j;
                    ls[o->shell[b]] += o->Tv[b] * o->dist[b] * proj(o->sch[q], o->csx[b], o->csy[b], o->csz[b]);
                }
                double c = 0.;
                for (int j = 0; j < o->nb[i]; j++) {
                    size_t b = (size_t)i * nn + j;
                    double dfdg = -2.0 * o->Kn[b] * o->dist[b] * proj(o->sch[q], o->csx[b], o->csy[b], o->csz[b]) -
                                  2.0 * ls[o->shell[b]];
                    c += -o->opp[b] / o->vol * o->dist[b] * dfdg * proj(o->sch[m], o->csx[b], o->csy[b], o->csz[b]);
                }
                o->Cab[(size_t)i * ns * ns + m * ns + q] = c;
            }
    }
}

/* computeBondForceCPMiehe return map for particle i,
 * src/constitutive.c:938-1318.  Writes slot 2 of dLp, cp_gy, cp_A, cp_A_single. */
static void cp_return_one(lpm_oracle *o, int i)
{
    int nn = o->nn, ns = o->nslip, nbi = o->nb[i];
    double dL[18], S[2], T[2], cx[18], cy[18], cz[18], st[6];
    double xdL[18], xS[2], xT[2], ddlp[18] = {0};
    double gamma[MAXSLIP], r[MAXSLIP], rr[MAXSLIP], D[MAXSLIP * MAXSLIP], yfn[MAXSLIP];
    double xgy[MAXSLIP], dgy[MAXSLIP];
    int ipiv[MAXSLIP];
    int *J = o->Jact + (size_t)i * ns;
    double *RSS = o->cp_RSS + (size_t)i * ns;
    const double *Cab = o->Cab + (size_t)i * ns * ns;
    stretch_one(o, i, o->dLp[0], dL, S, T, 0);
    unit_vectors(o, i, cx, cy, cz);
    for (int j = 0; j < nbi; j++)
        xdL[j] = dL[j];
    xS[0] = S[0], xS[1] = S[1], xT[0] = T[0], xT[1] = T[1];
    const double *gy0 = o->cp_gy[0] + (size_t)i * ns;
    double A0 = o->cp_A[0][i];
    double xA = A0, dA = 0.0;
    for (int m = 0; m < ns; m++) {
        xgy[m] = gy0[m];
        dgy[m] = 0.0;
        gamma[m] = 0.0;
    }
    trial_stress(o, i, xdL, xS, xT, cx, cy, cz, st);
    double tmax = 0.0;
    for (int m = 0; m < ns; m++) {
        RSS[m] = st[0] * o->sch[m][0] + st[1] * o->sch[m][1] + st[2] * o->sch[m][2] + st[3] * o->sch[m][3] +
                 st[4] * o->sch[m][4] + st[5] * o->sch[m][5];
        yfn[m] = RSS[m] - gy0[m];
        if (yfn[m] > tmax)
            tmax = yfn[m];
    }
    if (tmax <= EPSP) {
        for (int j = 0; j < nbi; j++)
            ddlp[j] = 0.0;
        dA = 0.0;
        for (int m = 0; m < ns; m++) {
            J[m] = 0;
            dgy[m] = 0.0;
        }
    } else {
        int nouter = 0;
        for (int m = 0; m < ns; m++)
            J[m] = 0;
        double dts = o->cp_taus - o->cp_tau0;
        for (;;) {
            nouter++;
            double nr = 1.0;
            for (int m = 0; m < ns; m++)
                gamma[m] = r[m] = rr[m] = 0.0;
            memset(D, 0, sizeof(double) * ns * ns);
            int ninner = 0;
            do {
                ninner++;
                double dpl[6] = {0};
                for (int s = 0; s < ns; s++)
                    for (int k = 0; k < 6; k++)
                        dpl[k] += J[s] * gamma[s] * o->sch[s][k];
                xS[0] = 0, xT[0] = 0;
                xS[1] = 0, xT[1] = 0;
                for (int j = 0; j < nbi; j++) {
                    size_t b = (size_t)i * nn + j;
                    double v = o->L0[b] * (dpl[0] * cx[j] * cx[j] + dpl[1] * cy[j] * cy[j] + dpl[2] * cz[j] * cz[j] +
                                           dpl[3] * cy[j] * cz[j] + dpl[4] * cx[j] * cz[j] + dpl[5] * cx[j] * cy[j]);
                    v *= o->brk[b]; /* damage_broken */
                    ddlp[j] = v;
                    xdL[j] = dL[j] - v;
                    xS[o->shell[b]] += xdL[j];
                    xT[o->shell[b]] += o->Tv[b] * xdL[j];
                }
                trial_stress(o, i, xdL, xS, xT, cx, cy, cz, st);
                dA = 0.0;
                for (int s = 0; s < ns; s++)
                    dA += gamma[s];
                xA = A0 + dA;
                double ch = cosh(o->cp_h0 * xA / dts);
                double hh = o->cp_h0 / (ch * ch);
                double hp = -2.0 * o->cp_h0 * o->cp_h0 / dts * tanh(o->cp_h0 * xA / dts) * hh;
                for (int a = 0; a < ns; a++) {
                    double t1 = 0.0;
                    for (int b2 = 0; b2 < ns; b2++) {
                        double hab = (a == b2) ? hh : o->cp_q * hh;
                        t1 += J[b2] * hab * gamma[b2];
                    }
                    dgy[a] = J[a] * t1;
                    xgy[a] = gy0[a] + dgy[a];
                }
                for (int m = 0; m < ns; m++) {
                    double t1 = pow(1. + gamma[m] * o->cp_eta / o->dtime, 1. / o->cp_p);
                    RSS[m] = st[0] * o->sch[m][0] + st[1] * o->sch[m][1] + st[2] * o->sch[m][2] +
                             st[3] * o->sch[m][3] + st[4] * o->sch[m][4] + st[5] * o->sch[m][5];
                    r[m] = J[m] * (RSS[m] - xgy[m] * t1);
                    rr[m] = r[m];
                }
                for (int m = 0; m < ns; m++)
                    for (int q = 0; q < ns; q++) {
                        if (J[m] == 1 && J[q] == 1) {
                            double hs = 0.0;
                            for (int d = 0; d < ns; d++) {
                                double hd;
                                if (m == d && q == d)
                                    hd = hh + hp * gamma[d];
                                else if (m == d && q != d)
                                    hd = hp * gamma[d];
                                else if (m != d && q == d)
                                    hd = o->cp_q * (hh + hp * gamma[d]);
                                else
                                    hd = o->cp_q * hp * gamma[d];
                                hs += J[d] * hd;
                            }
                            double t1 = xgy[m] * (o->cp_eta / o->cp_p / o->dtime *
                                                  pow(1. + o->cp_eta * gamma[m] / o->dtime, (1. - o->cp_p) / o->cp_p));
                            double t2 = hs * pow(1. + o->cp_eta * gamma[m] / o->dtime, (1. / o->cp_p));
                            if (m == q)
                                D[m * ns + q] = Cab[m * ns + q] + t1 + t2;
                            else
                                D[m * ns + q] = Cab[m * ns + q] + t2;
                        } else if (m == q) {
                            D[m * ns + q] = 1.0;
                        }
                    }
                int info = LAPACKE_dgesv(LAPACK_ROW_MAJOR, ns, 1, D, ns, ipiv, rr, 1);
                if (info > 0) {
                    o->error = 1; /* the reference exits here (src/constitutive.c:1216-1221) */
                    break;
                }
                for (int m = 0; m < ns; m++)
                    gamma[m] += J[m] * rr[m];
                nr = cblas_dnrm2(ns, r, 1);
            } while (nr > TOLITER_ && ninner < MAXSMALL_);
            int jflag = 0, mi = -1;
            double my = 0.0;
            for (int m = 0; m < ns; m++) {
                yfn[m] = RSS[m] - xgy[m];
                if (J[m] == 1 && gamma[m] <= 0.0 && yfn[m] < my) {
                    my = yfn[m];
                    mi = m;
                }
            }
            if (mi != -1) {
                J[mi] = 0;
                jflag = 1;
            }
            if (jflag == 1)
                continue;
            int ma = -1;
            double mxy = 0.0;
            for (int m = 0; m < ns; m++)
                if (J[m] == 0 && yfn[m] > 0.0 && yfn[m] > mxy) {
                    mxy = yfn[m];
                    ma = m;
                }
            if (ma != -1) {
                J[ma] = 1;
                jflag = 2;
            }
            if (jflag == 2 && nouter < o->cp_maxloop)
                continue;
            break;
        }
    }
    for (int j = 0; j < nn; j++) {
        size_t b = (size_t)i * nn + j;
        o->dLp[2][b] = o->brk[b] * (o->dLp[0][b] + (j < nbi ? ddlp[j] : 0.0));
    }
    for (int s = 0; s < ns; s++) {
        double das = J[s] * gamma[s];
        o->cp_gy[2][(size_t)i * ns + s] = xgy[s];
        o->cp_As[2][(size_t)i * ns + s] = o->cp_As[0][(size_t)i * ns + s] + das;
    }
    o->cp_A[2][i] = xA;
}

/* bond forces from the re-summed dilatation (src/constitutive.c:624-667):
 * phase 2 (stretches with slot-2 plastic stretch) then phase 3. */
static void final_forces(lpm_oracle *o)
{
    int n = o->n, nn = o->nn;
#pragma omp parallel for
    for (int i = 0; i < n; i++)
        stretch_one(o, i, o->dLp[2], o->dL + (size_t)i * nn, o->Ssum + 2 * i, o->Tsum + 2 * i, 1);
#pragma omp parallel for
    for (int i = 0; i < n; i++) {
        o->Pin[3 * i] = 0.0, o->Pin[3 * i + 1] = 0.0, o->Pin[3 * i + 2] = 0.0;
        for (int j = 0; j < o->nb[i]; j++) {
            size_t b = (size_t)i * nn + j;
            int p = o->nbr[b], s = o->shell[b];
            double dla = 0.5 * (o->dL[b] + o->dL[(size_t)p * nn + o->rev[b]]);
            double f = 2.0 * o->Kn[b] * dla + 0.5 * (o->Tsum[2 * i + s] + o->Tsum[2 * p + s]) +
                       0.5 * o->Tv[b] * (o->Ssum[2 * i + s] + o->Ssum[2 * p + s]);
            f *= o->dw[b]; /* damage_w */
            o->F[b] = f;
            o->Pin[3 * i] += o->csx[b] * f;
            o->Pin[3 * i + 1] += o->csy[b] * f;
            o->Pin[3 * i + 2] += o->csz[b] * f;
        }
    }
}

/* switchStateV, src/constitutive.c:10-85 */
void lo_switch_state(lpm_oracle *o, int flag)
{
    int from = flag == 0 ? 1 : (flag == 1 ? 0 : 2), to = flag == 1 ? 1 : 0;
    size_t nb = (size_t)o->n * o->nn, ns = (size_t)o->n * o->nslip;
    memcpy(o->dLp[to], o->dLp[from], nb * sizeof(double));
    memcpy(o->alpha[to], o->alpha[from], o->n * sizeof(double));
    memcpy(o->beta[to], o->beta[from], 6 * (size_t)o->n * sizeof(double));
    if (o->nslip) {
        memcpy(o->cp_gy[to], o->cp_gy[from], ns * sizeof(double));
        memcpy(o->cp_As[to], o->cp_As[from], ns * sizeof(double));
        memcpy(o->cp_A[to], o->cp_A[from], o->n * sizeof(double));
    }
    if (flag == 0 || flag == 1) { /* damage_D, damage_nonlocal: slots 0 and 1 only */
        memcpy(o->dD[to], o->dD[from], nb * sizeof(double));
        memcpy(o->dnl[to], o->dnl[from], o->n * sizeof(double));
    }
}

/* computeBondForceGeneral, src/constitutive.c:88-146 for plmode 0, 1, 4, 6 */
void lo_force(lpm_oracle *o, int plmode)
{
    int n = o->n;
    if (plmode == 4) {
        force_predictor(o);
    } else if (plmode == 6) {
        memcpy(o->dLp[2], o->dLp[0], sizeof(double) * n * o->nn);
        memcpy(o->alpha[2], o->alpha[0], sizeof(double) * n);
        memcpy(o->beta[2], o->beta[0], sizeof(double) * 6 * n);
        int nn = o->nn;
#pragma omp parallel for
        for (int i = 0; i < n; i++)
            stretch_one(o, i, o->dLp[0], o->dL + (size_t)i * nn, o->Ssum + 2 * i, o->Tsum + 2 * i, 1);
#pragma omp parallel for
        for (int i = 0; i < n; i++) {
            o->Pin[3 * i] = 0.0, o->Pin[3 * i + 1] = 0.0, o->Pin[3 * i + 2] = 0.0;
            for (int j = 0; j < o->nb[i]; j++) {
                size_t b = (size_t)i * nn + j;
                int p = o->nbr[b], s = o->shell[b];
                double f = 2.0 * o->Kn[b] * o->dL[b] + 0.5 * (o->Tsum[2 * i + s] + o->Tsum[2 * p + s]) +
                           0.5 * o->Tv[b] * (o->Ssum[2 * i + s] + o->Ssum[2 * p + s]);
                f *= o->brk[b]; /* damage_broken */
                o->F[b] = f;
                o->Pin[3 * i] += o->csx[b] * f;
                o->Pin[3 * i + 1] += o->csy[b] * f;
                o->Pin[3 * i + 2] += o->csz[b] * f;
            }
        }
    } else if (plmode == 0) {
#pragma omp parallel for schedule(dynamic, 64)
        for (int i = 0; i < n; i++)
            j2_return_one(o, i);
        final_forces(o);
    } else if (plmode == 1) {
#pragma omp parallel for schedule(dynamic, 16)
        for (int i = 0; i < n; i++)
            cp_return_one(o, i);
        final_forces(o);
    }
    stress_all(o);
    lo_switch_state(o, 2);
}

/* updateRR, src/stiffness.c:519-534 */
void lo_update_rr(lpm_oracle *o)
{
    int ii = 0;
    for (int i = 0; i < o->n; i++)
        for (int k = 0; k < 3; k++) {
            o->residual[3 * i + k] = o->mask[3 * i + k] * (o->Pex[3 * i + k] - o->Pin[3 * i + k]);
            if (o->mask[3 * i + k] == 0)
                o->reaction[ii++] = o->Pin[3 * i + k];
        }
}

void lo_init_state(lpm_oracle *o)
{
    int n = o->n;
    lo_computedL(o);
    if (o->lattice == 3) {
        fcc_slip_systems(o);
        size_t ns = (size_t)n * o->nslip;
        for (int s = 0; s < 3; s++) {
            o->cp_gy[s] = DALLOC(ns);
            o->cp_As[s] = DALLOC(ns);
            o->cp_A[s] = DALLOC(n);
            for (size_t k = 0; k < ns; k++)
                o->cp_gy[s][k] = o->cp_tau0;
        }
        o->Cab = DALLOC(ns * o->nslip);
        o->cp_RSS = DALLOC(ns);
        o->Jact = IALLOC(ns);
        compute_cab(o);
    }
}

/* one load step, src/lpmc_project.c:385-471 (damage and strain output
 * skipped; Newton and CG tolerances are parameters) */
int lo_load_step(lpm_oracle *o, int nbd, const lo_disp_bc *d, int nbf, const lo_force_bc *f,
                 double newton_tol, int maxiter, double cg_rtol_sq, double cg_atol_sq,
                 double *stats)
{
    int n = o->n;
    memcpy(o->xyz_temp, o->xyz, sizeof(double) * 3 * n);
    memcpy(o->F_temp, o->F, sizeof(double) * n * o->nn);
    memcpy(o->Pex_temp, o->Pex, sizeof(double) * 3 * n);
    lo_fd_stiffness(o);
    lo_set_disp_bc(o, nbd, d);
    lo_set_force_bc(o, nbf, f);
    lo_force(o, 4);
    lo_update_rr(o);
    double nr = cblas_dnrm2(3 * n, o->residual, 1);
    double nreac = cblas_dnrm2(o->nreact, o->reaction, 1);
    double tolm = nr > nreac ? nr : nreac, nr0 = nr;
    int ni = 0, cg = 0;
    while (nr > newton_tol * tolm && ni < maxiter) {
        lo_switch_state(o, 0);
        lo_bc_stiffness_update(o);
        int it = lo_solver_cg(o, cg_rtol_sq, cg_atol_sq);
        cg += it > 0 ? it : 0;
        lo_force(o, o->plmode);
        lo_update_rr(o);
        ni++;
        nr = cblas_dnrm2(3 * n, o->residual, 1);
    }
    lo_switch_state(o, 1);
    if (stats) {
        stats[0] = ni;
        stats[1] = nr0;
        stats[2] = nreac;
        stats[3] = nr;
        stats[4] = cg;
    }
    return ni;
}

/* ---------------------------------------------------------------------- */
/* damage and bond breaking (src/constitutive.c:149-164, :1399-1862) */

void lo_set_damage(lpm_oracle *o, double L, double threshold, double cA, double crit_bstrain, int nbreak)
{
    o->dmg_L = L;
    o->dmg_thr = threshold;
    o->dmg_cA = cA;
    o->dmg_crit = crit_bstrain;
    o->dmg_nbreak = nbreak;
}

static void log_bond(lpm_oracle *o, int i, int j)
{
    if (o->nblog == o->blog_cap) {
        o->blog_cap = o->blog_cap ? 2 * o->blog_cap : 256;
        o->blog = (int *)realloc(o->blog, sizeof(int) * 2 * (size_t)o->blog_cap);
        if (!o->blog) {
            fprintf(stderr, "lpm_oracle: out of memory\n");
            abort();
        }
    }
    o->blog[2 * o->nblog] = i;
    o->blog[2 * o->nblog + 1] = j;
    o->nblog++;
}

/* updateDuctileDamagePwiseNonlocal, src/constitutive.c:1757-1862: nonlocal
 * damage rate of particle i = Gaussian-weighted (length L, cut at 3L)
 * average over all particles j of dlambda_j (1 + A triaxiality_j) at the
 * initial positions, summed in ascending j; particles past the threshold are
 * clamped to 1 and lose every bond; intact bonds carry D = max of the two
 * particles' damage and w = 1 - D.  J2_triaxiality is never assigned in the
 * reference, so it is 0 here. */
static int damage_ductile_nonlocal(lpm_oracle *o)
{
    int n = o->n, nn = o->nn;
    const double L = o->dmg_L, thr = o->dmg_thr, cA = o->dmg_cA;
    const double PI_ = 3.14159265358979323846; /* include/lpm.h:34 */
#pragma omp parallel for schedule(dynamic, 16)
    for (int i = 0; i < n; i++) {
        if (o->dnl[0][i] > thr) {
            if (o->dnl[0][i] > 1.0)
                o->dnl[0][i] = 1.0;
            continue;
        }
        double Ddot = 0, A = 0;
        for (int j = 0; j < n; j++) {
            double DdotLocal = 0;
            double ex = o->xyz0[3 * j] - o->xyz0[3 * i], ey = o->xyz0[3 * j + 1] - o->xyz0[3 * i + 1],
                   ez = o->xyz0[3 * j + 2] - o->xyz0[3 * i + 2];
            double dis = sqrt(ex * ex + ey * ey + ez * ez);
            if (dis < 3 * L) {
                double triax = 0.0;
                double damage_f = (1.0 + cA * triax);
                if (damage_f > 0.0)
                    DdotLocal = o->dlambda[j] * (1.0 + cA * triax);
                double phi = 1.0 / L / sqrt(2 * PI_) * exp(-0.5 * dis * dis / L / L);
                Ddot += DdotLocal * phi * o->vol;
                A += phi * o->vol;
            }
        }
        if (Ddot > 0.0)
            o->dnl[0][i] += 1.0 / A * Ddot;
    }
    int k = 0;
    for (int i = 0; i < n; i++)
        for (int j = 0; j < o->nb[i]; j++) {
            size_t b = (size_t)i * nn + j;
            int p = o->nbr[b];
            if (o->dnl[0][i] > thr || o->dnl[0][p] > thr) {
                if (fabs(o->brk[b]) > EPSP) {
                    o->brk[b] = 0.0;
                    o->dD[0][b] = 1.0;
                    log_bond(o, i, p);
                    k++;
                }
            }
        }
    for (int i = 0; i < n; i++)
        for (int j = 0; j < o->nb[i]; j++) {
            size_t b = (size_t)i * nn + j;
            int p = o->nbr[b];
            if (fabs(o->brk[b]) > EPSP)
                o->dD[0][b] = o->dnl[0][i] > o->dnl[0][p] ? o->dnl[0][i] : o->dnl[0][p];
            o->dw[b] = 1.0 - o->dD[0][b];
        }
    return k;
}

/* The choice of updateBrittleDamage (src/constitutive.c:1471-1520) among k
 * candidates given in the reference's scan order: all of them when k <=
 * nbreak, else the reference's ascending shell sort (gaps k/2, k/4, ..., 1)
 * and the last nbreak.  Sorts (bi, bj, bs) in place and returns the index of
 * the first chosen entry. */
int lo_brittle_select(int *bi, int *bj, double *bs, int k, int nbreak)
{
    if (k <= nbreak)
        return 0;
    for (int r = k / 2; r >= 1; r = r / 2)
        for (int i = r; i < k; ++i) {
            int ti = bi[i], tj = bj[i];
            double tb = bs[i];
            int j = i - r;
            while (j >= 0 && bs[j] > tb) {
                bs[j + r] = bs[j];
                bi[j + r] = bi[j];
                bj[j + r] = bj[j];
                j = j - r;
            }
            bs[j + r] = tb;
            bi[j + r] = ti;
            bj[j + r] = tj;
        }
    return k - nbreak;
}

/* updateBrittleDamage, src/constitutive.c:1437-1527: bonds whose elastic
 * stretch / initial length reaches critical_bstrain are candidates (scan
 * order i, then j); at most nbreak of them break, the largest strains after
 * the reference's ascending shell sort; returns the number of candidates. */
static int damage_brittle(lpm_oracle *o)
{
    int n = o->n, nn = o->nn, nbreak = o->dmg_nbreak;
    int cap = 64, k = 0;
    int *bi = IALLOC(cap), *bj = IALLOC(cap);
    double *bs = DALLOC(cap);
    for (int i = 0; i < n; i++)
        for (int j = 0; j < o->nb[i]; j++) {
            size_t b = (size_t)i * nn + j;
            double ave_bstrain = o->dL[b] / o->L0[b];
            if (ave_bstrain >= o->dmg_crit) {
                if (k == cap) {
                    cap *= 2;
                    bi = (int *)realloc(bi, sizeof(int) * cap);
                    bj = (int *)realloc(bj, sizeof(int) * cap);
                    bs = (double *)realloc(bs, sizeof(double) * cap);
                    if (!bi || !bj || !bs) {
                        fprintf(stderr, "lpm_oracle: out of memory\n");
                        abort();
                    }
                }
                bi[k] = i;
                bj[k] = j;
                bs[k] = ave_bstrain;
                k++;
            }
        }
    int first = lo_brittle_select(bi, bj, bs, k, nbreak);
    for (int q = first; q < k; q++) {
        size_t b = (size_t)bi[q] * nn + bj[q];
        o->dD[0][b] = 1.0;
        o->dw[b] = 0.0;
        o->brk[b] = 0.0;
        log_bond(o, bi[q], o->nbr[b]);
    }
    free(bi);
    free(bj);
    free(bs);
    return k;
}

/* updateDamageGeneral, src/constitutive.c:149-164 (plmode 0: ductile
 * pointwise nonlocal; 6: brittle; others: none) */
int lo_damage_update(lpm_oracle *o, int plmode)
{
    if (plmode == 0)
        return damage_ductile_nonlocal(o);
    if (plmode == 6)
        return damage_brittle(o);
    return 0;
}

/* updateCrack, src/constitutive.c:1399-1434: current bond counts, damage
 * picture, F scaled by w and Pin re-summed, particles without bonds fixed */
void lo_update_crack(lpm_oracle *o)
{
    int n = o->n, nn = o->nn;
    for (int i = 0; i < n; i++) {
        o->nbc[i] = o->nb[i];
        o->dvis[i] = 0.0;
        o->Pin[3 * i] = 0.0, o->Pin[3 * i + 1] = 0.0, o->Pin[3 * i + 2] = 0.0;
        for (int j = 0; j < o->nb[i]; j++) {
            size_t b = (size_t)i * nn + j;
            if (o->brk[b] <= EPSP)
                o->nbc[i] -= 1;
            o->dvis[i] += o->brk[b];
            o->F[b] *= o->dw[b];
            o->Pin[3 * i] += o->csx[b] * o->F[b];
            o->Pin[3 * i + 1] += o->csy[b] * o->F[b];
            o->Pin[3 * i + 2] += o->csz[b] * o->F[b];
        }
        if (o->nbc[i] < 1) {
            o->fix[3 * i] = 0;
            o->fix[3 * i + 1] = 0;
            o->fix[3 * i + 2] = 0;
        }
        o->dvis[i] = 1 - o->dvis[i] / o->nb[i];
    }
}

int lo_broken_log(const lpm_oracle *o, int *pairs)
{
    if (pairs)
        memcpy(pairs, o->blog, sizeof(int) * 2 * (size_t)o->nblog);
    return o->nblog;
}

/* one load step of the reference's main with its damage stage
 * (src/lpmc_project.c:385-471 and :528-546): after the Newton loop,
 * updateDamageGeneral, updateCrack and switchStateV(1); when bonds broke,
 * the stiffness is recomputed and the same load step re-enters the Newton
 * loop at label_broken_bond, until a pass breaks nothing.  stats: [0] Newton
 * iterations over all passes, [1] first |residual|, [2] first |reaction|,
 * [3] final |residual|, [4] CG iterations, [5] passes, [6] bonds broken
 * (candidates counted as the reference's return value does). */
int lo_load_step_damage(lpm_oracle *o, int nbd, const lo_disp_bc *d, int nbf, const lo_force_bc *f,
                        double newton_tol, int maxiter, double cg_rtol_sq, double cg_atol_sq, int max_passes,
                        double *stats)
{
    int n = o->n;
    memcpy(o->xyz_temp, o->xyz, sizeof(double) * 3 * n);
    memcpy(o->F_temp, o->F, sizeof(double) * n * o->nn);
    memcpy(o->Pex_temp, o->Pex, sizeof(double) * 3 * n);
    lo_fd_stiffness(o);
    lo_set_disp_bc(o, nbd, d);
    lo_set_force_bc(o, nbf, f);
    lo_force(o, 4);
    int ni_tot = 0, cg = 0, passes = 0, broken_tot = 0;
    double nr0 = 0, nreac0 = 0, nr = 0;
    for (;;) {
        lo_update_rr(o);
        nr = cblas_dnrm2(3 * n, o->residual, 1);
        double nreac = cblas_dnrm2(o->nreact, o->reaction, 1);
        double tolm = nr > nreac ? nr : nreac;
        if (passes == 0) {
            nr0 = nr;
            nreac0 = nreac;
        }
        int ni = 0;
        while (nr > newton_tol * tolm && ni < maxiter) {
            lo_switch_state(o, 0);
            lo_bc_stiffness_update(o);
            int it = lo_solver_cg(o, cg_rtol_sq, cg_atol_sq);
            cg += it > 0 ? it : 0;
            lo_force(o, o->plmode);
            lo_update_rr(o);
            ni++;
            nr = cblas_dnrm2(3 * n, o->residual, 1);
        }
        ni_tot += ni;
        passes++;
        int broken = lo_damage_update(o, o->plmode);
        broken_tot += broken;
        lo_update_crack(o);
        lo_switch_state(o, 1);
        if (broken <= 0 || passes >= max_passes)
            break;
        lo_fd_stiffness(o);
    }
    if (stats) {
        stats[0] = ni_tot;
        stats[1] = nr0;
        stats[2] = nreac0;
        stats[3] = nr;
        stats[4] = cg;
        stats[5] = passes;
        stats[6] = broken_tot;
    }
    return ni_tot;
}

/* ---------------------------------------------------------------------- */
int lo_n(const lpm_oracle *o) { return o->n; }
int lo_nn(const lpm_oracle *o) { return o->nn; }
int lo_nnz(const lpm_oracle *o) { return o->nnz; }
int lo_nslip(const lpm_oracle *o) { return o->nslip; }
int lo_nconn_max(const lpm_oracle *o) { return o->nafem + 1; }

double *lo_d(lpm_oracle *o, const char *nm)
{
#define D_(k, p) if (!strcmp(nm, k)) return (p)
    D_("xyz", o->xyz); D_("xyz_initial", o->xyz0); D_("xyz_temp", o->xyz_temp);
    D_("distance_initial", o->L0); D_("csx_initial", o->cs0x); D_("csy_initial", o->cs0y);
    D_("csz_initial", o->cs0z); D_("Kn", o->Kn); D_("Tv", o->Tv); D_("opp", o->opp);
    D_("K_global", o->K); D_("dL", o->dL); D_("dL_total", o->Ssum); D_("TdL_total", o->Tsum);
    D_("csx", o->csx); D_("csy", o->csy); D_("csz", o->csz); D_("F", o->F); D_("F_temp", o->F_temp);
    D_("Pin", o->Pin); D_("Pex", o->Pex); D_("residual", o->residual); D_("reaction_force", o->reaction);
    D_("disp", o->disp); D_("stress_tensor", o->stress); D_("J2_dlambda", o->dlambda);
    D_("dLp0", o->dLp[0]); D_("dLp1", o->dLp[1]); D_("dLp2", o->dLp[2]);
    D_("alpha0", o->alpha[0]); D_("alpha1", o->alpha[1]); D_("alpha2", o->alpha[2]);
    D_("beta0", o->beta[0]); D_("beta1", o->beta[1]); D_("beta2", o->beta[2]);
    D_("cp_gy0", o->cp_gy[0]); D_("cp_gy1", o->cp_gy[1]); D_("cp_A0", o->cp_A[0]);
    D_("cp_A1", o->cp_A[1]); D_("cp_As0", o->cp_As[0]); D_("cp_As1", o->cp_As[1]);
    D_("cp_Cab", o->Cab); D_("schmid", &o->sch[0][0]); D_("KnTve", o->knt); D_("distance", o->dist);
    D_("cp_RSS", o->cp_RSS);
    D_("damage_broken", o->brk); D_("damage_w", o->dw); D_("damage_D0", o->dD[0]); D_("damage_D1", o->dD[1]);
    D_("damage_nonlocal0", o->dnl[0]); D_("damage_nonlocal1", o->dnl[1]); D_("damage_visual", o->dvis);
    return NULL;
#undef D_
}

int *lo_i(lpm_oracle *o, const char *nm)
{
#define I_(k, p) if (!strcmp(nm, k)) return (p)
    I_("neighbors", o->nbr); I_("nsign", o->shell); I_("nb", o->nb); I_("conn", o->conn);
    I_("nb_conn", o->nconn); I_("kp0", o->kp0); I_("kp1", o->kp1); I_("IK", o->IK); I_("JK", o->JK);
    I_("type", o->type); I_("rev", o->rev); I_("dispBC_index", o->mask); I_("cp_Jact", o->Jact);
    I_("neighbors1", o->nbr1); I_("neighbors2", o->nbr2); I_("error", &o->error);
    I_("nb_current", o->nbc); I_("fix_index", o->fix);
    return NULL;
#undef I_
}
