/*
 * lpm_host.c - C host driver of the GPU drop-in (liblpmhost.so).
 *
 * Plays the role of the reference's src/lpmc_project.c: it defines and
 * allocates the include/lpm.h global state (lpmc_project.c:19-45,
 * initialization.c:1120-1194) and runs the load-step loop of
 * lpmc_project.c:382-471, calling the reference-named solve-path functions,
 * which liblpmgpu_legacy.so implements on the GPU.  Particle positions and
 * bond lists come from the GPU library's setup (bit-identical to
 * createCuboid / searchNormalNeighbor / searchAFEMNeighbor).
 *
 * Exported for scripting (ctypes): lpmh_setup, lpmh_set_types,
 * lpmh_set_bc_groups, lpmh_set_material, lpmh_set_damage, lpmh_init,
 * lpmh_load_step, lpmh_get, lpmh_n.
 *
 * Per-particle moduli: the reference takes elastic constants per type
 * (Ce[type[i]], src/stiffness.c:186-200), so a material that varies from
 * particle to particle gives every particle its own type.  Its boundary
 * conditions, which setDispBC/setForceBC select by type
 * (src/boundary.c:12-70), are then given as BC groups: lpmh_set_bc_groups
 * stores one group label per particle, and each load step hands setDispBC
 * and setForceBC that label array in place of `type` (the functions
 * themselves are unchanged).
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "lpm_gpu.h"
#include "lpm_legacy.h"

#define NDIM 3
#define MAXV(a, b) ((a) > (b) ? (a) : (b))

struct dispBCPara {
    int type;
    char flag;
    double step;
};
struct forceBCPara {
    int type;
    char flag1;
    double step1;
    char flag2;
    double step2;
    char flag3;
    double step3;
};

/* ---- include/lpm.h:55-81 globals, defined as in src/lpmc_project.c:19-45 ---- */
int ntype, particles_first_row, nparticle, rows, layers, nneighbors, nneighbors1, nneighbors2, dim;
int lattice, nneighbors_AFEM, nneighbors_AFEM1, nneighbors_AFEM2, plmode, eulerflag, nslip_face;
int max_nslip_vector, nslipSys, nbreak;
int *IK, *JK, *type, *dispBC_index, *fix_index, *nslip_vector, *lacknblist, pbc[NDIM], *pl_flag;
int *nb, *nb_initial, *nb_conn, *state_v;
int **neighbors, **neighbors1, **neighbors2, **neighbors_AFEM;
int **K_pointer, **conn, **nsign, **cp_Jact;
double radius, hx, hy, hz, neighbor1_cutoff, neighbor2_cutoff, angle1, angle2, angle3, particle_volume;
double R_matrix[NDIM * NDIM], box[2 * NDIM], cp_tau0[3], cp_taus[3], cp_eta, cp_p, cp_h0, cp_q, cp_maxloop;
double box_x, box_y, box_z, dtime, cp_theta, J2_H, J2_xi, J2_C, damage_L;
double damage_threshold, damageb_A, damagec_A, critical_bstrain;
double *K_global, *plastic_K_global, *residual, *Pin, *Pex, *Pex_temp, *disp, *sigmay, *cp_dA;
double *reaction_force, *damage_visual;
double *J2_dlambda, *J2_stresseq, *J2_stressm, *J2_triaxiality;
double **xyz, **xyz_initial, **xyz_temp, **distance, **distance_initial, **KnTve, **F, **csx, **csy, **csz;
double **dL_total, **TdL_total, **csx_initial, **csy_initial, **csz_initial, **Ce;
double **slip_normal, **schmid_tensor, **schmid_tensor_local, **cp_RSS, **stress_tensor;
double **cp_Cab, **strain_tensor, **dL_ave, **ddL_total, **TddL_total, **F_temp, **ddLp;
double **dL, **ddL, **bond_stress, **damage_broken, **damage_w, **bond_stretch, **bond_vector, **bond_force;
double **Kn, **Tv, **J2_alpha, **damage_local, **damage_nonlocal, **cp_A, **cp_dgy, **cp_dA_single, **J2_beta_eq;
double ***slip_vector, ***dLp, ***J2_beta, ***damage_D, ***cp_gy, ***cp_A_single;

/* main's damage stage (src/lpmc_project.c:239-244 parameters, :466-470 and
 * :528-546 per load step): off unless lpmh_set_damage is called */
static int g_damage = 0, g_max_passes = 1000, g_step = 0;
static char g_bondfile[1024];
/* BC group per particle (lpmh_set_bc_groups); NULL: BCs select by type */
static int *g_bc_group, g_bc_ngroup;

/* ---- allocation helpers (src/lpm_basic.c:361-445 semantics) ---------------- */
static double *d1(int n, double v)
{
    double *p = (double *)malloc(sizeof(double) * (n > 0 ? n : 1));
    for (int i = 0; i < n; i++)
        p[i] = v;
    return p;
}
static int *i1(int n, int v)
{
    int *p = (int *)malloc(sizeof(int) * (n > 0 ? n : 1));
    for (int i = 0; i < n; i++)
        p[i] = v;
    return p;
}
static double **d2(int r, int c, double v)
{
    double **p = (double **)malloc(sizeof(double *) * r);
    for (int i = 0; i < r; i++)
        p[i] = d1(c, v);
    return p;
}
static int **i2(int r, int c, int v)
{
    int **p = (int **)malloc(sizeof(int *) * r);
    for (int i = 0; i < r; i++)
        p[i] = i1(c, v);
    return p;
}
static double ***d3(int r, int c, int l, double v)
{
    double ***p = (double ***)malloc(sizeof(double **) * r);
    for (int i = 0; i < r; i++)
        p[i] = d2(c, l, v);
    return p;
}

static double dnrm2(int n, const double *x)
{
    double s = 0.0;
    for (int i = 0; i < n; i++)
        s += x[i] * x[i];
    return sqrt(s);
}

/* initMatrices, src/initialization.c:1120-1194 (the arrays the solve path uses) */
static void init_matrices(void)
{
    int n = nparticle, nn = nneighbors;
    disp = d1(dim * n, 0);
    xyz_initial = d2(n, NDIM, 0);
    xyz_temp = d2(n, NDIM, 0);
    distance = d2(n, nn, 0.0);
    distance_initial = d2(n, nn, 0.0);
    csx = d2(n, nn, 0.0);
    csy = d2(n, nn, 0.0);
    csz = d2(n, nn, 0.0);
    csx_initial = d2(n, nn, 0.0);
    csy_initial = d2(n, nn, 0.0);
    csz_initial = d2(n, nn, 0.0);
    dL = d2(n, nn, 0.0);
    dL_total = d2(n, 2, 0);
    TdL_total = d2(n, 2, 0);
    dL_ave = d2(n, nn, 0.);
    dLp = d3(n, nn, 3, 0.);
    ddL = d2(n, nn, 0.0);
    ddL_total = d2(n, 2, 0);
    TddL_total = d2(n, 2, 0);
    ddLp = d2(n, nn, 0.);
    bond_stress = d2(n, nn, 0);
    bond_stretch = d2(n, nn, 0);
    state_v = i1(n, 0);
    pl_flag = i1(n, 0);
    nb = i1(n, -1);
    nb_initial = i1(n, -1);
    nb_conn = i1(n, -1);
    neighbors = i2(n, nn, -1);
    neighbors1 = i2(n, nneighbors1, -1);
    neighbors2 = i2(n, nneighbors2, -1);
    nsign = i2(n, nn, -1);
    conn = i2(n, nneighbors_AFEM + 1, -1);
    K_pointer = i2(n + 1, 2, 0);
    residual = d1(dim * n, 0);
    Pin = d1(NDIM * n, 0);
    Pex = d1(dim * n, 0);
    Pex_temp = d1(dim * n, 0);
    dispBC_index = i1(dim * n, 1);
    fix_index = i1(dim * n, 1);
    Kn = d2(n, nn, 0.0);
    Tv = d2(n, nn, 0.0);
    stress_tensor = d2(n, 2 * NDIM, 0.);
    strain_tensor = d2(n, 2 * NDIM, 0.);
    damage_broken = d2(n, nn, 1.);
    damage_D = d3(n, nn, 2, 0.);
    damage_w = d2(n, nn, 1.);
    damage_visual = d1(n, 0.0);
    damage_local = d2(n, 2, 0.0);
    damage_nonlocal = d2(n, 2, 0.0);
    F = d2(n, nn, 0.);
    F_temp = d2(n, nn, 0.);
    bond_force = d2(n, nn, 0.);
    J2_beta = d3(n, 2 * NDIM, 3, 0.);
    J2_alpha = d2(n, 3, 0.);
    J2_beta_eq = d2(n, 3, 0.);
    J2_stresseq = d1(n, 0.);
    J2_stressm = d1(n, 0.);
    J2_triaxiality = d1(n, 0.);
    J2_dlambda = d1(n, 0.);
    /* crystal-plasticity state (slipSysDefine3D, src/initialization.c:816-826) */
    cp_gy = d3(n, nslipSys, 3, cp_tau0[0]);
    cp_RSS = d2(n, nslipSys, 0.);
    cp_Jact = i2(n, nslipSys, 0);
    cp_A = d2(n, 3, 0.);
    cp_A_single = d3(n, nslipSys, 3, 0.);
    cp_Cab = d2(n, nslipSys * nslipSys, 0.);
    cp_dA_single = d2(n, nslipSys, 0.0);
    cp_dA = d1(n, 0.0);
    cp_dgy = d2(n, nslipSys, 0.0);
}

static lpm_ctx *g_setup = NULL;

/* Lattice + bond lists + AFEM connectivity into the globals.  Returns n. */
int lpmh_setup(int lat, double rad, const double *bx, int nslip)
{
    g_damage = 0;
    g_step = 0;
    free(g_bc_group); /* a new specimen: BCs select by type until groups are set again */
    g_bc_group = NULL;
    g_bc_ngroup = 0;
    lattice = lat;
    dim = 3;
    radius = rad;
    for (int k = 0; k < 6; k++)
        box[k] = bx[k];
    nneighbors = 18;
    nneighbors1 = lat == 2 ? 6 : 12;
    nneighbors2 = lat == 2 ? 12 : 6;
    nneighbors_AFEM = 60;
    neighbor1_cutoff = 2.0 * radius;
    neighbor2_cutoff = 2.0 * sqrt(2.0) * radius;
    particle_volume = lat == 2 ? pow(2 * radius, 3) : 4.0 * sqrt(2.0) * pow(radius, 3);
    nslipSys = nslip;
    if (lpm_create(&g_setup, 0) != LPM_OK)
        return -1;
    int n = lpm_setup_lattice(g_setup, lat, rad, bx);
    if (n <= 0)
        return -1;
    nparticle = n;
    init_matrices();
    int nn = nneighbors;
    double *tx = d1(3 * n, 0), *tb = d1(n * nn, 0), *tc = d1(3 * n * nn, 0);
    int *ti = i1(n * 61, 0);
    lpm_get(g_setup, "xyz", tx, sizeof(double) * 3 * n);
    xyz = d2(n, NDIM, 0);
    for (int i = 0; i < n; i++)
        for (int d = 0; d < 3; d++)
            xyz[i][d] = xyz_initial[i][d] = tx[3 * i + d];
    lpm_get(g_setup, "neighbors", ti, sizeof(int) * n * nn);
    for (int i = 0; i < n; i++)
        memcpy(neighbors[i], ti + (size_t)i * nn, sizeof(int) * nn);
    lpm_get(g_setup, "nsign", ti, sizeof(int) * n * nn);
    for (int i = 0; i < n; i++)
        memcpy(nsign[i], ti + (size_t)i * nn, sizeof(int) * nn);
    lpm_get(g_setup, "nb", nb, sizeof(int) * n);
    memcpy(nb_initial, nb, sizeof(int) * n);
    lpm_get(g_setup, "distance_initial", tb, sizeof(double) * n * nn);
    for (int i = 0; i < n; i++)
        memcpy(distance_initial[i], tb + (size_t)i * nn, sizeof(double) * nn);
    lpm_get(g_setup, "cs_initial", tc, sizeof(double) * 3 * n * nn);
    for (int i = 0; i < n; i++)
        for (int j = 0; j < nn; j++) {
            csx_initial[i][j] = tc[3 * ((size_t)i * nn + j)];
            csy_initial[i][j] = tc[3 * ((size_t)i * nn + j) + 1];
            csz_initial[i][j] = tc[3 * ((size_t)i * nn + j) + 2];
        }
    lpm_get(g_setup, "conn", ti, sizeof(int) * n * 61);
    for (int i = 0; i < n; i++)
        memcpy(conn[i], ti + (size_t)i * 61, sizeof(int) * 61);
    lpm_get(g_setup, "nb_conn", nb_conn, sizeof(int) * n);
    int *kp = i1(2 * (n + 1), 0);
    lpm_get(g_setup, "K_pointer", kp, sizeof(int) * 2 * (n + 1));
    for (int i = 0; i <= n; i++) {
        K_pointer[i][0] = kp[2 * i];
        K_pointer[i][1] = kp[2 * i + 1];
    }
    int nnz = K_pointer[n][1];
    JK = i1(nnz, -1);
    IK = i1(dim * n + 1, -1);
    K_global = d1(nnz, -1);
    free(kp);
    free(tx);
    free(tb);
    free(tc);
    free(ti);
    lpm_destroy(g_setup);
    g_setup = NULL;
    ntype = 0;
    type = i1(n, ntype++);
    return n;
}

int lpmh_n(void) { return nparticle; }

void lpmh_set_types(const int *t, int nt)
{
    for (int i = 0; i < nparticle; i++)
        type[i] = t[i];
    ntype = nt;
}

/* BC group label per particle (NULL: boundary conditions select by type) */

void lpmh_set_bc_groups(const int *g, int ngroup)
{
    free(g_bc_group);
    g_bc_group = NULL;
    g_bc_ngroup = 0;
    if (!g)
        return;
    g_bc_group = (int *)malloc(sizeof(int) * (size_t)nparticle);
    memcpy(g_bc_group, g, sizeof(int) * (size_t)nparticle);
    g_bc_ngroup = ngroup;
}

/* setDispBC + setForceBC (src/lpmc_project.c:402-403), selecting particles by
 * BC group when groups are set */
static void apply_bcs(int nbd, struct dispBCPara *dbp, int nbf, struct forceBCPara *fbp)
{
    int *t = type, nt = ntype;
    if (g_bc_group) {
        type = g_bc_group;
        ntype = g_bc_ngroup;
    }
    setDispBC(nbd, dbp);
    setForceBC(nbf, fbp);
    type = t;
    ntype = nt;
}

/* ce: ntype x 3; sy: per particle; cp: tau0, taus, h0, p, q, eta, maxloop, dtime */
void lpmh_set_material(const double *ce, int pl, const double *sy, double xi, double H, const double *cp)
{
    Ce = d2(ntype, 3, 0.);
    for (int i = 0; i < ntype; i++)
        for (int k = 0; k < 3; k++)
            Ce[i][k] = ce[3 * i + k];
    plmode = pl;
    sigmay = d1(nparticle, 0.0);
    if (sy)
        memcpy(sigmay, sy, sizeof(double) * nparticle);
    J2_xi = xi;
    J2_H = H;
    if (cp) {
        cp_tau0[0] = cp[0];
        cp_taus[0] = cp[1];
        cp_h0 = cp[2];
        cp_p = cp[3];
        cp_q = cp[4];
        cp_eta = cp[5];
        cp_maxloop = cp[6];
        dtime = cp[7];
        for (int i = 0; i < nparticle; i++)
            for (int s = 0; s < nslipSys; s++)
                for (int k = 0; k < 3; k++)
                    cp_gy[i][s][k] = cp_tau0[0];
    }
}

/* computedL, src/lpm_basic.c:252-291 */
static void computed_l(void)
{
    for (int i = 0; i < nparticle; i++) {
        dL_total[i][0] = 0, TdL_total[i][0] = 0;
        dL_total[i][1] = 0, TdL_total[i][1] = 0;
        for (int j = 0; j < nb_initial[i]; j++) {
            int p = neighbors[i][j];
            double dx = xyz[i][0] - xyz[p][0], dy = xyz[i][1] - xyz[p][1], dz = xyz[i][2] - xyz[p][2];
            distance[i][j] = sqrt(dx * dx + dy * dy + dz * dz);
            dL[i][j] = distance[i][j] - distance_initial[i][j];
            dL[i][j] -= dLp[i][j][0];
            dL_total[i][nsign[i][j]] += dL[i][j];
            TdL_total[i][nsign[i][j]] += Tv[i][j] * dL[i][j];
            csx[i][j] = dx / distance[i][j];
            csy[i][j] = dy / distance[i][j];
            csz[i][j] = dz / distance[i][j];
        }
    }
}

/* src/lpmc_project.c:339-345 */
void lpmh_init(void)
{
    calcKnTv();
    computed_l();
    if (lattice == 3 || lattice == 4)
        computeCab();
}

void lpmh_set_damage(double L, double threshold, double cA, double crit, int nbr, const char *bondfile,
                     int max_passes)
{
    damage_L = L;
    damage_threshold = threshold;
    damagec_A = cA;
    critical_bstrain = crit;
    nbreak = nbr;
    snprintf(g_bondfile, sizeof g_bondfile, "%s", bondfile ? bondfile : "result_brokenbonds.txt");
    g_max_passes = max_passes > 0 ? max_passes : 1000;
    g_damage = 1;
}

/*
 * One load step, src/lpmc_project.c:385-471, and with the damage stage on
 * :466-470 and the re-entry after broken bonds (:528-546: new stiffness, then
 * label_broken_bond).  computeStrain and the output writers are left out.
 * stats (7 values): Newton iterations, |r0|, |reaction0|, |r| final, 0,
 * Newton passes, sum of updateDamageGeneral's return values.
 */
int lpmh_load_step(int nbd, struct dispBCPara *dbp, int nbf, struct forceBCPara *fbp, double newton_tol,
                   int maxiter, double *stats)
{
    int n = nparticle;
    g_step++;
    for (int i = 0; i < n; i++) {
        memcpy(xyz_temp[i], xyz[i], sizeof(double) * NDIM);
        memcpy(F_temp[i], F[i], sizeof(double) * nneighbors);
    }
    memcpy(Pex_temp, Pex, sizeof(double) * dim * n);
    calcStiffness3DFiniteDifference(6);
    apply_bcs(nbd, dbp, nbf, fbp);
    computeBondForceGeneral(4, 1);
    double nr = 0.0, nr0 = 0.0, nreac0 = 0.0;
    int ni_tot = 0, passes = 0, broken_tot = 0;
    for (;;) {
        updateRR(); /* label_broken_bond */
        int nreact = 0;
        for (int k = 0; k < n * dim; k++)
            nreact += (dispBC_index[k] != 1);
        nr = dnrm2(dim * n, residual);
        double nreac = dnrm2(nreact, reaction_force);
        double tolm = MAXV(nr, nreac);
        if (passes == 0) {
            nr0 = nr;
            nreac0 = nreac;
        }
        int ni = 0;
        while (nr > newton_tol * tolm && ni < maxiter) {
            switchStateV(0);
            setDispBC_stiffnessUpdate3D();
            solverCG();
            computeBondForceGeneral(plmode, 1);
            updateRR();
            ni++;
            nr = dnrm2(dim * n, residual);
        }
        ni_tot += ni;
        passes++;
        if (!g_damage) {
            switchStateV(1);
            break;
        }
        int broken = updateDamageGeneral(g_bondfile, g_step, plmode);
        updateCrack();
        switchStateV(1);
        broken_tot += broken;
        if (broken <= 0 || passes >= g_max_passes)
            break;
        calcStiffness3DFiniteDifference(6);
    }
    if (stats) {
        stats[0] = ni_tot;
        stats[1] = nr0;
        stats[2] = nreac0;
        stats[3] = nr;
        stats[4] = 0.0;
        stats[5] = passes;
        stats[6] = broken_tot;
    }
    return ni_tot;
}

/* flat copies of a few globals (row-major) */
int lpmh_get(const char *name, double *out)
{
    int n = nparticle, nn = nneighbors;
    if (!strcmp(name, "xyz")) {
        for (int i = 0; i < n; i++)
            memcpy(out + 3 * (size_t)i, xyz[i], sizeof(double) * 3);
    } else if (!strcmp(name, "xyz_initial")) {
        for (int i = 0; i < n; i++)
            memcpy(out + 3 * (size_t)i, xyz_initial[i], sizeof(double) * 3);
    } else if (!strcmp(name, "J2_alpha")) {
        for (int i = 0; i < n; i++)
            out[i] = J2_alpha[i][1];
    } else if (!strcmp(name, "F")) {
        for (int i = 0; i < n; i++)
            memcpy(out + (size_t)i * nn, F[i], sizeof(double) * nn);
    } else if (!strcmp(name, "csz")) {
        for (int i = 0; i < n; i++)
            memcpy(out + (size_t)i * nn, csz[i], sizeof(double) * nn);
    } else if (!strcmp(name, "Kn") || !strcmp(name, "Tv")) {
        double **a = name[0] == 'K' ? Kn : Tv;
        for (int i = 0; i < n; i++)
            memcpy(out + (size_t)i * nn, a[i], sizeof(double) * nn);
    } else if (!strcmp(name, "dL")) {
        for (int i = 0; i < n; i++)
            memcpy(out + (size_t)i * nn, dL[i], sizeof(double) * nn);
    } else if (!strcmp(name, "damage_broken") || !strcmp(name, "damage_w")) {
        double **a = name[7] == 'b' ? damage_broken : damage_w;
        for (int i = 0; i < n; i++)
            memcpy(out + (size_t)i * nn, a[i], sizeof(double) * nn);
    } else if (!strcmp(name, "damage_nonlocal")) {
        for (int i = 0; i < n; i++)
            out[i] = damage_nonlocal[i][1];
    } else if (!strcmp(name, "nb")) {
        for (int i = 0; i < n; i++)
            out[i] = nb[i];
    } else if (!strcmp(name, "strain_tensor")) {
        for (int i = 0; i < n; i++)
            memcpy(out + 6 * (size_t)i, strain_tensor[i], sizeof(double) * 6);
    } else {
        return -1;
    }
    return 0;
}
