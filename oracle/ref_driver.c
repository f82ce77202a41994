/*
 * Driver for the LPM-C reference built from its own sources (oracle/_ref).
 *
 * TEST INFRASTRUCTURE ONLY.  The reference has no library API: all state is
 * in the globals of include/lpm.h and its only driver is the hard-coded
 * main() of src/lpmc_project.c.  This file replaces that main with callable
 * steps, so tests and the golden-vector generator can run the reference's
 * own functions on chosen configurations:
 *   refd_setup      -> src/lpmc_project.c:75-182 (lattice, createCuboid,
 *                      initMatrices, searchNormalNeighbor, searchAFEMNeighbor)
 *   refd_material   -> src/lpmc_project.c:185-222 (Ce per type, plmode data)
 *   refd_init_state -> src/lpmc_project.c:339-345 (calcKnTv, computedL,
 *                      slipSysDefine3D, computeCab)
 *   refd_load_step  -> src/lpmc_project.c:382-471 (one load step with the
 *                      Newton loop); the Newton tolerance is a parameter
 *                      instead of TOLITER, damage/crack updates are skipped
 *                      (the configurations exercised have no damage) and
 *                      computeStrain (output only) is skipped.
 *   refd_load_step_damage -> the same load step with main's damage stage
 *                      and re-solve (src/lpmc_project.c:466-470, :528-546).
 * Displacement BCs use the reference's setDispBC/setForceBC on `type`, or,
 * when refd_set_bc_groups() was given a group array (materials per particle
 * need one type per particle), the same semantics restated over the groups.
 */
#include "lpm.h"

/* The reference's globals are defined in src/lpmc_project.c, compiled with
 * its main() renamed; nothing else is needed here. */

static int *g_bcgroup = NULL; /* optional BC group per particle */

int refd_setup(int lat, double rad, const double *bx)
{
    lattice = lat;
    dim = (lattice < 2) ? 2 : 3;
    radius = rad;
    pbc[0] = pbc[1] = pbc[2] = 0;
    eulerflag = 0;
    angle1 = angle2 = angle3 = 0.0;
    for (int i = 0; i < 6; i++)
        box[i] = bx[i];
    box_x = box[1] - box[0];
    box_y = box[3] - box[2];
    box_z = box[5] - box[4];
    createCuboid();
    initMatrices();
    copyDouble2D(xyz_initial, xyz, nparticle, NDIM);
    searchNormalNeighbor();
    int len = searchAFEMNeighbor();
    ntype = 0;
    type = allocInt1D(nparticle, ntype++);
    return len >= 0 ? nparticle : -1;
}

/* type[i] for all particles; ntype_total = number of distinct types. */
void refd_set_types(const int *t, int ntype_total)
{
    for (int i = 0; i < nparticle; i++)
        type[i] = t[i];
    ntype = ntype_total;
}

void refd_set_bc_groups(const int *g)
{
    free(g_bcgroup);
    g_bcgroup = NULL;
    if (g) {
        g_bcgroup = (int *)malloc(sizeof(int) * nparticle);
        for (int i = 0; i < nparticle; i++)
            g_bcgroup[i] = g[i];
    }
}

/* Ce: ntype x 3 (C11, C12, C44); sy: yield stress per particle. */
void refd_material(const double *ce, int pl, const double *sy, double xi, double H,
                   const double *cp /* tau0, taus, h0, p, q, eta, maxloop, dtime */)
{
    Ce = allocDouble2D(ntype, 3, 0.);
    for (int i = 0; i < ntype; i++)
        for (int k = 0; k < 3; k++)
            Ce[i][k] = ce[3 * i + k];
    plmode = pl;
    sigmay = allocDouble1D(nparticle, 0.0);
    if (sy)
        for (int i = 0; i < nparticle; i++)
            sigmay[i] = sy[i];
    J2_xi = xi;
    J2_H = H;
    if (cp) {
        cp_tau0[0] = cp[0];
        cp_tau0[1] = cp_tau0[2] = 0.0;
        cp_taus[0] = cp[1];
        cp_taus[1] = cp_taus[2] = 0.0;
        cp_h0 = cp[2];
        cp_p = cp[3];
        cp_q = cp[4];
        cp_eta = cp[5];
        cp_maxloop = cp[6];
        dtime = cp[7];
    }
}

void refd_init_state(void)
{
    calcKnTv();
    computedL();
    slipSysDefine3D();
    if (lattice == 3 || lattice == 4)
        computeCab();
}

/* boundary.c:12-45 semantics over g_bcgroup instead of type */
static void group_disp_bc(int n, struct dispBCPara *d)
{
    for (int i = 0; i < nparticle; i++)
        for (int k = 0; k < n; k++)
            if (g_bcgroup[i] == d[k].type) {
                int c = d[k].flag == 'x' ? 0 : (d[k].flag == 'y' ? 1 : 2);
                xyz[i][c] += d[k].step;
                dispBC_index[dim * i + c] = 0;
            }
    reaction_force = allocDouble1D(countNEqual(dispBC_index, nparticle * dim, 1), 0.);
}

/* boundary.c:48-70 semantics over g_bcgroup instead of type */
static void group_force_bc(int n, struct forceBCPara *f)
{
    for (int k = 0; k < n; k++) {
        int cnt = 0;
        for (int i = 0; i < nparticle; i++)
            if (g_bcgroup[i] == f[k].type)
                cnt++;
        for (int i = 0; i < nparticle; i++)
            if (g_bcgroup[i] == f[k].type) {
                Pex[dim * i] += f[k].step1 / cnt;
                Pex[dim * i + 1] += f[k].step2 / cnt;
                Pex[dim * i + 2] += f[k].step3 / cnt;
            }
    }
}

/*
 * One load step (src/lpmc_project.c:385-471).  stats (may be NULL):
 * [0] Newton iterations, [1] initial |residual|, [2] initial |reaction|,
 * [3] final |residual|, [4] total CG iterations.
 */
static double *g_trace = NULL; /* optional per-iteration |residual| record */
void refd_set_trace(double *t) { g_trace = t; }

int refd_load_step(int nbd, struct dispBCPara *dbp, int nbf, struct forceBCPara *fbp,
                   int load_ind, double newton_tol, int maxiter, double *stats)
{
    copyDouble2D(xyz_temp, xyz, nparticle, NDIM);
    copyDouble2D(F_temp, F, nparticle, nneighbors);
    copyDouble1D(Pex_temp, Pex, dim * nparticle);

    calcStiffness3DFiniteDifference(6);

    if (g_bcgroup) {
        group_disp_bc(nbd, dbp);
        group_force_bc(nbf, fbp);
    } else {
        setDispBC(nbd, dbp);
        setForceBC(nbf, fbp);
    }
    computeBondForceGeneral(4, load_ind);
    updateRR();

    double nr = cblas_dnrm2(dim * nparticle, residual, 1);
    double nreac = cblas_dnrm2(countNEqual(dispBC_index, nparticle * dim, 1), reaction_force, 1);
    double tolm = MAX(nr, nreac);
    double nr0 = nr;
    int ni = 0, cgtot = 0;
    while (nr > newton_tol * tolm && ni < maxiter) {
        switchStateV(0);
        setDispBC_stiffnessUpdate3D();
        solverCG();
        cgtot += lpm_shim_last_cg_iters();
        computeBondForceGeneral(plmode, load_ind);
        updateRR();
        nr = cblas_dnrm2(dim * nparticle, residual, 1);
        if (g_trace)
            g_trace[ni] = nr;
        ni++;
    }
    switchStateV(1);
    if (stats) {
        stats[0] = ni;
        stats[1] = nr0;
        stats[2] = nreac;
        stats[3] = nr;
        stats[4] = cgtot;
    }
    return ni;
}

/* Damage parameters (the globals src/lpmc_project.c:239-244 sets in main). */
void refd_set_damage(double L, double threshold, double cA, double crit_bstrain, int nbreak_)
{
    damage_L = L;
    damage_threshold = threshold;
    damagec_A = cA;
    critical_bstrain = crit_bstrain;
    nbreak = nbreak_;
}

/*
 * One load step of main with its damage stage (src/lpmc_project.c:385-471
 * and :528-546): the Newton loop, then computeStrain, updateDamageGeneral
 * (broken bonds appended to `bondfile`), updateCrack and switchStateV(1);
 * when bonds broke, calcStiffness3DFiniteDifference and back to
 * label_broken_bond, until a pass breaks nothing (or max_passes).  stats:
 * [0] Newton iterations over all passes, [1] first |residual|, [2] first
 * |reaction|, [3] final |residual|, [4] CG iterations, [5] passes, [6] sum of
 * updateDamageGeneral's return values.
 */
int refd_load_step_damage(int nbd, struct dispBCPara *dbp, int nbf, struct forceBCPara *fbp, int load_ind,
                          double newton_tol, int maxiter, int max_passes, const char *bondfile, int step,
                          double *stats)
{
    copyDouble2D(xyz_temp, xyz, nparticle, NDIM);
    copyDouble2D(F_temp, F, nparticle, nneighbors);
    copyDouble1D(Pex_temp, Pex, dim * nparticle);
    calcStiffness3DFiniteDifference(6);
    if (g_bcgroup) {
        group_disp_bc(nbd, dbp);
        group_force_bc(nbf, fbp);
    } else {
        setDispBC(nbd, dbp);
        setForceBC(nbf, fbp);
    }
    computeBondForceGeneral(4, load_ind);
    int ni_tot = 0, cgtot = 0, passes = 0, broken_tot = 0;
    double nr0 = 0, nreac0 = 0, nr = 0;
    for (;;) {
        updateRR();
        nr = cblas_dnrm2(dim * nparticle, residual, 1);
        double nreac = cblas_dnrm2(countNEqual(dispBC_index, nparticle * dim, 1), reaction_force, 1);
        double tolm = MAX(nr, nreac);
        if (passes == 0) {
            nr0 = nr;
            nreac0 = nreac;
        }
        int ni = 0;
        while (nr > newton_tol * tolm && ni < maxiter) {
            switchStateV(0);
            setDispBC_stiffnessUpdate3D();
            solverCG();
            cgtot += lpm_shim_last_cg_iters();
            computeBondForceGeneral(plmode, load_ind);
            updateRR();
            nr = cblas_dnrm2(dim * nparticle, residual, 1);
            ni++;
        }
        ni_tot += ni;
        passes++;
        computeStrain();
        int broken = updateDamageGeneral(bondfile, step, plmode);
        broken_tot += broken;
        updateCrack();
        switchStateV(1);
        if (broken <= 0 || passes >= max_passes)
            break;
        calcStiffness3DFiniteDifference(6);
    }
    if (stats) {
        stats[0] = ni_tot;
        stats[1] = nr0;
        stats[2] = nreac0;
        stats[3] = nr;
        stats[4] = cgtot;
        stats[5] = passes;
        stats[6] = broken_tot;
    }
    return ni_tot;
}

/* ---- flat accessors for the pointer-of-pointer globals ---------------- */
void refd_get_d2(double **a, int rows, int cols, double *out)
{
    for (int i = 0; i < rows; i++)
        for (int j = 0; j < cols; j++)
            out[(size_t)i * cols + j] = a[i][j];
}

void refd_get_i2(int **a, int rows, int cols, int *out)
{
    for (int i = 0; i < rows; i++)
        for (int j = 0; j < cols; j++)
            out[(size_t)i * cols + j] = a[i][j];
}

void refd_get_d3(double ***a, int rows, int cols, int slot, double *out)
{
    for (int i = 0; i < rows; i++)
        for (int j = 0; j < cols; j++)
            out[(size_t)i * cols + j] = a[i][j][slot];
}

void refd_set_d2(double **a, int rows, int cols, const double *in)
{
    for (int i = 0; i < rows; i++)
        for (int j = 0; j < cols; j++)
            a[i][j] = in[(size_t)i * cols + j];
}

void refd_set_d3(double ***a, int rows, int cols, int slot, const double *in)
{
    for (int i = 0; i < rows; i++)
        for (int j = 0; j < cols; j++)
            a[i][j][slot] = in[(size_t)i * cols + j];
}

int refd_nnz_upper(void) { return K_pointer[nparticle][1]; }
void refd_set_threads(int n) { omp_set_num_threads(n); }
void refd_set_cg_tol(double r, double a) { lpm_shim_set_cg_tol(r, a); }
