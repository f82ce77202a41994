/*
 * lpm_oracle: CPU restatement of the LPM-C quasi-static solve path (FP64).
 *
 * TEST INFRASTRUCTURE ONLY.  This is the checker for the GPU library: tests,
 * __graft_entry__.smoke() and bench.py's CPU-baseline leg may call it; the
 * product never links it.  It restates, in plain C with an explicit state
 * struct instead of the reference's globals, the algorithm of:
 *   createCuboid            src/initialization.c:6-459  (SC, FCC; no rotation)
 *   searchNormalNeighbor    src/neighbor.c:9-46
 *   searchAFEMNeighbor      src/neighbor.c:49-141
 *   calcKnTv                src/stiffness.c:145-235
 *   computedL               src/lpm_basic.c:252-291
 *   computeBondForceElastic src/constitutive.c:228-283
 *   calcStiffness3DFiniteDifference src/stiffness.c:384-516
 *   setDispBC / setForceBC  src/boundary.c:12-70
 *   setDispBC_stiffnessUpdate3D src/boundary.c:159-281
 *   solverCG                src/solver.c:188-270
 *   computeBondForceIncrementalUpdating src/constitutive.c:167-225
 *   computeBondForceJ2mixedLinear3D     src/constitutive.c:466-686
 *   computeBondForceCPMiehe             src/constitutive.c:866-1396
 *   computeCab              src/constitutive.c:1864-1917
 *   slipSysDefine3D         src/initialization.c:563-638
 *   computeStress           src/lpm_basic.c:53-125
 *   switchStateV            src/constitutive.c:10-85
 *   updateRR                src/stiffness.c:519-534
 *   load-step Newton loop   src/lpmc_project.c:382-471
 *   updateDamageGeneral     src/constitutive.c:149-164 (ductile pointwise
 *                           nonlocal :1757-1862, brittle :1437-1527)
 *   updateCrack             src/constitutive.c:1399-1434
 *   main's damage stage and re-solve  src/lpmc_project.c:466-470, :528-546
 * Arithmetic follows the reference's operation order (compile with
 * -ffp-contract=off), and the BLAS/LAPACK/RCI-CG calls go through the same
 * MKL-API shim the reference is linked against, so results are bit-identical
 * to the reference run single-threaded.  Extensions beyond the reference:
 * elastic constants, yield stress and hardening modulus per particle.
 */
#ifndef LPM_ORACLE_H
#define LPM_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct lpm_oracle lpm_oracle;

typedef struct {
    int type;
    char flag;
    double step;
} lo_disp_bc; /* layout of struct dispBCPara (include/lpm.h:83-88) */

typedef struct {
    int type;
    char flag1;
    double step1;
    char flag2;
    double step2;
    char flag3;
    double step3;
} lo_force_bc; /* layout of struct forceBCPara (include/lpm.h:90-99) */

lpm_oracle *lo_create(void);
void lo_free(lpm_oracle *o);
/* lattice 2 (SC) or 3 (FCC); returns the particle count or -1 */
int lo_setup_lattice(lpm_oracle *o, int lattice, double radius, const double *box);
/* user-supplied particle positions instead of a generated lattice */
int lo_setup_particles(lpm_oracle *o, int lattice, double radius, int n, const double *xyz);
void lo_set_types(lpm_oracle *o, const int *type);
/* per-particle C11/C12/C44, yield stress, hardening; xi = kinematic share */
void lo_set_material(lpm_oracle *o, const double *c11, const double *c12, const double *c44,
                     const double *sy, const double *H, double xi, int plmode);
/* cp: tau0, taus, h0, p, q, eta, maxloop, dtime */
void lo_set_cp(lpm_oracle *o, const double *cp);
void lo_init_state(lpm_oracle *o);
void lo_set_threads(int n);

void lo_computedL(lpm_oracle *o);
void lo_fd_stiffness(lpm_oracle *o);
void lo_fd_stiffness_range(lpm_oracle *o, int i0, int i1);
double lo_fd_stiffness_timing(lpm_oracle *o, int count, int threads);
void lo_set_disp_bc(lpm_oracle *o, int n, const lo_disp_bc *d);
void lo_set_force_bc(lpm_oracle *o, int n, const lo_force_bc *f);
void lo_bc_stiffness_update(lpm_oracle *o);
int lo_solver_cg(lpm_oracle *o, double rtol_sq, double atol_sq);
void lo_force(lpm_oracle *o, int plmode);
/* damage parameters (damage_L, damage_threshold, damagec_A,
 * critical_bstrain, nbreak; defaults as src/lpmc_project.c:239-244) */
void lo_set_damage(lpm_oracle *o, double L, double threshold, double cA, double crit_bstrain, int nbreak);
int lo_damage_update(lpm_oracle *o, int plmode);
void lo_update_crack(lpm_oracle *o);
/* the brittle pass's choice among k candidates in scan order: sorts the
 * arrays in place, returns the index of the first chosen entry */
int lo_brittle_select(int *bi, int *bj, double *bs, int k, int nbreak);
/* broken bonds logged so far as (i, neighbour) pairs; pairs may be NULL */
int lo_broken_log(const lpm_oracle *o, int *pairs);
int lo_load_step_damage(lpm_oracle *o, int nbd, const lo_disp_bc *d, int nbf, const lo_force_bc *f,
                        double newton_tol, int maxiter, double cg_rtol_sq, double cg_atol_sq, int max_passes,
                        double *stats);
void lo_switch_state(lpm_oracle *o, int flag);
void lo_update_rr(lpm_oracle *o);
/* stats: iterations, |r0|, |reaction0|, |r| final, total CG iterations */
int lo_load_step(lpm_oracle *o, int nbd, const lo_disp_bc *d, int nbf, const lo_force_bc *f,
                 double newton_tol, int maxiter, double cg_rtol_sq, double cg_atol_sq,
                 double *stats);
/* Compute the upper CSR pattern (IK, JK 1-based) without values. */
void lo_csr_pattern(lpm_oracle *o);
/* CPU-baseline timing: nit threaded CG iterations on the current K/residual. */
int lo_cg_iterations(lpm_oracle *o, int nit);

/* sizes and raw views (row-major [i][j]) */
int lo_n(const lpm_oracle *o);
int lo_nn(const lpm_oracle *o);
int lo_nnz(const lpm_oracle *o);
int lo_nslip(const lpm_oracle *o);
int lo_nconn_max(const lpm_oracle *o);
double *lo_d(lpm_oracle *o, const char *name);
int *lo_i(lpm_oracle *o, const char *name);

#ifdef __cplusplus
}
#endif

#endif
