/*
 * lpm_gpu.h - C ABI of the GB300 (sm_103a) implementation of the LPM-C
 * quasi-static solve path.
 *
 * One context owns one lattice specimen resident on one GPU: particle
 * positions, bond lists, the fixed block-CSR stiffness pattern, material,
 * state variables and solver work space.  All entry points return LPM_OK (0)
 * or a negative LPM_ERR_* code; lpm_last_error() gives the message.  A
 * context is not thread-safe; use one host thread per context.
 *
 * Each entry point replaces one function (or a fixed sequence) of the
 * reference, cited as file:line of ymlasu/LPM-C.  The reference-named
 * drop-in symbols operating on the include/lpm.h globals are declared in
 * lpm_legacy.h.
 */
#ifndef LPM_GPU_H
#define LPM_GPU_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define LPM_OK 0
#define LPM_ERR_ARG (-1)      /* bad argument or call order */
#define LPM_ERR_CUDA (-2)     /* CUDA runtime failure */
#define LPM_ERR_NOMEM (-3)    /* device or host allocation failed */
#define LPM_ERR_DEVICE (-4)   /* a device-side check failed (status word) */

/* step status bits (lpm_step_stats.status); the step still completes */
#define LPM_STATUS_NEWTON_MAXIT 1 /* Newton loop stopped at maxiter (reference: MAXITER) */
#define LPM_STATUS_CG_MAXIT 2     /* a linear solve stopped at its iteration cap */
#define LPM_STATUS_NAN 4          /* a residual norm was not finite */
#define LPM_STATUS_CP_SINGULAR 8  /* singular slip-system Jacobian (reference exits) */
#define LPM_STATUS_DEVICE_WAIT 16 /* a bounded device-side wait ran out (streamed product); the solve stopped */

#define LPM_PREC_FP64 0  /* FP64 stiffness, SpMV and PCG */
#define LPM_PREC_MIXED 1 /* FP32 stiffness/SpMV/PCG inside FP64 iterative refinement */
#define LPM_PRECOND_BJ 0  /* block-Jacobi (3 x 3 diagonal blocks), as solverCG's diagonal preconditioner */
#define LPM_PRECOND_AMG 1 /* smoothed-aggregation multigrid V-cycle (rigid-body modes, FP64 vectors) */

/* constitutive modes (plmode, src/constitutive.c:88-146) */
#define LPM_PL_J2 0        /* J2 mixed linear hardening */
#define LPM_PL_CP 1        /* crystal plasticity (Miehe) */
#define LPM_PL_PREDICTOR 4 /* elastic incremental predictor */
#define LPM_PL_ELASTIC 6   /* elastic */

typedef struct lpm_ctx lpm_ctx;

/* same layout as struct dispBCPara (include/lpm.h:83-88) */
typedef struct {
    int type;
    char flag; /* 'x', 'y' or 'z' */
    double step;
} lpm_disp_bc;

/* same layout as struct forceBCPara (include/lpm.h:90-99) */
typedef struct {
    int type;
    char flag1;
    double step1;
    char flag2;
    double step2;
    char flag3;
    double step3;
} lpm_force_bc;

typedef struct {
    int precision;      /* LPM_PREC_FP64 or LPM_PREC_MIXED */
    double newton_tol;  /* stop when |r| <= tol * max(|r0|, |reaction0|) (TOLITER, include/lpm.h:41) */
    int newton_maxiter; /* MAXITER (include/lpm.h:39) */
    double cg_rtol;     /* linear solve: |b - K x| <= cg_rtol * |b| */
    int cg_maxiter;     /* cap on PCG iterations per solve (FP64) or per inner solve (mixed) */
    double inner_rtol;  /* mixed: FP32 residual drop between FP64 reliable updates (default 0.1) */
    int refine_maxiter; /* mixed: cap on FP64 reliable updates per solve */
    int check_every;    /* PCG iterations between host convergence checks (graph chunk) */
    int use_graphs;     /* capture PCG chunks as CUDA graphs */
    int mixed_vectors;  /* mixed: 32 = FP32 CG vectors, 64 = FP64 CG vectors (FP32 stiffness and products);
                           with 32, a solve whose FP32 iteration stagnates is redone with FP64
                           vectors, and so are the context's later solves */
    int newton_accel;   /* 0: modified Newton as the reference (u += K^-1 r); m > 0: the same
                           fixed-point iteration with Anderson acceleration of depth m (<= 16) */
    double cg_forcing;  /* 0 (default): every linear solve to cg_rtol.  eta_max in (0, 1): inexact
                           Newton, the k-th solve of a step only to eta_k = the Eisenstat-Walker
                           choice 2 (0.9 (|r_k| / |r_k-1|)^2, safeguarded), capped at eta_max, never
                           tighter than cg_rtol nor than half the Newton target over |r_k|.  The
                           step converges to the same Newton tolerance with far fewer PCG
                           iterations when modified Newton contracts slowly (plastic range). */
    int preconditioner; /* LPM_PRECOND_BJ (default) or LPM_PRECOND_AMG.  AMG: the PCG runs with FP64
                           vectors (FP32 stiffness and FP64 reliable updates under LPM_PREC_MIXED) and
                           a V-cycle of a smoothed-aggregation hierarchy built on the host at the
                           first solve; it is rebuilt when the constrained DOFs change or a solve
                           needs more than amg_rebuild times the iterations of the first solve after
                           the last build.  Single specimens only (batches use block-Jacobi). */
    double amg_spacing; /* AMG: edge of a level-0 aggregate box; 0 (default) = 6 particle radii
                           (3 x 3 x 3 nearest-neighbour spacings) */
    double amg_rebuild; /* AMG: iteration growth that triggers a rebuild (default 2.5) */
    int amg_sweeps;     /* AMG: damped block-Jacobi sweeps before and after each coarse correction
                           (1..4, default 1: fewest stiffness passes per solve) */
    int recycle;        /* 0 (default): every linear solve starts from zero.  m in 1..8: the
                           Newton solves of one load step share the stiffness, so each starts
                           from the Galerkin combination of the step's last m solutions (their
                           right-hand sides are K times them, so neither the guess nor its
                           residual needs an extra product beyond one true residual); the solve
                           still ends at cg_rtol relative to its own right-hand side.  In the
                           plastic range, where modified Newton contracts slowly, the guess
                           removes 2 to 4 of the 10 decades a solve must gain. */
} lpm_solver_opts;

typedef struct {
    int newton_iters;
    int cg_iters;      /* PCG iterations summed over the step (inner iterations for mixed) */
    int refine_iters;  /* FP64 refinement sweeps summed over the step */
    int spmv_calls;
    int status;        /* LPM_STATUS_* bits */
    double res0, reac0, res_final;
    double ms_stiffness, ms_solve, ms_force;
    int damage_passes;   /* damage stage: Newton passes of the step (1 + re-solves after breaking) */
    int bonds_broken;    /* damage stage: sum of updateDamageGeneral's return values over the passes */
    int amg_builds;      /* AMG: hierarchy builds during the step */
    double ms_amg_build; /* AMG: host time of those builds (stiffness download, setup, upload) */
    int fp64_fallbacks;  /* mixed multigrid: solves that failed with FP32 products and were redone
                            with FP64 ones (the context keeps FP64 products from then on) */
} lpm_step_stats;

/* ---- context ------------------------------------------------------------ */
int lpm_create(lpm_ctx **ctx, int device);
void lpm_destroy(lpm_ctx *ctx);
const char *lpm_last_error(void);
/* Launch everything on the given cudaStream_t (NULL = the context's own stream). */
int lpm_set_stream(lpm_ctx *ctx, void *stream);
void lpm_default_solver_opts(lpm_solver_opts *opts);
int lpm_set_solver(lpm_ctx *ctx, const lpm_solver_opts *opts);

/* ---- setup -------------------------------------------------------------- */
/* createCuboid (src/initialization.c:6-459, lattice 2 = SC, 3 = FCC, no
 * rotation) + initMatrices + searchNormalNeighbor (src/neighbor.c:9-46) +
 * searchAFEMNeighbor (src/neighbor.c:49-141).  Returns the particle count
 * (>0) or an error code. */
int lpm_setup_lattice(lpm_ctx *ctx, int lattice, double radius, const double box[6]);
/* Same, with caller-supplied positions (n x 3, row-major). */
int lpm_setup_particles(lpm_ctx *ctx, int lattice, double radius, int n, const double *xyz);
int lpm_nparticle(const lpm_ctx *ctx);
/* particle type: selects boundary conditions as in setDispBC/setForceBC */
int lpm_set_types(lpm_ctx *ctx, const int *type);
/* calcKnTv (src/stiffness.c:145-235) with per-particle C11, C12, C44, plus
 * per-particle yield stress and hardening modulus (sigmay, J2_H) and the
 * kinematic share J2_xi; plmode selects the constitutive law. */
int lpm_set_material(lpm_ctx *ctx, const double *c11, const double *c12, const double *c44,
                     const double *sigmay, const double *hardening, double xi, int plmode);
/* crystal plasticity constants: tau0, taus, h0, p, q, eta, maxloop, dtime
 * (cp_tau0, cp_taus, cp_h0, cp_p, cp_q, cp_eta, cp_maxloop, dtime of include/lpm.h) */
int lpm_set_cp(lpm_ctx *ctx, const double cp[8]);
/* computedL (src/lpm_basic.c:252-291), slipSysDefine3D
 * (src/initialization.c:563-638) and computeCab (src/constitutive.c:1864-1917);
 * resets the state variables to zero. */
int lpm_init_state(lpm_ctx *ctx);

/* ---- the hot path -------------------------------------------------------- */
/* One load step: src/lpmc_project.c:385-471 (stiffness, displacement and force
 * BCs, elastic predictor, Newton loop of PCG solve + bond force update +
 * residual, state commit).  With the damage stage enabled (lpm_set_damage),
 * also main's damage updates and re-solves after broken bonds
 * (src/lpmc_project.c:466-470, :528-546). */
int lpm_load_step(lpm_ctx *ctx, int nbd, const lpm_disp_bc *dbc, int nbf, const lpm_force_bc *fbc,
                  lpm_step_stats *stats);
/* calcStiffness3DFiniteDifference (src/stiffness.c:384-516): the elastic
 * tangent at the current configuration, computed analytically, symmetrised
 * as the reference does, into the device block-CSR. */
int lpm_assemble_stiffness(lpm_ctx *ctx);
/* setDispBC / setForceBC (src/boundary.c:12-70) on the device state. */
int lpm_apply_bc(lpm_ctx *ctx, int nbd, const lpm_disp_bc *dbc, int nbf, const lpm_force_bc *fbc);
/* computeBondForceGeneral (src/constitutive.c:88-146) for plmode 0, 1, 4, 6,
 * including computeStress and switchStateV(2), then updateRR
 * (src/stiffness.c:519-534).  norms (may be NULL): |residual|, |reaction|. */
int lpm_compute_force(lpm_ctx *ctx, int plmode, double norms[2]);
/* computeStrain (src/lpm_basic.c:127-249): weighted least-squares strain
 * tensor of every particle from its bond stretches of the last force
 * evaluation; read it as "strain_tensor" (n x 6, s11 s22 s33 s23 s13 s12
 * order). */
int lpm_compute_strain(lpm_ctx *ctx);
/* ---- damage stage ---------------------------------------------------------
 * The reference's main runs, after each converged load step,
 * updateDamageGeneral (src/constitutive.c:149-164: ductile pointwise nonlocal
 * damage for J2, :1757-1862; brittle bond breaking for elastic bonds,
 * :1437-1527; nothing for crystal plasticity), then updateCrack (:1399-1434:
 * bond forces scaled by 1 - D, current bond counts) and, when bonds broke,
 * recomputes the stiffness and re-enters the Newton loop of the same load
 * step (src/lpmc_project.c:528-546).  Off by default (the parity target of
 * the solve path); lpm_set_damage after lpm_init_state switches it on with
 * all bonds intact.  The stress-averaging weights follow the broken bonds as
 * the reference's opp_flag does; the stiffness drops broken bonds (exact when
 * a bond and its reverse break together, which the ductile update always
 * does).  Not combined with batches or the adjoint. */
typedef struct {
    int enabled;             /* 0: no damage stage (default) */
    double length;           /* damage_L: nonlocal length; weights cut at 3 L */
    double threshold;        /* damage_threshold: particles above it lose all bonds */
    double triax_coeff;      /* damagec_A (J2_triaxiality is 0 in the reference) */
    double critical_bstrain; /* brittle: elastic bond strain at which a bond breaks */
    int nbreak;              /* brittle: at most this many bonds break per pass */
    int max_passes;          /* cap on Newton passes of one load step */
} lpm_damage_opts;
/* enabled = 0 and the values of src/lpmc_project.c:239-244 (L 0.5,
 * threshold 0.9, A 0, critical strain 1e-2, nbreak 20), max_passes 1000 */
void lpm_default_damage_opts(lpm_damage_opts *opts);
int lpm_set_damage(lpm_ctx *ctx, const lpm_damage_opts *opts);
/* Bonds broken so far, as (particle, partner) pairs in the order the
 * reference writes them to its bond file.  pairs may be NULL to query the
 * count; otherwise it holds 2 * capacity ints. */
int lpm_damage_log(lpm_ctx *ctx, int *pairs, int capacity, int *count);
/* main's damage stage one function at a time, for the reference-named
 * drop-in: lpm_damage_update is updateDamageGeneral (src/constitutive.c:149-164)
 * on the context's current state for its plmode (ductile nonlocal damage for
 * J2, :1757-1862; brittle bond breaking for elastic bonds, :1437-1527;
 * nothing for crystal plasticity), *broken its return value, the broken
 * bonds appended to lpm_damage_log; lpm_damage_crack is updateCrack
 * (:1399-1434).  Both need the damage stage on (lpm_set_damage). */
int lpm_damage_update(lpm_ctx *ctx, int *broken);
int lpm_damage_crack(lpm_ctx *ctx);
/* The brittle pass's choice (updateBrittleDamage, src/constitutive.c:1471-1520)
 * among k candidate bonds b = slot * n + particle, given in any order with
 * their bond strains: scan order, then, above nbreak candidates, the
 * reference's shell sort and its last nbreak entries.  Host logic only (no
 * context, no GPU); chosen receives up to k bonds, *nchosen their count. */
int lpm_damage_brittle_select(const int *bonds, const double *strain, int k, int n, int nbreak, int *chosen,
                              int *nchosen);

/* switchStateV (src/constitutive.c:10-85): 0 = converged -> current,
 * 1 = current -> converged. */
int lpm_switch_state(lpm_ctx *ctx, int flag);
/* solverCG (src/solver.c:188-270) with setDispBC_stiffnessUpdate3D
 * (src/boundary.c:159-281) folded in: solve K du = residual on the
 * unconstrained DOFs, then xyz += du. */
int lpm_solve(lpm_ctx *ctx, lpm_step_stats *stats);
/* Start-of-step bookkeeping of src/lpmc_project.c:387-389: remember xyz and
 * the bond forces for the elastic predictor. */
int lpm_begin_step(lpm_ctx *ctx);

/* ---- data exchange --------------------------------------------------------- */
/* Copy a named array between host and device.  Names and shapes (n = particles,
 * nn = bond slots per particle, row-major like the reference's [i][j]):
 *   xyz, xyz_initial, xyz_temp (n x 3), Pin, Pex, residual, disp (3n),
 *   F, dL, csx, csy, csz, Kn, Tv, distance_initial (n x nn),
 *   dLp (n x nn, converged), dLp_trial, J2_alpha (n, converged), J2_beta (n x 6),
 *   stress_tensor, strain_tensor (n x 6), neighbors, nsign (n x nn, int32), nb (n, int32),
 *   dispBC_index (3n, int32), type (n, int32), conn (n x 61, int32), nb_conn (n),
 *   cp_gy (n x nslip), cp_A (n), cp_A_single (n x nslip), J2_dlambda (n);
 *   with the damage stage on: damage_broken, damage_w, damage_D (n x nn,
 *   converged), damage_D0 (n x nn, current), damage_nonlocal (n, converged),
 *   damage_nonlocal0 (n, current), damage_visual (n), nb_current (n, int32:
 *   intact bonds; nb stays nb_initial); damage_visual and nb_current are
 *   read-only. */
int lpm_get(lpm_ctx *ctx, const char *name, void *dst, size_t bytes);
int lpm_set(lpm_ctx *ctx, const char *name, const void *src, size_t bytes);
int lpm_get_sizes(const lpm_ctx *ctx, int *n, int *nn, int *nslip, long long *nnz_blocks);
/* The current stiffness in the reference's layout: 1-based upper-triangular
 * scalar CSR (K_global, IK, JK of calcStiffness3DFiniteDifference).  Any
 * pointer may be NULL; *nnz receives the entry count. */
int lpm_export_upper_csr(lpm_ctx *ctx, double *K_global, int *IK, int *JK, long long *nnz);
/* y = K x on the full (unmodified) block-CSR; x, y host arrays of 3n. */
int lpm_spmv(lpm_ctx *ctx, const double *x, double *y);
/* Solve K x = b (with the BC mask) for a host right-hand side; no xyz update. */
int lpm_solve_rhs(lpm_ctx *ctx, const double *b, double *x, lpm_step_stats *stats);
/* Average duration (ms) of the SpMV kernel launches since the last reset,
 * measured with CUDA events on the context's stream, and their count. */
int lpm_spmv_timing(lpm_ctx *ctx, double *avg_ms, long long *count, int reset);
/* Block-CSR byte count of one SpMV (values + column indices + vectors),
 * for the given precision, unpadded (algorithmic). */
double lpm_spmv_bytes(const lpm_ctx *ctx, int precision);

/* ---- autotuner ------------------------------------------------------------------ */
/* Launch shapes of the solve: the SpMV tile (lanes per block row x
 * consecutive blocks per lane: variant 0 = 16 x 4, 1 = 8 x 4, 2 = 32 x 2,
 * 3 = 4 x 4), its thread blocks per SM, and the thread blocks per SM of the
 * PCG vector kernels.  No counterpart in the reference, whose solve is MKL's. */
typedef struct lpm_tuning {
    int spmv_variant;
    int spmv_lanes;        /* output: lanes per block row */
    int spmv_blocks;       /* output: consecutive blocks per lane */
    int spmv_per_sm;
    int cg_per_sm;
    double spmv_ms;        /* lpm_autotune: time of the chosen SpMV shape */
    double spmv_ms_default;/* lpm_autotune: time of the default shape (0, 8, 8) */
    int smooth_lanes;      /* output: lanes per block row of the multigrid level-0 smoother (16, 8, 4) */
    double smooth_ms;      /* lpm_autotune: time of one smoother pass in the chosen shape (0: not tuned) */
    int diff_stream;       /* mixed multigrid PCG: difference-form product fed by registers (0) or
                              streamed through shared memory by the bulk-copy engine: tiles of 16
                              rows with 1 or 2 thread blocks per SM (1, 2), tiles of 8 rows with 5
                              (3); same arithmetic per row */
    int smooth_stream;     /* multigrid level-0 smoother: register-fed (0, smooth_lanes per row) or
                              streamed as diff_stream (1, 2; 3: tiles of 8 rows, 6 thread blocks per
                              SM; 16 lanes per row) */
} lpm_tuning;
/* Time every SpMV shape (and vector-kernel grid) on the context's current
 * stiffness with CUDA events and keep the fastest.  Needs an assembled
 * stiffness (lpm_assemble_stiffness or a load step).  Different shapes sum a
 * row in different orders, so results can change in the last bits. */
int lpm_autotune(lpm_ctx *ctx, lpm_tuning *out);
int lpm_set_tuning(lpm_ctx *ctx, const lpm_tuning *t);
int lpm_get_tuning(const lpm_ctx *ctx, lpm_tuning *t);

/* ---- batched specimens ------------------------------------------------------- */
/* Many independent specimens of uneven size (parameter sweeps, random
 * heterogeneity) in one context.  The reference runs one specimen per process
 * (the main loop of src/lpmc_project.c:382-471); here the specimens'
 * particles are concatenated (specimen s owns particles offsets[s] ..
 * offsets[s+1]-1) and every kernel covers all of them in one launch.
 *
 * lpm_setup_batch: createCuboid + searchNormalNeighbor + searchAFEMNeighbor
 * (src/initialization.c:241-284, src/neighbor.c:9-141) for nspec boxes
 * (boxes[6 s .. 6 s + 5] as lpm_setup_lattice's box), one lattice and radius.
 * Returns the total particle count.  Types, material (per particle, so per
 * specimen) and lpm_init_state then act on the concatenated particles. */
int lpm_setup_batch(lpm_ctx *ctx, int lattice, double radius, int nspec, const double *boxes);
/* Specimen count; offsets (may be NULL) receives nspec + 1 particle offsets. */
int lpm_batch_offsets(const lpm_ctx *ctx, int *offsets);
/* One load step of src/lpmc_project.c:385-471 for every specimen at once:
 * dbc holds nbd displacement BCs per specimen (nspec x nbd, specimen-major),
 * stats (may be NULL) nspec records.  Each specimen runs its own Newton test
 * and its own PCG scalars and convergence test (block-Jacobi PCG of all
 * specimens in one launch per kernel, chunks of iterations as CUDA graphs).
 * A specimen that has left the Newton loop keeps its configuration while the
 * others iterate; its bond forces are re-evaluated at that configuration.
 * Force BCs are not supported in a batch. */
int lpm_batch_load_step(lpm_ctx *ctx, int nbd, const lpm_disp_bc *dbc, lpm_step_stats *stats);

/* ---- adjoint ------------------------------------------------------------------ */
/* Gradients of a function of the reaction-force curve with respect to the
 * per-particle material (E, nu, yield stress, hardening modulus) of a J2
 * isotropic-hardening load path, as a forward/backward pair: forward runs the
 * load steps and returns the curve, backward takes dL/dR per step and
 * returns dL/d(material), like a torch.autograd.Function.  No counterpart in
 * the reference (whose observable is writeReaction, src/data_handler.c:309-335:
 * R_n = -sum over particles of type rtype of the internal force component
 * rcomp after load step n). */
typedef struct lpm_adjoint_opts {
    int checkpoint_every; /* load steps between stored states (default 10); the
                             backward run recomputes the steps in between */
    int gmres_restart;    /* Krylov basis of the adjoint solve (default 30) */
    int gmres_maxiter;    /* per load step (default 600) */
    double gmres_rtol;    /* relative residual of the adjoint solve (default 1e-10) */
} lpm_adjoint_opts;
typedef struct lpm_adjoint_stats {
    int steps, recomputed_steps, checkpoints;
    int gmres_iters;       /* adjoint Krylov iterations of the backward run */
    int cg_iters;          /* PCG iterations of the forward run */
    int cg_iters_backward; /* PCG iterations of the backward run (preconditioner) */
    int status;            /* LPM_STATUS_* bits of the forward run and the adjoint solves */
    double ms_forward, ms_backward;
} lpm_adjoint_stats;
void lpm_default_adjoint_opts(lpm_adjoint_opts *opts);
/* Sets the material from E, nu (C11, C12, C44 as src/lpmc_project.c:188-190),
 * sigmay, H (n each; J2, isotropic hardening), initialises the state and runs
 * nsteps load steps with bcs (nsteps x nbd, step-major).  R (may be NULL)
 * receives the nsteps reactions.  The context's solver options apply; every
 * step must take at least one Newton iteration. */
int lpm_adjoint_forward(lpm_ctx *ctx, const double *E, const double *nu, const double *sigmay, const double *H,
                        int nsteps, int nbd, const lpm_disp_bc *bcs, int rtype, int rcomp,
                        const lpm_adjoint_opts *opts, double *R);
/* dLdR: nsteps values.  Outputs (n each, any may be NULL): dL/dE, dL/dnu,
 * dL/dsigmay, dL/dH.  The context is left at the end of the forward run. */
int lpm_adjoint_backward(lpm_ctx *ctx, const double *dLdR, double *gE, double *gnu, double *gsy, double *gH,
                         lpm_adjoint_stats *stats);
/* Reverse mode of one J2 force evaluation (lpm_compute_force(ctx, LPM_PL_J2)
 * made from the converged state, e.g. after lpm_switch_state(ctx, 0)):
 * cotangents Pbar (3n) of the internal force, mu_dLp (n x nn) and mu_alpha (n)
 * of the new plastic state (may be NULL) -> xbar (3n), dLp_bar (n x nn),
 * alpha_bar (n), theta_bar (5 x n: C11, C12, C44, sigmay, H).  Outputs may be
 * NULL.  Allocates its work space. */
int lpm_force_vjp(lpm_ctx *ctx, const double *Pbar, const double *mu_dLp, const double *mu_alpha, double *xbar,
                  double *dLp_bar, double *alpha_bar, double *theta_bar);

/* ---- output in the reference's file formats ---------------------------------- */
/* writeDump (src/data_handler.c:42-85, LAMMPS dump; J2 or crystal-plasticity
 * columns by the context's plmode; damage columns are 0), writeDisp (:278-306),
 * writeReaction (:309-335), writeStress (:110-135): same text, byte for byte,
 * for the same data.  flag 's' starts the dump file, anything else appends.
 * lpm_write_dump copies the device arrays into pinned memory on the context's
 * stream and writes the file on a host thread (the next load step may run
 * meanwhile); lpm_write_wait joins it and reports its error.  The other
 * writers are synchronous. */
int lpm_write_dump(lpm_ctx *ctx, const char *path, int step, char flag, const double box[6]);
int lpm_write_wait(lpm_ctx *ctx);
int lpm_write_disp(lpm_ctx *ctx, const char *path, char c, int t1, int tstep);
int lpm_write_reaction(lpm_ctx *ctx, const char *path, char c, int t1, int tstep);
int lpm_write_stress(lpm_ctx *ctx, const char *path, int t1, int tstep);
int lpm_write_strain(lpm_ctx *ctx, const char *path, int t1, int tstep);  /* after lpm_compute_strain */
/* The same formats from host arrays in the reference's per-particle layout
 * (xyz n x 3, stress n x 6 as s11 s22 s33 s23 s13 s12, bond arrays n x nn;
 * plmode 1 reads cp_As (n x nslip) and cp_A, otherwise alpha). */
int lpm_format_dump(const char *path, int step, char flag, int n, const double box[6], int plmode, const int *type,
                    const double *xyz, const double *xyz0, const double *stress, const double *alpha,
                    const int *pl_flag, const double *cp_As, int nslip, const double *cp_A);
int lpm_format_disp(const char *path, char c, int t1, int tstep, int n, const int *type, const double *xyz,
                    const double *xyz0);
int lpm_format_reaction(const char *path, char c, int t1, int tstep, int n, int nn, const int *type, const int *nb,
                        const double *csx, const double *csy, const double *csz, const double *F);
int lpm_format_stress(const char *path, int t1, int tstep, int n, const int *type, const double *stress);
int lpm_format_strain(const char *path, int t1, int tstep, int n, const int *type, const double *strain);

/* ---- no-allocation entry point ----------------------------------------------- */
/* No counterpart in the reference: an allocation-free form of the residual
 * update for callers that cannot call cudaMalloc (their device memory comes
 * from their own pool or a fixed budget, so a library may not allocate).
 *
 * residual[d] = dispBC_index[d] * (Pex[d] - Pin[d]) over the 3n DOFs, and
 * norms = {|residual|, |Pin on the DOFs with dispBC_index == 0|} (the
 * quantities lpm_compute_force reports).  Pin, Pex, dispBC_index and residual
 * are DEVICE arrays of 3n entries on the current device, in the reference's
 * per-particle (x, y, z) order; norms is a host array or NULL.  With norms the
 * call waits for the stream, so norms must be NULL on a stream that is being
 * captured (the call then returns LPM_ERR_ARG); without norms it only enqueues
 * work on the stream.
 *
 * Allocates nothing: its only work space is a fixed 256 KB device array in
 * the library (held on every GPU that loads the library until exit), shared by
 * all calls on a device and keeping the last call's contents.  n beyond
 * LPM_NOALLOC_MAX_PARTICLES is rejected with LPM_ERR_ARG.  The first call on
 * each device looks up that array's device address and keeps it for the
 * process; make that first call before any stream capture.  A device reset
 * (cudaDeviceReset) can move the array, so after one the entry point must not
 * be called again in that process.  Calls whose kernels overlap on the GPU
 * race on the shared array: order them on one stream. */
#define LPM_NOALLOC_MAX_PARTICLES 4194304
int lpm_update_rr_noalloc(int n, const double *Pin, const double *Pex, const int *dispBC_index,
                          double *residual, double norms[2], void *stream);

#ifdef __cplusplus
}
#endif

#endif
