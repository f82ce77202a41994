/*
 * lpm_legacy.h - reference-named drop-in entry points (liblpmgpu_legacy.so).
 *
 * These keep the signatures of the LPM-C reference's solve path and operate
 * on its global state (the extern variables of include/lpm.h: xyz, Kn, Tv,
 * F, dLp, J2_alpha, K_global, residual, ...), which the host program defines
 * and allocates exactly as src/lpmc_project.c:19-45 and
 * src/initialization.c:1120-1194 do.  Linking this library in place of the
 * reference's src/stiffness.c, src/solver.c, src/constitutive.c and
 * src/boundary.c moves the hot path onto the GPU; the host keeps the rest
 * (lattice generation, neighbour search, strain recovery, output).
 *
 * Data ownership: the host globals stay authoritative.  Each call uploads
 * the globals it reads and writes back every global the reference function
 * writes, so host code that inspects or edits them between calls sees the
 * reference's values.  The first call (calcKnTv) builds the GPU specimen
 * from the host's particle positions on device 0.
 *
 * Error convention (as the reference): fatal errors print a message and
 * exit(); lpm_legacy_status() reports the last step status bits.
 * Not thread-safe; not reentrant (global state, like the reference).
 */
#ifndef LPM_LEGACY_H
#define LPM_LEGACY_H

#ifdef __cplusplus
extern "C" {
#endif

struct dispBCPara;
struct forceBCPara;

/* src/stiffness.c:11 (include/stiffness.h:5) */
void calcKnTv(void);
/* src/lpm_basic.c:127 (include/lpm_basic.h:13): strain_tensor from the bond
 * stretches dL of the last force evaluation (weighted least squares). */
void computeStrain(void);
/* src/stiffness.c:519 (include/stiffness.h:6); called with an ignored
 * argument at src/lpmc_project.c:462, hence the unprototyped form. */
void updateRR();
/* src/stiffness.c:271 (include/stiffness.h:7): 2D is not supported (exits) */
void calcStiffness2DFiniteDifference(int plmode);
/* src/stiffness.c:384 (include/stiffness.h:8): analytic tangent on the GPU,
 * written to K_global/IK/JK in the reference's upper CSR layout */
void calcStiffness3DFiniteDifference(int plmode);

/* src/solver.c:3 (include/solver.h:5): solved with the GPU PCG */
void solverPARDISO(void);
/* src/solver.c:188 (include/solver.h:6) */
void solverCG(void);

/* src/constitutive.c:10 (include/constitutive.h:9) */
void switchStateV(int conv_flag);
/* src/constitutive.c:1864 (include/constitutive.h:11) */
void computeCab(void);
/* src/constitutive.c:88 (include/constitutive.h:14): plmode 0, 1, 4, 6 */
void computeBondForceGeneral(int plmode, int temp);
/* src/constitutive.c:228 (include/constitutive.h:15): all particles */
void computeBondForceElastic(int i);
/* src/constitutive.c:466 (include/constitutive.h:16): all particles */
void computeBondForceJ2mixedLinear3D(int ii);
/* src/constitutive.c:866 (include/constitutive.h:18): all particles */
void computeBondForceCPMiehe(int ii);
/* src/constitutive.c:167 (include/constitutive.h:19): all particles */
void computeBondForceIncrementalUpdating(int ii);
/* src/constitutive.c:689, :286: not on the GPU path (exit with a message) */
void computeBondForceJ2nonlinearIso(int ii);
void computeBondForceJ2energyReturnMap(int ii, int load_indicator);
/* src/constitutive.c:149-164 (include/constitutive.h:22-27): main's damage
 * update on the GPU damage stage (lpm_damage_update), which the first damage
 * call switches on with the globals damage_L, damage_threshold, damagec_A,
 * critical_bstrain and nbreak: ductile nonlocal damage for plmode 0, brittle
 * bond breaking for plmode 6 (the global nbreak; a different nbreak argument
 * of updateBrittleDamage is not applied), 0 for crystal plasticity.  Reads and
 * writes damage_broken, damage_w, damage_D[.][.][0], damage_nonlocal[.][0];
 * appends the broken bonds to dataName in the reference's format. */
int updateDamageGeneral(const char *dataName, int tstep, int plmode);
int updateBrittleDamage(const char *dataName, int tstep, int nbreak);
int updateDuctileDamagePwiseNonlocal(const char *dataName, int tstep);
/* src/constitutive.c:1529-1756: models main does not select; not on the GPU
 * path (exit with a message) */
int updateDuctileDamageBwiseLocal(const char *dataName, int tstep);
int updateDuctileDamagePwiseLocal(const char *dataName, int tstep);
int updateDuctileDamageBwiseNonlocal(const char *dataName, int tstep);
/* src/constitutive.c:1399-1434 (include/constitutive.h:29): F scaled by
 * damage_w, Pin, nb, damage_visual, fix_index of particles without bonds */
void updateCrack(void);

/* src/boundary.c:12, :48 (include/boundary.h:13-14) */
void setDispBC(int nboundDisp, struct dispBCPara *dBP);
void setForceBC(int nboundForce, struct forceBCPara *fBP);
/* src/boundary.c:72 (include/boundary.h:10): 2D is not supported (exits) */
void setDispBC_stiffnessUpdate2D(void);
/* src/boundary.c:159 (include/boundary.h:11) */
void setDispBC_stiffnessUpdate3D(void);

/* ---- additions (no counterpart in the reference) ----------------------- */
/* Solver options for the legacy path: a pointer to an lpm_solver_opts of
 * lpm_gpu.h (precision, tolerances). */
int lpm_legacy_set_solver(const void *lpm_solver_opts_ptr);
/* Status bits of the last solve / force call (LPM_STATUS_* of lpm_gpu.h). */
int lpm_legacy_status(void);
/* Release the GPU specimen (the next calcKnTv rebuilds it). */
void lpm_legacy_reset(void);
/* Host<->device bytes moved by the legacy calls since the last reset. */
void lpm_legacy_traffic(long long *h2d, long long *d2h, int reset);

#ifdef __cplusplus
}
#endif

#endif
