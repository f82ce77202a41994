// Reference-named drop-in layer (include/lpm_legacy.h) over the C ABI of
// include/lpm_gpu.h.  Operates on the host program's include/lpm.h globals:
// uploads what each reference function reads, runs it on the GPU, and writes
// back what it writes.  Host-side bookkeeping functions (setDispBC,
// setForceBC, updateRR, switchStateV, the K_global edit of
// setDispBC_stiffnessUpdate3D) run on the host exactly as in the reference,
// so the globals always hold the reference's values.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <utility>
#include <vector>
#include "lpm_gpu.h"
#include "lpm_legacy.h"

// Globals of include/lpm.h:55-81 used by the solve path (defined by the host
// program, as src/lpmc_project.c:19-45 does).
extern "C" {
extern int nparticle, nneighbors, dim, lattice, plmode, ntype, nslipSys, nbreak;
extern int *IK, *JK, *type, *dispBC_index, *fix_index, *nb, *nb_initial, *nb_conn;
extern int **neighbors, **K_pointer, **conn, **nsign;
extern double radius, particle_volume, J2_H, J2_xi, cp_tau0[3], cp_taus[3], cp_eta, cp_p, cp_h0, cp_q,
    cp_maxloop, dtime, damage_L, damage_threshold, damagec_A, critical_bstrain;
extern double *K_global, *residual, *Pin, *Pex, *disp, *sigmay, *reaction_force;
extern double *J2_dlambda, *J2_stresseq, *J2_stressm, *J2_triaxiality, *damage_visual;
extern double **xyz, **xyz_initial, **xyz_temp, **F, **F_temp, **csx, **csy, **csz, **Ce, **dL, **Kn, **Tv;
extern double **stress_tensor, **bond_stress, **J2_alpha, **J2_beta_eq, **cp_A, **cp_Cab;
extern double **damage_local, **damage_nonlocal, **strain_tensor, **damage_broken, **damage_w;
extern double ***dLp, ***J2_beta, ***cp_gy, ***cp_A_single, ***damage_D;
}

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

namespace {

lpm_ctx *g_ctx = nullptr;
lpm_solver_opts g_opts;
bool g_opts_set = false;
int g_status = 0;
long long g_h2d = 0, g_d2h = 0;
int g_plmode_dev = -1;
bool g_damage_on = false;  // the context's damage stage is on (first damage call)
int g_log_written = 0;     // broken bonds of lpm_damage_log already in the bond file

[[noreturn]] void die(const char *what)
{
    std::printf("LPM GPU drop-in: %s: %s\n", what, lpm_last_error());
    std::exit(5);
}

void check(int rc, const char *what)
{
    if (rc < 0)
        die(what);
}

lpm_ctx *ctx()
{
    if (!g_ctx) {
        std::printf("LPM GPU drop-in: calcKnTv() must run before the other solve-path calls\n");
        std::exit(5);
    }
    return g_ctx;
}

// Host vectors whose resize() does not zero-fill: every element is written
// by the parallel loop or the copy that fills it.
template <typename T>
struct NoInit : std::allocator<T> {
    template <typename U>
    struct rebind {
        typedef NoInit<U> other;
    };
    NoInit() = default;
    template <typename U>
    NoInit(const NoInit<U> &) noexcept
    {
    }
    template <typename U>
    void construct(U *p) noexcept
    {
        ::new (static_cast<void *>(p)) U;
    }
    template <typename U, typename... A>
    void construct(U *p, A &&...a)
    {
        ::new (static_cast<void *>(p)) U(std::forward<A>(a)...);
    }
};
typedef std::vector<double, NoInit<double>> dvec;

// flatten / scatter helpers for the pointer-of-pointer globals (rows in parallel)
dvec flat2(double **a, int rows, int cols)
{
    dvec v((size_t)rows * cols);
#pragma omp parallel for schedule(static)
    for (int i = 0; i < rows; i++)
        std::memcpy(&v[(size_t)i * cols], a[i], sizeof(double) * cols);
    return v;
}

void scatter2(double **a, const dvec &v, int rows, int cols)
{
#pragma omp parallel for schedule(static)
    for (int i = 0; i < rows; i++)
        std::memcpy(a[i], &v[(size_t)i * cols], sizeof(double) * cols);
}

dvec flat3(double ***a, int rows, int cols, int slot)
{
    dvec v((size_t)rows * cols);
#pragma omp parallel for schedule(static)
    for (int i = 0; i < rows; i++)
        for (int j = 0; j < cols; j++)
            v[(size_t)i * cols + j] = a[i][j][slot];
    return v;
}

void scatter3(double ***a, const dvec &v, int rows, int cols, int slot)
{
#pragma omp parallel for schedule(static)
    for (int i = 0; i < rows; i++)
        for (int j = 0; j < cols; j++)
            a[i][j][slot] = v[(size_t)i * cols + j];
}

void put(const char *name, const dvec &v)
{
    check(lpm_set(ctx(), name, v.data(), v.size() * sizeof(double)), name);
    g_h2d += (long long)(v.size() * sizeof(double));
}

dvec get(const char *name, size_t count)
{
    dvec v(count);
    check(lpm_get(ctx(), name, v.data(), v.size() * sizeof(double)), name);
    g_d2h += (long long)(v.size() * sizeof(double));
    return v;
}

void put_mask()
{
    std::vector<int> m(3 * (size_t)nparticle);
    for (int k = 0; k < 3 * nparticle; k++)
        m[k] = (dispBC_index[k] != 0 && fix_index[k] != 0) ? 1 : 0;
    check(lpm_set(ctx(), "dispBC_index", m.data(), m.size() * sizeof(int)), "dispBC_index");
    g_h2d += (long long)(m.size() * sizeof(int));
}

// computeStress's derived outputs (src/lpm_basic.c:101-123) from the stress tensor
void stress_derived()
{
#pragma omp parallel for schedule(static)
    for (int i = 0; i < nparticle; i++) {
        double *s = stress_tensor[i];
        double q = 0.0;
        for (int j = 0; j < 6; j++)
            q += (j < 3 ? 1.0 : 2.0) * s[j] * s[j];
        J2_stresseq[i] = std::sqrt(3.0 / 2.0 * q);
        J2_stressm[i] = 1.0 / 3.0 * (s[0] + s[1] + s[2]);
        if (J2_stresseq[i] > 1e-6)
            J2_triaxiality[i] = J2_stressm[i] / J2_stresseq[i];
        for (int j = 0; j < nb_initial[i]; j++)
            bond_stress[i][j] = s[0] * csx[i][j] * csx[i][j] + s[1] * csy[i][j] * csy[i][j] +
                                s[2] * csz[i][j] * csz[i][j] + 2 * s[3] * csy[i][j] * csz[i][j] +
                                2 * s[4] * csx[i][j] * csz[i][j] + 2 * s[5] * csx[i][j] * csy[i][j];
    }
}

// Upload what a force evaluation reads, run it, write back what it writes.
// The reference's switchStateV(2) is done by the caller on the host.
void device_force(int pl, bool stress_outputs)
{
    const int n = nparticle, nn = nneighbors;
    put("xyz", flat2(xyz, n, 3));
    put("Pex", dvec(Pex, Pex + 3 * (size_t)n));
    put_mask();
    put("dLp0", flat3(dLp, n, nn, 0));
    if (pl == 4) {
        put("xyz_temp", flat2(xyz_temp, n, 3));
        put("F_temp", flat2(F_temp, n, nn));
        put("csx", flat2(csx, n, nn));
        put("csy", flat2(csy, n, nn));
        put("csz", flat2(csz, n, nn));
    } else {
        put("J2_alpha0", [&] {
            dvec a(n);
            for (int i = 0; i < n; i++)
                a[i] = J2_alpha[i][0];
            return a;
        }());
        put("J2_beta0", flat3(J2_beta, n, 6, 0));
        if (pl == 1 && nslipSys > 0) {
            put("cp_gy0", flat3(cp_gy, n, nslipSys, 0));
            put("cp_A_single0", flat3(cp_A_single, n, nslipSys, 0));
            dvec a(n);
            for (int i = 0; i < n; i++)
                a[i] = cp_A[i][0];
            put("cp_A0", a);
        }
    }
    double norms[2];
    check(lpm_compute_force(ctx(), pl, norms), "computeBondForceGeneral");
    scatter2(F, get("F", (size_t)n * nn), n, nn);
    const dvec pin = get("Pin", 3 * (size_t)n);
    std::memcpy(Pin, pin.data(), pin.size() * sizeof(double));
    if (pl != 4) {
        scatter2(csx, get("csx", (size_t)n * nn), n, nn);
        scatter2(csy, get("csy", (size_t)n * nn), n, nn);
        scatter2(csz, get("csz", (size_t)n * nn), n, nn);
        scatter2(dL, get("dL", (size_t)n * nn), n, nn);
        scatter3(dLp, get("dLp2", (size_t)n * nn), n, nn, 2);
    }
    if (pl == 0) {
        const dvec a = get("J2_alpha2", n);
        for (int i = 0; i < n; i++)
            J2_alpha[i][2] = a[i];
        scatter3(J2_beta, get("J2_beta2", 6 * (size_t)n), n, 6, 2);
        const dvec dl = get("J2_dlambda", n);
        std::memcpy(J2_dlambda, dl.data(), dl.size() * sizeof(double));
    }
    if (pl == 1 && nslipSys > 0) {
        scatter3(cp_gy, get("cp_gy2", (size_t)n * nslipSys), n, nslipSys, 2);
        scatter3(cp_A_single, get("cp_A_single2", (size_t)n * nslipSys), n, nslipSys, 2);
        const dvec a = get("cp_A2", n);
        for (int i = 0; i < n; i++)
            cp_A[i][2] = a[i];
    }
    if (stress_outputs) {
        scatter2(stress_tensor, get("stress_tensor", 6 * (size_t)n), n, 6);
        stress_derived();
    }
}

// The context's damage stage with main's parameters (src/lpmc_project.c:239-244
// set them as globals), switched on by the first damage call.
void ensure_damage()
{
    if (g_damage_on)
        return;
    lpm_damage_opts o;
    lpm_default_damage_opts(&o);
    o.enabled = 1;
    o.length = damage_L;
    o.threshold = damage_threshold;
    o.triax_coeff = damagec_A;
    o.critical_bstrain = critical_bstrain;
    o.nbreak = nbreak;
    check(lpm_set_damage(ctx(), &o), "damage stage");
    g_damage_on = true;
    g_log_written = 0;
}

// Upload the damage state the damage functions read (current slots).
void put_damage()
{
    const int n = nparticle, nn = nneighbors;
    put("damage_broken", flat2(damage_broken, n, nn));
    put("damage_w", flat2(damage_w, n, nn));
    put("damage_D0", flat3(damage_D, n, nn, 0));
    dvec a(n);
    for (int i = 0; i < n; i++)
        a[i] = damage_nonlocal[i][0];
    put("damage_nonlocal0", a);
}

}  // namespace

extern "C" {

int lpm_legacy_set_solver(const void *p)
{
    if (!p)
        return LPM_ERR_ARG;
    std::memcpy(&g_opts, p, sizeof(g_opts));
    g_opts_set = true;
    return g_ctx ? lpm_set_solver(g_ctx, &g_opts) : LPM_OK;
}

int lpm_legacy_status(void) { return g_status; }

void lpm_legacy_reset(void)
{
    if (g_ctx)
        lpm_destroy(g_ctx);
    g_ctx = nullptr;
}

void lpm_legacy_traffic(long long *h2d, long long *d2h, int reset)
{
    if (h2d)
        *h2d = g_h2d;
    if (d2h)
        *d2h = g_d2h;
    if (reset)
        g_h2d = g_d2h = 0;
}

// src/stiffness.c:11-268: builds the GPU specimen from the host's particles,
// checks its bond lists against the host's, sets the material and returns
// Kn/Tv in the host globals.
void calcKnTv(void)
{
    if (dim != 3 || (lattice != 2 && lattice != 3)) {
        std::printf("LPM GPU drop-in: only the 3D simple cubic and FCC lattices are supported\n");
        std::exit(5);
    }
    lpm_legacy_reset();
    g_damage_on = false;
    check(lpm_create(&g_ctx, 0), "lpm_create");
    {
        // LPM_PRECOND=amg selects the multigrid preconditioner for an
        // unmodified reference driver
        lpm_solver_opts o;
        if (g_opts_set)
            o = g_opts;
        else
            lpm_default_solver_opts(&o);
        const char *pc = std::getenv("LPM_PRECOND");
        const bool amg = pc && std::strcmp(pc, "amg") == 0;
        if (amg)
            o.preconditioner = LPM_PRECOND_AMG;
        if (g_opts_set || amg)
            check(lpm_set_solver(g_ctx, &o), "lpm_set_solver");
    }
    const int n = nparticle, nn = nneighbors;
    dvec x0 = flat2(xyz_initial, n, 3);
    check(lpm_setup_particles(g_ctx, lattice, radius, n, x0.data()), "lpm_setup_particles");
    std::vector<int> nbr((size_t)n * 18);
    check(lpm_get(g_ctx, "neighbors", nbr.data(), nbr.size() * sizeof(int)), "neighbors");
    for (int i = 0; i < n; i++)
        for (int j = 0; j < nn; j++)
            if (nbr[(size_t)i * 18 + j] != neighbors[i][j]) {
                std::printf("LPM GPU drop-in: host bond list of particle %d differs from the GPU's\n", i);
                std::exit(5);
            }
    check(lpm_set_types(g_ctx, type), "lpm_set_types");
    std::vector<double> c11(n), c12(n), c44(n), sy(n, 0.0), H(n, J2_H);
    for (int i = 0; i < n; i++) {
        c11[i] = Ce[type[i]][0];
        c12[i] = Ce[type[i]][1];
        c44[i] = Ce[type[i]][2];
        if (sigmay)
            sy[i] = sigmay[i];
    }
    g_plmode_dev = (plmode == 0 || plmode == 1) ? plmode : 6;
    check(lpm_set_material(g_ctx, c11.data(), c12.data(), c44.data(), sy.data(), H.data(), J2_xi, g_plmode_dev),
          "lpm_set_material");
    if (g_plmode_dev == 1) {
        const double cp[8] = {cp_tau0[0], cp_taus[0], cp_h0, cp_p, cp_q, cp_eta, cp_maxloop, dtime};
        check(lpm_set_cp(g_ctx, cp), "lpm_set_cp");
    }
    check(lpm_init_state(g_ctx), "lpm_init_state");
    scatter2(Kn, get("Kn", (size_t)n * nn), n, nn);
    scatter2(Tv, get("Tv", (size_t)n * nn), n, nn);
}

// src/constitutive.c:1864-1917: the GPU computed Cab in calcKnTv; copy it out.
void computeStrain(void)
{
    const int n = nparticle, nn = nneighbors;
    put("dL", flat2(dL, n, nn));  // the host's dL, as the last force call wrote it back
    check(lpm_compute_strain(ctx()), "computeStrain");
    scatter2(strain_tensor, get("strain_tensor", 6 * (size_t)n), n, 6);
}

void computeCab(void)
{
    if (g_plmode_dev != 1 || nslipSys <= 0 || !cp_Cab)
        return;
    const int n = nparticle, w = nslipSys * nslipSys;
    scatter2(cp_Cab, get("cp_Cab", (size_t)n * w), n, w);
}

void calcStiffness2DFiniteDifference(int)
{
    std::printf("LPM GPU drop-in: 2D stiffness is not supported\n");
    std::exit(5);
}

// src/stiffness.c:384-516.  The reference's finite-difference sweep leaves
// the elastic-law bond forces of the current configuration in F and Pin
// (:390-418, computeBondForceElastic per particle).  Where a caller reads them
// before the next force evaluation - main's re-entry after broken bonds
// (src/lpmc_project.c:528-546 -> updateRR) - they are needed: with the damage
// stage on, the elastic forces are computed and written back here as well.
void calcStiffness3DFiniteDifference(int)
{
    const int n = nparticle, nn = nneighbors;
    put("xyz", flat2(xyz, n, 3));
    put("dLp0", flat3(dLp, n, nn, 0));
    check(lpm_assemble_stiffness(ctx()), "calcStiffness3DFiniteDifference");
    if (!std::getenv("LPM_LEGACY_NO_KEXPORT")) {
        long long nnz = 0;
        check(lpm_export_upper_csr(ctx(), K_global, IK, JK, &nnz), "K export");
        g_d2h += nnz * 12;
    }
    if (g_damage_on)
        device_force(6, false);
}

// src/stiffness.c:519-534
void updateRR()
{
    int ii = 0;
    for (int i = 0; i < nparticle; i++)
        for (int k = 0; k < dim; k++) {
            residual[dim * i + k] = dispBC_index[dim * i + k] * (Pex[dim * i + k] - Pin[3 * i + k]);
            if (dispBC_index[dim * i + k] == 0)
                reaction_force[ii++] = Pin[3 * i + k];
        }
}

// src/solver.c:188-270: GPU PCG (block-Jacobi, FP64 or mixed precision) on the
// stiffness of the last calcStiffness3DFiniteDifference with the BC mask.
void solverCG(void)
{
    const int n = nparticle;
    put_mask();
    std::vector<double> b(residual, residual + 3 * (size_t)n), x(3 * (size_t)n);
    g_h2d += (long long)(b.size() * sizeof(double));
    lpm_step_stats st;
    std::memset(&st, 0, sizeof(st));
    check(lpm_solve_rhs(ctx(), b.data(), x.data(), &st), "solverCG");
    g_d2h += (long long)(x.size() * sizeof(double));
    g_status = st.status;
    if (st.status)
        std::printf("The computation FAILED as the solver has returned the ERROR code %d\n", st.status);
    std::memcpy(disp, x.data(), x.size() * sizeof(double));
    for (int i = 0; i < n; i++)
        for (int j = 0; j < dim; j++)
            xyz[i][j] += disp[dim * i + j];
}

void solverPARDISO(void) { solverCG(); }

// src/constitutive.c:10-85
void switchStateV(int f)
{
    const int from = f == 0 ? 1 : (f == 1 ? 0 : 2), to = f == 1 ? 1 : 0;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < nparticle; i++) {
        for (int j = 0; j < nneighbors; j++) {
            dLp[i][j][to] = dLp[i][j][from];
            if (f != 2 && damage_D)
                damage_D[i][j][to] = damage_D[i][j][from];
        }
        for (int j = 0; j < 6; j++)
            J2_beta[i][j][to] = J2_beta[i][j][from];
        for (int j = 0; j < nslipSys; j++) {
            cp_gy[i][j][to] = cp_gy[i][j][from];
            cp_A_single[i][j][to] = cp_A_single[i][j][from];
        }
        J2_alpha[i][to] = J2_alpha[i][from];
        J2_beta_eq[i][to] = J2_beta_eq[i][from];
        if (f != 2) {
            if (damage_local)
                damage_local[i][to] = damage_local[i][from];
            if (damage_nonlocal)
                damage_nonlocal[i][to] = damage_nonlocal[i][from];
        }
        cp_A[i][to] = cp_A[i][from];
    }
}

// src/constitutive.c:88-146
void computeBondForceGeneral(int pl, int)
{
    if (pl != 0 && pl != 1 && pl != 4 && pl != 6) {
        std::printf("LPM GPU drop-in: constitutive mode %d is not on the GPU path\n", pl);
        std::exit(5);
    }
    if ((pl == 0 || pl == 1) && pl != g_plmode_dev) {
        std::printf("LPM GPU drop-in: plmode %d requested but the specimen was built for %d\n", pl, g_plmode_dev);
        std::exit(5);
    }
    device_force(pl, true);
    switchStateV(2);
}

void computeBondForceElastic(int) { device_force(6, false); }
void computeBondForceJ2mixedLinear3D(int) { device_force(0, false); }
void computeBondForceCPMiehe(int) { device_force(1, false); }
void computeBondForceIncrementalUpdating(int) { device_force(4, false); }

void computeBondForceJ2nonlinearIso(int)
{
    std::printf("LPM GPU drop-in: J2 with nonlinear hardening is not on the GPU path\n");
    std::exit(5);
}

void computeBondForceJ2energyReturnMap(int, int)
{
    std::printf("LPM GPU drop-in: energy-based J2 is not on the GPU path\n");
    std::exit(5);
}

// src/constitutive.c:149-164 on the GPU damage stage: the ductile nonlocal
// update for J2 (plmode 0, updateDuctileDamagePwiseNonlocal, :1757-1862), the
// brittle one for elastic bonds (plmode 6, updateBrittleDamage with the global
// nbreak, :1437-1527), nothing for crystal plasticity.  Uploads the damage
// state and the update's input (J2_dlambda, or dL), writes back the damage
// state and appends the step's broken bonds to dataName as the reference
// does ("TIMESTEP t", then "i j " per bond).
int updateDamageGeneral(const char *dataName, int tstep, int pl)
{
    if (pl == 5) {
        std::printf("LPM GPU drop-in: bond-wise local ductile damage (plmode 5) is not on the GPU path\n");
        std::exit(5);
    }
    if (pl != 0 && pl != 6)
        return 0;
    if (pl != g_plmode_dev) {
        std::printf("LPM GPU drop-in: damage for plmode %d requested but the specimen was built for %d\n", pl,
                    g_plmode_dev);
        std::exit(5);
    }
    ensure_damage();
    const int n = nparticle, nn = nneighbors;
    const size_t nb = (size_t)n * nn;
    put_damage();
    if (pl == 0)
        put("J2_dlambda", dvec(J2_dlambda, J2_dlambda + n));
    else
        put("dL", flat2(dL, n, nn));
    int broken = 0;
    check(lpm_damage_update(ctx(), &broken), "updateDamageGeneral");
    scatter2(damage_broken, get("damage_broken", nb), n, nn);
    scatter2(damage_w, get("damage_w", nb), n, nn);
    scatter3(damage_D, get("damage_D0", nb), n, nn, 0);
    if (pl == 0) {
        const dvec a = get("damage_nonlocal0", n);
        for (int i = 0; i < n; i++)
            damage_nonlocal[i][0] = a[i];
    }
    int total = 0;
    check(lpm_damage_log(ctx(), nullptr, 0, &total), "damage log");
    std::vector<int> pairs(2 * (size_t)total + 2);
    if (total > 0)
        check(lpm_damage_log(ctx(), pairs.data(), total, &total), "damage log");
    if (FILE *f = dataName ? std::fopen(dataName, "a+") : nullptr) {
        std::fprintf(f, "TIMESTEP %d\n", tstep);
        for (int k = g_log_written; k < total; k++)
            std::fprintf(f, "%d %d \n", pairs[2 * (size_t)k], pairs[2 * (size_t)k + 1]);
        std::fclose(f);
    }
    g_log_written = total;
    return broken;
}

int updateBrittleDamage(const char *dataName, int tstep, int)
{
    return updateDamageGeneral(dataName, tstep, 6);
}

int updateDuctileDamagePwiseNonlocal(const char *dataName, int tstep)
{
    return updateDamageGeneral(dataName, tstep, 0);
}

int updateDuctileDamageBwiseLocal(const char *, int)
{
    std::printf("LPM GPU drop-in: updateDuctileDamageBwiseLocal is not on the GPU path\n");
    std::exit(5);
}

int updateDuctileDamagePwiseLocal(const char *, int)
{
    std::printf("LPM GPU drop-in: updateDuctileDamagePwiseLocal is not on the GPU path\n");
    std::exit(5);
}

int updateDuctileDamageBwiseNonlocal(const char *, int)
{
    std::printf("LPM GPU drop-in: updateDuctileDamageBwiseNonlocal is not on the GPU path\n");
    std::exit(5);
}

// src/constitutive.c:1399-1434: bond forces scaled by damage_w, internal
// forces, intact-bond counts nb, damage_visual, and fix_index cleared for
// particles left without bonds.
void updateCrack(void)
{
    ensure_damage();
    const int n = nparticle, nn = nneighbors;
    const size_t nb3 = (size_t)n * nn;
    put_damage();
    put("F", flat2(F, n, nn));
    put("csx", flat2(csx, n, nn));
    put("csy", flat2(csy, n, nn));
    put("csz", flat2(csz, n, nn));
    check(lpm_damage_crack(ctx()), "updateCrack");
    scatter2(F, get("F", nb3), n, nn);
    const dvec pin = get("Pin", 3 * (size_t)n);
    std::memcpy(Pin, pin.data(), pin.size() * sizeof(double));
    const dvec vis = get("damage_visual", n);
    std::memcpy(damage_visual, vis.data(), vis.size() * sizeof(double));
    std::vector<int> cnt(n);
    check(lpm_get(ctx(), "nb_current", cnt.data(), cnt.size() * sizeof(int)), "nb_current");
    g_d2h += (long long)(cnt.size() * sizeof(int));
    for (int i = 0; i < n; i++) {
        nb[i] = cnt[i];
        if (nb[i] < 1)
            for (int k = 0; k < dim; k++)
                fix_index[dim * i + k] = 0;
    }
}

// src/boundary.c:12-45
void setDispBC(int nbd, struct dispBCPara *d)
{
    for (int i = 0; i < nparticle; i++)
        for (int k = 0; k < nbd; k++)
            if (type[i] == d[k].type) {
                if (d[k].flag == 'x') {
                    xyz[i][0] += d[k].step;
                    dispBC_index[dim * i] = 0;
                }
                if (d[k].flag == 'y') {
                    xyz[i][1] += d[k].step;
                    dispBC_index[dim * i + 1] = 0;
                }
                if (d[k].flag == 'z') {
                    xyz[i][2] += d[k].step;
                    dispBC_index[dim * i + 2] = 0;
                }
            }
    int c = 0;
    for (int k = 0; k < nparticle * dim; k++)
        c += (dispBC_index[k] != 1);
    std::free(reaction_force);
    reaction_force = (double *)std::calloc(c > 0 ? c : 1, sizeof(double));
}

// src/boundary.c:48-70
void setForceBC(int nbf, struct forceBCPara *f)
{
    for (int k = 0; k < nbf; k++) {
        int cnt = 0;
        for (int i = 0; i < nparticle; i++)
            cnt += (type[i] == f[k].type);
        for (int i = 0; i < nparticle; i++)
            if (type[i] == f[k].type) {
                Pex[dim * i] += f[k].step1 / cnt;
                Pex[dim * i + 1] += f[k].step2 / cnt;
                if (dim == 3)
                    Pex[dim * i + 2] += f[k].step3 / cnt;
            }
    }
}

void setDispBC_stiffnessUpdate2D(void)
{
    std::printf("LPM GPU drop-in: 2D stiffness is not supported\n");
    std::exit(5);
}

// src/boundary.c:159-281: the GPU solve eliminates the constrained DOFs by a
// mask (same iteration as CG on the row/column-eliminated matrix), so only the
// residual entries are cleared here; K_global keeps the exported tangent.
void setDispBC_stiffnessUpdate3D(void)
{
    for (int k = 0; k < nparticle * dim; k++)
        if (dispBC_index[k] == 0 || fix_index[k] == 0)
            residual[k] = 0.0;
}

}  // extern "C"
