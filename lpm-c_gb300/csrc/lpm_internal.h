// Internal declarations of the GB300 LPM library: the context, device
// layouts and the kernel launchers.  Not part of the public C ABI.
//
// Device layouts (n particles, NN = 18 bond slots per particle):
//   particle vectors      dvec4 / float4 per particle (x, y, z, 0)
//   bond arrays           slot-major [NN][n] so that thread i of a warp reads
//                         bond j of particle i coalesced
//   stiffness             block-CSR over particles, 3x3 blocks; the blocks of
//                         row i are padded to a multiple of 4 (npad_i) and
//                         stored component-major: value (r,c) of block b is at
//                         val[9*rowoff_i + (3r+c)*npad_i + b], so a lane can
//                         read 4 consecutive blocks' component with one
//                         128-bit load; cols[rowoff_i + b] (padding -> i, 0)
#pragma once
#include <cstdint>
#include <cstddef>
#include <string>
#include <memory>
#include <utility>
#include <vector>
#include <cuda_runtime.h>
#include "../../include/lpm_gpu.h"

#define LPM_NN 18     // bond slots per particle (SC and FCC: 2 shells)
#define LPM_NSLIP 24  // FCC signed {111}<110> systems
#define LPM_MAXCONN 64

// 32-byte aligned FP64 4-vector (x, y, z, 0) of one particle
typedef double4_32a dvec4;
__host__ __device__ inline dvec4 make_dvec4(double x, double y, double z, double w)
{
    return make_double4_32a(x, y, z, w);
}

namespace lpm {

extern thread_local std::string g_err;
int fail(int code, const std::string &msg);

#define LPM_CUDA(call)                                                                   \
    do {                                                                                 \
        cudaError_t e_ = (call);                                                         \
        if (e_ != cudaSuccess)                                                           \
            return ::lpm::fail(LPM_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

// Allocator whose resize() leaves trivial elements uninitialised, so that
// gigabyte-sized setup arrays are first written (and their pages first
// touched) by the parallel loops that fill them, not by a serial zero fill.
template <typename T>
struct NoInitAlloc : std::allocator<T> {
    template <typename U>
    struct rebind {
        typedef NoInitAlloc<U> other;
    };
    NoInitAlloc() = default;
    template <typename U>
    NoInitAlloc(const NoInitAlloc<U> &) noexcept
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
template <typename T>
using hvec = std::vector<T, NoInitAlloc<T>>;

// Host-side setup data (built once per specimen, see setup.cpp).
struct HostSetup {
    int lattice = 0, n = 0, nn1 = 0, nn2 = 0;
    double radius = 0, vol = 0, cut1 = 0, cut2 = 0;
    hvec<double> xyz;          // n x 3
    hvec<int> nbr;             // n x NN (row-major), -1 padded
    hvec<int> shell;           // n x NN
    hvec<int> nb;              // n
    hvec<int> rev;             // n x NN: slot of the reverse bond
    hvec<double> L0, cs0;      // n x NN, n x NN x 3
    hvec<double> oppv;         // n x NN: opposite-bond weight / particle volume
    hvec<int> conn;            // n x 61 sorted, -1 padded (searchAFEMNeighbor)
    hvec<int> nconn;           // n
    hvec<int> kp0, kp1;        // K_pointer[i][0], K_pointer[i][1]
    // block-CSR pattern
    hvec<long long> rowoff;    // n+1, in blocks (padded)
    hvec<int> npad;            // n
    hvec<int> cols;            // rowoff[n]
};

int build_lattice(HostSetup &h, int lattice, double radius, const double *box);
int build_particles(HostSetup &h, int lattice, double radius, int n, const double *xyz);
int build_neighbors(HostSetup &h);  // LPM_OK, or LPM_ERR_ARG when a particle has too many bonds
void build_afem(HostSetup &h);
void build_bond_tables(HostSetup &h);
void build_block_pattern(HostSetup &h);
void merge_setups(HostSetup &dst, const std::vector<HostSetup> &parts, std::vector<int> &offsets);
int build_batch(HostSetup &dst, int lattice, double radius, int nspec, const double *boxes,
                std::vector<int> &offsets);
void kntv_per_particle(int lattice, double radius, const double *c11, const double *c12,
                       const double *c44, int n, double *knt);
template <typename T>  // T = double (FP64 stiffness) or float (FP32 values, widened exactly)
void export_upper_csr_host(const HostSetup &h, const T *val, double *Kg, int *IK, int *JK);

// Device scalars used by the PCG (one 128-byte record).
// done: 0 running, 1 converged (recursive residual), 2 iteration cap,
// 3 non-finite, 4 reliable update requested (mixed precision)
struct CgScalars {
    double rz, rz_old, pq, rr, alpha, beta, bnorm2, tol2;
    double rr_max, upd_delta2;
    int it, done, maxit, upd_req;
};

struct AdjointState;
struct AsyncWriter;

// One level of the multigrid hierarchy on the device, all in FP32.  Level 0
// operates with the FP32 stiffness Kf and its block-Jacobi inverse Pinv_f on
// float4 vectors; the levels above hold 6 DOFs per block row (aggregate),
// vectors with 6 floats per row, and their own 6 x 6 block-CSR operator.
struct AmgDevLevel {
    int nb = 0, bs = 0;  // block rows, DOFs per block row
    int nnext = 0;       // block rows of the next level
    double omega = 1.0;  // smoother damping 4/3 / rho(D^-1 A)
    long long *a_ptr = nullptr;   // levels >= 1: operator, 6 x 6 blocks (FP16 values times a_scale)
    int *a_col = nullptr;
    unsigned short *a_val = nullptr;
    float a_scale = 1.0f;
    float *dinv = nullptr;        // levels >= 1: 6 x 6 diagonal-block inverses
    long long *p_ptr = nullptr;   // prolongation, bs x 6 blocks (FP16 values)
    int *p_col = nullptr;
    unsigned short *p_val = nullptr;
    long long *pt_ptr = nullptr;  // restriction, 6 x bs blocks (FP16 values)
    int *pt_col = nullptr;
    unsigned short *pt_val = nullptr;
    float *b = nullptr, *x = nullptr, *y = nullptr;  // levels >= 1: right-hand side, two iterates
};

struct AmgDev {
    std::vector<AmgDevLevel> lv;
    int nc = 0;                    // scalar size of the coarsest operator
    int cbs = 0;                   // its DOFs per block row (3 when level 0 is the coarsest)
    double *cinv = nullptr;        // its dense inverse, row-major (FP64)
    float *cb = nullptr, *cx = nullptr;
    std::vector<uint8_t> mask_h;   // DOF mask the hierarchy was built for
    int ref_iters = -1;            // PCG iterations of the first solve after the build
    bool stale = false;            // rebuild before the next solve
    int builds = 0;
    double build_ms = 0.0;         // host time of the last build (download, setup, upload)
};

// Per-specimen PCG state of a batch (device pointers, passed by value).
// done: 0 running, 1 recursive residual met the tolerance, 2 iteration cap,
// 3 non-finite, 5 specimen inactive (its Newton loop has converged),
// 6 true residual met the tolerance (mixed precision)
struct BatchCg {
    int n = 0, nspec = 0, nchunk = 0, nseg = 0, maxit = 0, maxrel = 0;
    double upd_delta2 = 0.0;
    const int *spec_of = nullptr;   // [n] specimen of each particle
    const int *off = nullptr;       // [nspec + 1] first particle of each specimen
    const int *seg_base = nullptr;  // [nchunk + 1] first reduction segment of each chunk
    double *rz = nullptr, *rz_old = nullptr, *rr = nullptr, *rr_max = nullptr, *tol2 = nullptr;
    double *alpha = nullptr, *beta = nullptr, *bscale = nullptr;
    int *it = nullptr, *done = nullptr, *upd = nullptr, *nrel = nullptr, *active = nullptr;
    double *partials = nullptr;     // [3][nseg]
    unsigned *counter = nullptr;
    int *all_done = nullptr;        // 1 once every specimen has stopped
    int *act_chunk = nullptr;       // [nchunk] chunks holding a running specimen (any order)
    int *n_act = nullptr;           // number of entries in act_chunk
};

// Host-side bookkeeping of a batch context.
struct BatchHost {
    int nspec = 0;
    std::vector<int> off;            // [nspec + 1]
    double *norms_d = nullptr;       // [2 nspec] squared |residual|, |reaction| per specimen
    double *norms_h = nullptr;       // pinned mirror
    double *bscale_h = nullptr;      // pinned [nspec]
    int *active_h = nullptr;         // pinned [nspec]
    int *it_h = nullptr, *done_h = nullptr, *nrel_h = nullptr;  // pinned [nspec]
    int *all_done_h = nullptr;       // pinned
    void *bc_d = nullptr;            // per-specimen displacement BC lists
    size_t bc_cap = 0;
    dvec4 *bs = nullptr;             // right-hand side scaled per specimen
    cudaGraphExec_t graph = nullptr;
    int graph_chunk = 0, graph_k32 = -1;
};

// Launch shapes of the solver kernels, set by lpm_autotune or lpm_set_tuning.
// spmv_variant: 0 = 16 lanes x 4 blocks per row chunk, 1 = 8 x 4, 2 = 32 x 2,
// 3 = 4 x 4 (lanes per block row x consecutive blocks per lane).
struct Tune {
    int smooth_variant = 0;  // multigrid level-0 smoother: 16 (0), 8 (1) or 4 (2) lanes per block row
    int diff_stream = 0;     // difference-form product: register-fed (0) or streamed (1..3)
    int smooth_stream = 0;   // multigrid level-0 smoother: register-fed (0) or streamed (1..3)
    int spmv_variant = 0;
    int spmv_per_sm = 8;  // SpMV thread blocks per SM (grid-stride over rows)
    int vec_per_sm = 8;   // PCG vector-kernel thread blocks per SM
    int sms = 0;          // SM count of the device
};
constexpr int TUNE_MAX_PER_SM = 16;
constexpr int STREAM_MAX_STAGES = 8;  // shared-memory stages of the streamed product

struct Ctx {
    int device = 0;
    Tune tune;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    int n = 0, nslip = 0, plmode = 0;
    HostSetup hs;
    lpm_solver_opts opts{};
    double xi = 0.0;
    double cp[8] = {0};
    bool ready = false;   // init_state done
    bool have_K = false;

    // ---- device: particles
    dvec4 *xyz = nullptr, *xyz0 = nullptr, *xyz_temp = nullptr;
    dvec4 *Pin = nullptr, *Pex = nullptr, *res = nullptr, *du = nullptr;
    uint8_t *mask = nullptr;  // bit d set = DOF d free (dispBC_index == 1)
    int *type = nullptr;
    double *G = nullptr, *sy = nullptr, *Hh = nullptr;
    double *stress = nullptr;  // [6][n]
    double *strain = nullptr;  // [6][n] (computeStrain)
    double *dlambda = nullptr;
    // ---- device: bonds [NN][n]
    int *nbr = nullptr;
    int8_t *shell = nullptr, *rev = nullptr;
    int8_t *nbv = nullptr;     // nb per particle (int8)
    int8_t *nconn_d = nullptr; // AFEM connectivity count per particle
    double *L0 = nullptr, *Kn = nullptr, *Tv = nullptr, *oppv = nullptr;
    double *dL = nullptr;      // elastic stretch after the last force evaluation
    double *csx = nullptr, *csy = nullptr, *csz = nullptr;  // unit vectors of the last evaluation
    double *F = nullptr, *F_prev = nullptr;
    double2 *S = nullptr, *T = nullptr;  // shell sums (dL_total, TdL_total)
    double *ddL = nullptr;     // predictor increments
    double2 *dS = nullptr, *dT = nullptr;
    // state variables in the reference's three slots (src/constitutive.c:10-85):
    // [0] current (read by a force evaluation), [1] last converged,
    // [2] freshly computed (written by a force evaluation)
    double *dLp[3] = {nullptr, nullptr, nullptr};     // [NN][n]
    double *alpha[3] = {nullptr, nullptr, nullptr};   // [n]
    double *beta[3] = {nullptr, nullptr, nullptr};    // [6][n]
    double *gy[3] = {nullptr, nullptr, nullptr};      // [nslip][n]
    double *As[3] = {nullptr, nullptr, nullptr};      // [nslip][n]
    double *A[3] = {nullptr, nullptr, nullptr};       // [n]
    double *Cab = nullptr;    // [nslip*nslip][n]
    double *sch = nullptr;    // [nslip][6]
    int *jact = nullptr;      // active set bitmask per particle
    // stiffness geometry (tangent assembly)
    double *U = nullptr, *W = nullptr;  // [6][n]: shell-sums of unit vectors (U) and Tv-weighted (W)
    // ---- device: block-CSR
    long long nblk = 0;       // padded block count
    long long nblk_real = 0;  // structural blocks
    long long *rowoff = nullptr;
    int *npad = nullptr;
    int *cols = nullptr;
    double *Kd = nullptr;     // FP64 values (9*nblk)
    float *Kf = nullptr;      // FP32 values (9*nblk)
    long long kd_cap = 0, kf_cap = 0;  // blocks Kd / Kf were allocated for
    long long k_version = 0;   // stiffness assemblies so far
    long long kf_version = -1; // the assembly Kf holds (FP32 assembly, or the copy of Kd for the smoother)
    double *Pinv_d = nullptr; // block-Jacobi inverse, [9][n]
    float *Pinv_f = nullptr;
    float *Pinv_rf = nullptr;  // multigrid smoother: the FP32 inverse per row, [n][9]
    // ---- solver vectors
    dvec4 *x_d = nullptr, *r_d = nullptr, *p_d = nullptr, *q_d = nullptr, *z_d = nullptr;
    float4 *x_f = nullptr, *r_f = nullptr, *p_f = nullptr, *q_f = nullptr, *z_f = nullptr;
    // the FP64 search direction split into two FP32 parts (p = hi + lo) for
    // the difference-form FP32 product, and the FP32 stiffness's block row
    // sums [n][9] it needs (for the assembly numbered krs_version)
    float4 *p_split = nullptr;  // [2 i] = hi, [2 i + 1] = lo: one 32-byte record per particle
    float *Krs = nullptr;
    long long krs_version = -1;
    // multigrid: FP16 copy of Kf scaled by 1 / kh_scale[0] (device) for the
    // level-0 smoother, of the assembly numbered kh_version
    unsigned short *Kh = nullptr;
    float *kh_scale = nullptr;
    // streamed difference-form product, per variant (tune.diff_stream - 1:
    // tiles of 16 rows with 1 or 2 CTAs per SM, tiles of 8 rows with 5):
    // stages per CTA (0: does not fit), bytes per stage, offsets in a stage
    int stream_stages[3] = {0, 0, 0};
    int stream_stage_bytes[3] = {0, 0, 0}, stream_cols_off[3] = {0, 0, 0}, stream_vals_off[3] = {0, 0, 0};
    // the same for the streamed level-0 smoother (FP16 values; variant 3:
    // tiles of 8 rows with 6 CTAs per SM)
    int smooth_stages[3] = {0, 0, 0};
    int smooth_stage_bytes[3] = {0, 0, 0}, smooth_cols_off[3] = {0, 0, 0}, smooth_vals_off[3] = {0, 0, 0};
    unsigned *kh_max = nullptr;
    long long kh_cap = 0, kh_version = -1;
    // mixed multigrid: Kc is the exact FP64 copy of Kf of assembly kc_version
    // (-1: none), read by the reliable updates' true residual; Kd keeps the
    // FP64 assembly, for the FP64-product fallback (amg_k64: a mixed solve
    // failed with FP32 products, and the context solves with FP64 ones since)
    double *Kc = nullptr;
    long long kc_cap = 0, kc_version = -1;
    bool amg_k64 = false;
    dvec4 *b_d = nullptr;
    CgScalars *sc = nullptr;     // device
    CgScalars *sc_host = nullptr; // pinned mirror
    double *partials = nullptr;  // reduction partials
    unsigned *counter = nullptr; // last-block counters
    double *norms = nullptr;     // device norms [4]
    double *norms_host = nullptr;
    int *status = nullptr, *status_host = nullptr;
    int red_blocks = 0;
    // timing of the SpMV launches
    cudaEvent_t ev_a = nullptr, ev_b = nullptr;
    double spmv_ms_sum = 0;
    long long spmv_count = 0;
    bool time_spmv = false;
    // CUDA graphs of PCG chunks
    cudaGraphExec_t graph_fp64 = nullptr, graph_fp32 = nullptr;
    int graph_chunk = 0, graph_mode = -1;
    bool graph_timed = false;
    bool time_this = false;  // the next SpMV launch carries the timing events
    bool vec64_fallback = false;  // mixed: FP32-vector PCG stagnated, use FP64 vectors
    double cg_rtol_now = 0.0;     // relative tolerance of the current solve (0: opts.cg_rtol)
    // pinned host staging of lpm_get / lpm_set / lpm_export_upper_csr copies,
    // allocated on first use and kept, so repeated exchanges of the same
    // arrays neither reallocate nor page-fault host memory
    void *stage_h = nullptr;
    size_t stage_cap = 0;
    bool trace = false;           // LPM_TRACE set: one stderr line per Newton iteration and solve
    long long trace_step = 0;     // load steps run by this context (trace numbering)
    // batched specimens (lpm_setup_batch); nspec == 0 for a single specimen
    int nspec = 0;
    BatchCg bcg;
    BatchHost bh;
    AdjointState *adj = nullptr;  // lpm_adjoint_forward / lpm_adjoint_backward
    AsyncWriter *writer = nullptr; // lpm_write_dump (output.cpp)
    int *pl_flag = nullptr;        // [n] set once a particle's return map has yielded (pl_flag)
    // damage stage (lpm_set_damage; src/constitutive.c:149-164, :1399-1862).
    // All pointers stay null while it is off, and the force and stiffness
    // kernels then take their undamaged path unchanged.
    struct Damage {
        int on = 0;
        lpm_damage_opts opts{};
        double *brk = nullptr, *dw = nullptr;            // damage_broken, damage_w [NN][n]
        double *D[2] = {nullptr, nullptr};               // damage_D slots 0, 1 [NN][n]
        double *dnl[2] = {nullptr, nullptr};             // damage_nonlocal slots 0, 1 [n]
        double *dvis = nullptr;                          // damage_visual [n]
        int8_t *nbc = nullptr;                           // intact bonds per particle (current nb)
        int8_t *opp = nullptr;                           // slot of the opposite bond, -1 none [NN][n]
        int *cstart = nullptr, *corder = nullptr;        // cell list of the initial positions
        int g[3] = {0, 0, 0};
        double lo[3] = {0, 0, 0}, cs = 0;                // grid origin and cell size (>= 3 L)
        int *list = nullptr;                             // bonds found by a damage kernel
        double *lval = nullptr;                          // their bond strains (brittle)
        int *count = nullptr, *count_h = nullptr;        // list length (device, pinned)
        std::vector<int> log;                            // broken (particle, partner) pairs, in order
    } dmg;
    // smoothed-aggregation multigrid preconditioner (opts.preconditioner ==
    // LPM_PRECOND_AMG): the hierarchy built on the host (amg_setup.cpp) and
    // kept on the device; null until the first solve that uses it
    AmgDev *amg = nullptr;
    // Anderson acceleration of the Newton loop (opts.newton_accel)
    struct Anderson {
        int m = 0;
        dvec4 *dU = nullptr, *dF = nullptr;      // m difference vectors each
        dvec4 *u_prev = nullptr, *f_prev = nullptr;
        double *dots = nullptr, *dots_h = nullptr;
    } acc;
    // initial guesses of the Newton solves from the load step's earlier
    // solutions (opts.recycle): pairs (du_j, b_j) with K du_j = b_j in slots
    // of a ring, the Galerkin matrix G_ij = du_i . b_j on the host
    struct Recycle {
        int m = 0, count = 0, head = 0;
        dvec4 *du = nullptr, *b = nullptr, *x0 = nullptr, *r0 = nullptr;
        double *dots = nullptr, *dots_h = nullptr;
        std::vector<double> G;
        long long k_version = -1;  // the assembly the stored pairs belong to
    } rec;
    ~Ctx();
};

// relative tolerance of the linear solve being run (inexact Newton sets it per solve)
inline double solve_rtol(const Ctx &c) { return c.cg_rtol_now > 0.0 ? c.cg_rtol_now : c.opts.cg_rtol; }

// ---- kernel launchers (stream-ordered, no synchronisation) ----
// force path (k_force.cu, FP64, no FMA contraction)
void launch_stretch(Ctx &c, const double *dLp, bool store_cs);
void launch_elastic_force(Ctx &c);
void launch_predictor(Ctx &c);
void launch_j2(Ctx &c);
void launch_cp(Ctx &c);
void launch_final_force(Ctx &c);
void launch_residual(Ctx &c);  // updateRR + norms into c.norms[0..1]
void launch_add_du(Ctx &c);
void launch_apply_disp_bc(Ctx &c, int nbd, const lpm_disp_bc *d);
void launch_apply_force_bc(Ctx &c, int nbf, const lpm_force_bc *f, const int *counts);
void launch_cab(Ctx &c);
void launch_strain(Ctx &c);  // k_strain.cu
// damage stage (k_damage.cu; updateCrack in k_force.cu)
void launch_dmg_nonlocal(Ctx &c);     // damage_nonlocal += weighted dlambda (slot 0)
void launch_dmg_ductile_break(Ctx &c);// bonds of particles past the threshold -> list
void launch_dmg_ductile_w(Ctx &c);    // D = max of the two particles, w = 1 - D
void launch_dmg_brittle_cand(Ctx &c); // bonds at the critical strain -> list, lval
void launch_dmg_break_list(Ctx &c, const int *bonds, int k);  // D = 1, w = 0, broken
void launch_dmg_oppv(Ctx &c);         // stress weights from the intact bonds
void launch_crack(Ctx &c);            // updateCrack + updateRR norms
// stiffness (k_stiff.cu)
void launch_tangent_geometry(Ctx &c);
void launch_assemble(Ctx &c, bool fp32);
void launch_block_jacobi(Ctx &c, bool fp32);
// multigrid preconditioner (k_amg.cu): PCG with z = V-cycle(r), FP64
// vectors; k32 selects the FP32 stiffness for the PCG product (mixed
// precision); the V-cycle smooths with the FP32 stiffness in both precisions
void launch_amg_init(Ctx &c, const dvec4 *b, double scale, double delta2, bool k32);  // x = 0, r, z, p, rz
void launch_amg_iter(Ctx &c, bool k32);
void launch_amg_reliable(Ctx &c, const dvec4 *rtrue);  // r = rtrue (masked), z, rz; p kept
void launch_amg_vcycle(Ctx &c, const dvec4 *r, dvec4 *z);  // z = V(r), FP32 inside (Kf, Pinv_f, x_f/q_f/r_f)
void launch_amg_smoother_pass(Ctx &c);  // one level-0 residual pass on scratch vectors (autotuner timing)
void launch_amg_stiffness32(Ctx &c);  // Kf = (float) Kd, for the smoother under FP64 precision
void init_stream_product(Ctx &c, int max_npad);  // layouts of the streamed product for the pattern
void init_stream_smoother(Ctx &c, int max_npad); // and of the streamed level-0 smoother
void launch_amg_stiffness16(Ctx &c);  // Kh = half(Kf / s), s = max |Kf| / 2^14 into kh_scale
void launch_stiffness64_of32(Ctx &c); // Kc = (double) Kf, exactly
int amg_prepare(Ctx &c);  // (re)build the hierarchy when missing, stale or the mask changed
void free_amg(Ctx &c);
// solver (k_solve.cu)
void launch_spmv_d(Ctx &c, const dvec4 *x, dvec4 *y, bool masked, bool dot_pq);
void launch_spmv_f(Ctx &c, const float4 *x, float4 *y, bool masked, bool dot_pq);
void launch_refine_residual(Ctx &c, const dvec4 *x, const dvec4 *b, dvec4 *r, double bscale);  // r = s b - K32 x (FP64)
void launch_refine_residual64(Ctx &c, const double *K, const dvec4 *x, const dvec4 *b, dvec4 *r);  // r = b - K x
void launch_spmv_fx(Ctx &c, const dvec4 *x, dvec4 *y, bool masked, bool dot);
void launch_cg_init_fx(Ctx &c, const dvec4 *b, double scale, double delta2);
void launch_cg_iter_fx(Ctx &c);
void launch_cg_p_d(Ctx &c, bool split = false);  // p = z + beta p (FP64 vectors); split: also p_split
void launch_row_sums(Ctx &c);  // Krs = block row sums of Kf (FP64 sums of the FP32 values)
// y = K32 p in difference form from p_split and Krs (masked); dot: p.y and alpha
void launch_spmv_diff(Ctx &c, dvec4 *y, bool dot);
void launch_reliable_d(Ctx &c, const dvec4 *rtrue);
void launch_cg_init_d(Ctx &c, const dvec4 *b, double scale);
void launch_cg_init_f(Ctx &c, const dvec4 *r64, double scale, double rtol, double delta2);
void launch_reliable(Ctx &c, const dvec4 *r64, double scale);
void launch_scale_copy(Ctx &c, dvec4 *y, const dvec4 *x, double s);
void launch_cg_iter_d(Ctx &c);
void launch_cg_iter_f(Ctx &c);
void launch_axpy_refine(Ctx &c, double scale);  // x_d += x_f / scale
void launch_norm2(Ctx &c, const dvec4 *v, int slot);
int red_grid(const Ctx &c);
int spmv_grid(const Ctx &c);
int spmv_variant_lanes(int variant);
int spmv_variant_blocks(int variant);
// host steps of the load-step loop (lpm_api.cu), shared with the adjoint
int sync(Ctx &c);
void switch_state(Ctx &c, int flag);
int solve_device(Ctx &c, const dvec4 *b, lpm_step_stats *st);  // K du = b (masked) -> c.du
int assemble(Ctx &c);
int prepare_preconditioner(Ctx &c);
int force_eval(Ctx &c, int plmode);

// adjoint (k_adjoint.cu): reverse mode of one J2 force evaluation
struct AdjBuffers {
    double *gx = nullptr, *gy = nullptr, *gz = nullptr;  // [NN][n] bond position cotangents
    double *knbar = nullptr, *tvbar = nullptr;           // [NN][n]
    double *Gbar = nullptr, *sybar = nullptr, *Hbar = nullptr;  // [n]
    double *E = nullptr, *nu = nullptr;                  // [n] material of the forward run
    double *gE = nullptr, *gnu = nullptr, *gsy = nullptr, *gH = nullptr;  // [n] accumulated
    double *gC = nullptr;                                // [3][n] accumulated C11, C12, C44 (may be null)
};
struct AdjointState;
void free_adjoint(Ctx &c);
void free_writer(Ctx &c);
// reverse of the last J2 force evaluation (state read from slot 1, forward
// results from F, dL, S, T): Pbar on the internal force, mu on the new state
void adj_vjp(Ctx &c, const dvec4 *Pbar, const double *mu_dLp, const double *mu_alpha, double *dLp_bar,
             double *alpha_bar, bool theta, AdjBuffers &w);
// x-bar from the bond cotangents (masked: prescribed DOFs zeroed); theta:
// add the material cotangents to w.gE .. w.gH
void adj_gather(Ctx &c, dvec4 *xbar, bool masked, bool theta, AdjBuffers &w);
void adj_dot(Ctx &c, const dvec4 *x, const dvec4 *y, double *out);          // out[0] = x.y
void adj_axpby(Ctx &c, double alpha, const dvec4 *x, double beta, dvec4 *y); // y = a x + b y
void adj_multidot(Ctx &c, int K, const dvec4 *const *A, const dvec4 *w, double *out);  // out[k] = A_k.w, K <= 16
void adj_reaction(Ctx &c, int type, int comp, double *out);                   // -sum Pin over a type
void adj_reaction_seed(Ctx &c, int type, int comp, double w, const dvec4 *lam, dvec4 *Pbar);

// batched specimens (k_batch.cu)
constexpr int BATCH_TPB = 256;  // particles per reduction chunk
void launch_spmv_batch(Ctx &c, const dvec4 *x, dvec4 *y, bool k32);  // k_solve.cu
void launch_refine_batch(Ctx &c, const dvec4 *x, const dvec4 *b, dvec4 *r);  // k_solve.cu
void launch_bnorm(Ctx &c);                       // per-specimen norms -> c.bh.norms_d
void launch_bcg_init(Ctx &c, const dvec4 *b);   // per-specimen PCG start (uses bcg.active, bcg.bscale)
void launch_bcg_compact(Ctx &c);                // act_chunk = chunks of running specimens
void launch_bcg_iter(Ctx &c, bool k32);         // one PCG iteration of every running specimen
void launch_bcg_reliable(Ctx &c);               // true residual + residual replacement (FP32 matrix)
void launch_bcg_finish(Ctx &c);                 // du = x / bscale
int launch_disp_bc_batch(Ctx &c, int nbd, const lpm_disp_bc *d);

}  // namespace lpm

struct lpm_ctx {
    lpm::Ctx c;
};
