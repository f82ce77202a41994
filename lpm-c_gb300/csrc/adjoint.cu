// Adjoint of the quasi-static load-step sequence: gradients of a function of
// the reaction-force curve with respect to per-particle E, nu, yield stress
// and hardening modulus, as a forward/backward pair (lpm_adjoint_forward,
// lpm_adjoint_backward).
//
// Step n solves Pin_free(u_n, q_{n-1}; theta) = Pex with q_n = Q(u_n, q_{n-1};
// theta) (the J2 return map) and reports R_n = -sum_{type t} Pin_c
// (writeReaction, src/data_handler.c:309-335).  For L = sum_n l_n(R_n) the
// backward sweep runs n = N .. 1 with the state cotangent mu_n (mu_N = 0):
//   K_t^T lam_n = -[d(l_n R_n)/du + (dQ/du)^T mu_n]_free
//   mu_{n-1} = [dPin/dq]^T (lam_n + l'_n e_R) + (dQ/dq)^T mu_n
//   dL/dtheta += [dPin/dtheta]^T (lam_n + l'_n e_R) + (dQ/dtheta)^T mu_n
// where every product is one reverse pass of the force evaluation (k_adjoint.cu)
// and K_t^T (the consistent tangent, which the load steps never assemble) is
// only applied, never formed.  K_t^T lam = b is solved by restarted flexible
// GMRES preconditioned with the elastic tangent: each preconditioner
// application is one block-Jacobi PCG solve with the load steps' solver.
//
// States are checkpointed every opts.checkpoint_every steps in the forward
// run; the backward run restores each checkpoint, recomputes its segment
// (the load steps are deterministic, so the recomputation is bit-identical)
// and keeps the segment's states on the device.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>
#include "lpm_internal.h"

namespace lpm {

// one stored configuration: what a load step reads before writing
struct Snapshot {
    dvec4 *xyz = nullptr;
    double *F = nullptr, *dLp = nullptr, *alpha = nullptr, *beta = nullptr;
};

struct AdjointState {
    int nsteps = 0, nbd = 0, rtype = 0, rcomp = 2;
    lpm_adjoint_opts opts{};
    std::vector<lpm_disp_bc> bcs;
    std::vector<double> R;
    std::vector<Snapshot> ckpt;  // state after steps 0, every, 2 every, ...
    Snapshot final_state;
    std::vector<Snapshot> seg;   // states of the segment being swept
    AdjBuffers w;
    dvec4 *V = nullptr, *Z = nullptr;  // GMRES bases, (m + 1) and m vectors
    dvec4 *lam = nullptr, *rhs = nullptr, *Pbar = nullptr, *tmp = nullptr;
    double *mu_dLp[2] = {nullptr, nullptr}, *mu_alpha[2] = {nullptr, nullptr};
    double *dots = nullptr, *dots_h = nullptr;
    bool forward_done = false;
    lpm_adjoint_stats st{};
};

namespace {

template <typename T>
int aalloc(T *&p, size_t count)
{
    if (p)
        cudaFree(p);
    p = nullptr;
    cudaError_t e = cudaMalloc((void **)&p, std::max<size_t>(count, 1) * sizeof(T));
    if (e != cudaSuccess) {
        p = nullptr;
        return fail(LPM_ERR_NOMEM, std::string("adjoint: cudaMalloc: ") + cudaGetErrorString(e));
    }
    cudaMemset(p, 0, std::max<size_t>(count, 1) * sizeof(T));
    return LPM_OK;
}

template <typename T>
void afree(T *&p)
{
    if (p)
        cudaFree(p);
    p = nullptr;
}

int snap_alloc(Ctx &c, Snapshot &s)
{
    const size_t n = c.n, nb = n * LPM_NN;
    int rc;
    if ((rc = aalloc(s.xyz, n)) || (rc = aalloc(s.F, nb)) || (rc = aalloc(s.dLp, nb)) || (rc = aalloc(s.alpha, n)) ||
        (rc = aalloc(s.beta, 6 * n)))
        return rc;
    return LPM_OK;
}

void snap_free(Snapshot &s)
{
    afree(s.xyz);
    afree(s.F);
    afree(s.dLp);
    afree(s.alpha);
    afree(s.beta);
}

// state at a step boundary: the three state slots are equal there
int snap_take(Ctx &c, Snapshot &s)
{
    const size_t n = c.n, nb = n * LPM_NN;
    LPM_CUDA(cudaMemcpyAsync(s.xyz, c.xyz, n * sizeof(dvec4), cudaMemcpyDeviceToDevice, c.stream));
    LPM_CUDA(cudaMemcpyAsync(s.F, c.F, nb * sizeof(double), cudaMemcpyDeviceToDevice, c.stream));
    LPM_CUDA(cudaMemcpyAsync(s.dLp, c.dLp[1], nb * sizeof(double), cudaMemcpyDeviceToDevice, c.stream));
    LPM_CUDA(cudaMemcpyAsync(s.alpha, c.alpha[1], n * sizeof(double), cudaMemcpyDeviceToDevice, c.stream));
    LPM_CUDA(cudaMemcpyAsync(s.beta, c.beta[1], 6 * n * sizeof(double), cudaMemcpyDeviceToDevice, c.stream));
    return LPM_OK;
}

// the state of a snapshot into every slot (and xyz, F unless state_only)
int snap_put(Ctx &c, const Snapshot &s, bool state_only)
{
    const size_t n = c.n, nb = n * LPM_NN;
    if (!state_only) {
        LPM_CUDA(cudaMemcpyAsync(c.xyz, s.xyz, n * sizeof(dvec4), cudaMemcpyDeviceToDevice, c.stream));
        LPM_CUDA(cudaMemcpyAsync(c.F, s.F, nb * sizeof(double), cudaMemcpyDeviceToDevice, c.stream));
    }
    for (int k = 0; k < 3; k++) {
        LPM_CUDA(cudaMemcpyAsync(c.dLp[k], s.dLp, nb * sizeof(double), cudaMemcpyDeviceToDevice, c.stream));
        LPM_CUDA(cudaMemcpyAsync(c.alpha[k], s.alpha, n * sizeof(double), cudaMemcpyDeviceToDevice, c.stream));
        LPM_CUDA(cudaMemcpyAsync(c.beta[k], s.beta, 6 * n * sizeof(double), cudaMemcpyDeviceToDevice, c.stream));
    }
    return LPM_OK;
}

int alloc_work(Ctx &c, AdjointState &A)
{
    const size_t n = c.n, nb = n * LPM_NN;
    AdjBuffers &w = A.w;
    const int m = A.opts.gmres_restart;
    int rc;
    if ((rc = aalloc(w.gx, nb)) || (rc = aalloc(w.gy, nb)) || (rc = aalloc(w.gz, nb)) || (rc = aalloc(w.knbar, nb)) ||
        (rc = aalloc(w.tvbar, nb)) || (rc = aalloc(w.Gbar, n)) || (rc = aalloc(w.sybar, n)) ||
        (rc = aalloc(w.Hbar, n)) || (rc = aalloc(w.E, n)) || (rc = aalloc(w.nu, n)) || (rc = aalloc(w.gE, n)) ||
        (rc = aalloc(w.gnu, n)) || (rc = aalloc(w.gsy, n)) || (rc = aalloc(w.gH, n)) ||
        (rc = aalloc(A.V, (size_t)(m + 1) * n)) || (rc = aalloc(A.Z, (size_t)m * n)) || (rc = aalloc(A.lam, n)) ||
        (rc = aalloc(A.rhs, n)) || (rc = aalloc(A.Pbar, n)) || (rc = aalloc(A.tmp, n)) ||
        (rc = aalloc(A.mu_dLp[0], nb)) || (rc = aalloc(A.mu_dLp[1], nb)) || (rc = aalloc(A.mu_alpha[0], n)) ||
        (rc = aalloc(A.mu_alpha[1], n)) || (rc = aalloc(A.dots, 4)))
        return rc;
    if (!A.dots_h)
        LPM_CUDA(cudaMallocHost((void **)&A.dots_h, 4 * sizeof(double)));
    return LPM_OK;
}

double dot_now(Ctx &c, AdjointState &A, const dvec4 *x, const dvec4 *y, int &rc)
{
    adj_dot(c, x, y, A.dots);
    cudaMemcpyAsync(A.dots_h, A.dots, sizeof(double), cudaMemcpyDeviceToHost, c.stream);
    rc = sync(c);
    return A.dots_h[0];
}

// y = K_t^T x on the free DOFs (x zero on the prescribed ones)
void apply_KtT(Ctx &c, AdjointState &A, const dvec4 *x, dvec4 *y)
{
    adj_vjp(c, x, nullptr, nullptr, nullptr, nullptr, false, A.w);
    adj_gather(c, y, true, false, A.w);
}

// z = K_e^{-1} x (masked block-Jacobi PCG with the load steps' solver)
int apply_prec(Ctx &c, AdjointState &A, const dvec4 *x, dvec4 *z)
{
    lpm_step_stats st;
    std::memset(&st, 0, sizeof(st));
    int rc = solve_device(c, x, &st);
    if (rc)
        return rc;
    A.st.cg_iters += st.cg_iters;
    LPM_CUDA(cudaMemcpyAsync(z, c.du, c.n * sizeof(dvec4), cudaMemcpyDeviceToDevice, c.stream));
    return LPM_OK;
}

// Restarted flexible GMRES for K_t^T lam = rhs (right preconditioning).
int gmres(Ctx &c, AdjointState &A)
{
    const int n = c.n, m = A.opts.gmres_restart;
    int rc = 0;
    auto Vk = [&](int k) { return A.V + (size_t)k * n; };
    auto Zk = [&](int k) { return A.Z + (size_t)k * n; };
    LPM_CUDA(cudaMemsetAsync(A.lam, 0, n * sizeof(dvec4), c.stream));
    const double bnorm = std::sqrt(dot_now(c, A, A.rhs, A.rhs, rc));
    if (rc)
        return rc;
    if (!(bnorm > 0.0))
        return LPM_OK;
    const double tol = A.opts.gmres_rtol * bnorm;
    // r = rhs - A lam (lam = 0 at the start)
    LPM_CUDA(cudaMemcpyAsync(A.tmp, A.rhs, n * sizeof(dvec4), cudaMemcpyDeviceToDevice, c.stream));
    double beta = bnorm;
    int total = 0;
    std::vector<double> H((size_t)(m + 1) * m), cs(m), sn(m), g(m + 1), y(m);
    while (total < A.opts.gmres_maxiter) {
        adj_axpby(c, 1.0 / beta, A.tmp, 0.0, Vk(0));
        std::fill(g.begin(), g.end(), 0.0);
        g[0] = beta;
        int k = 0;
        for (; k < m && total < A.opts.gmres_maxiter; k++, total++) {
            if ((rc = apply_prec(c, A, Vk(k), Zk(k))))
                return rc;
            apply_KtT(c, A, Zk(k), Vk(k + 1));
            for (int i = 0; i <= k; i++) {  // modified Gram-Schmidt
                const double h = dot_now(c, A, Vk(k + 1), Vk(i), rc);
                if (rc)
                    return rc;
                H[(size_t)i * m + k] = h;
                adj_axpby(c, -h, Vk(i), 1.0, Vk(k + 1));
            }
            const double hn = std::sqrt(dot_now(c, A, Vk(k + 1), Vk(k + 1), rc));
            if (rc)
                return rc;
            H[(size_t)(k + 1) * m + k] = hn;
            if (hn > 0.0)
                adj_axpby(c, 1.0 / hn, Vk(k + 1), 0.0, Vk(k + 1));
            for (int i = 0; i < k; i++) {  // previous Givens rotations
                const double a0 = H[(size_t)i * m + k], a1 = H[(size_t)(i + 1) * m + k];
                H[(size_t)i * m + k] = cs[i] * a0 + sn[i] * a1;
                H[(size_t)(i + 1) * m + k] = -sn[i] * a0 + cs[i] * a1;
            }
            const double a0 = H[(size_t)k * m + k], a1 = H[(size_t)(k + 1) * m + k];
            const double r = std::hypot(a0, a1);
            cs[k] = r > 0.0 ? a0 / r : 1.0;
            sn[k] = r > 0.0 ? a1 / r : 0.0;
            H[(size_t)k * m + k] = r;
            H[(size_t)(k + 1) * m + k] = 0.0;
            g[k + 1] = -sn[k] * g[k];
            g[k] = cs[k] * g[k];
            if (std::fabs(g[k + 1]) <= tol || hn == 0.0) {
                k++;
                total++;
                break;
            }
        }
        // lam += Z y with H y = g (upper triangular k x k)
        for (int i = k - 1; i >= 0; i--) {
            double s = g[i];
            for (int j = i + 1; j < k; j++)
                s -= H[(size_t)i * m + j] * y[j];
            y[i] = H[(size_t)i * m + i] != 0.0 ? s / H[(size_t)i * m + i] : 0.0;
        }
        for (int i = 0; i < k; i++)
            adj_axpby(c, y[i], Zk(i), 1.0, A.lam);
        // true residual
        apply_KtT(c, A, A.lam, A.tmp);
        adj_axpby(c, 1.0, A.rhs, -1.0, A.tmp);
        beta = std::sqrt(dot_now(c, A, A.tmp, A.tmp, rc));
        if (rc)
            return rc;
        if (beta <= tol || !std::isfinite(beta))
            break;
    }
    A.st.gmres_iters += total;
    if (!(beta <= tol))
        A.st.status |= LPM_STATUS_CG_MAXIT;
    return LPM_OK;
}

}  // namespace

void free_adjoint(Ctx &c)
{
    AdjointState *A = c.adj;
    if (!A)
        return;
    for (Snapshot &s : A->ckpt)
        snap_free(s);
    for (Snapshot &s : A->seg)
        snap_free(s);
    snap_free(A->final_state);
    AdjBuffers &w = A->w;
    double **ptrs[] = {&w.gx, &w.gy, &w.gz, &w.knbar, &w.tvbar, &w.Gbar, &w.sybar, &w.Hbar, &w.E, &w.nu,
                       &w.gE, &w.gnu, &w.gsy, &w.gH, &w.gC, &A->mu_dLp[0], &A->mu_dLp[1], &A->mu_alpha[0],
                       &A->mu_alpha[1], &A->dots};
    for (double **p : ptrs)
        afree(*p);
    dvec4 **vp[] = {&A->V, &A->Z, &A->lam, &A->rhs, &A->Pbar, &A->tmp};
    for (dvec4 **p : vp)
        afree(*p);
    if (A->dots_h)
        cudaFreeHost(A->dots_h);
    delete A;
    c.adj = nullptr;
}

}  // namespace lpm

using namespace lpm;

extern "C" {

void lpm_default_adjoint_opts(lpm_adjoint_opts *o)
{
    if (!o)
        return;
    o->checkpoint_every = 10;
    o->gmres_restart = 30;
    o->gmres_maxiter = 600;
    o->gmres_rtol = 1e-10;
}

int lpm_adjoint_forward(lpm_ctx *ctx, const double *E, const double *nu, const double *sigmay, const double *H,
                        int nsteps, int nbd, const lpm_disp_bc *bcs, int rtype, int rcomp,
                        const lpm_adjoint_opts *opts, double *R)
{
    if (!ctx || !E || !nu || !sigmay || !H || nsteps <= 0 || nbd < 0 || (nbd > 0 && !bcs) || rcomp < 0 ||
        rcomp > 2)
        return fail(LPM_ERR_ARG, "lpm_adjoint_forward: bad argument");
    Ctx &c = ctx->c;
    if (c.n <= 0 || c.nspec > 0)
        return fail(LPM_ERR_ARG, "lpm_adjoint_forward: set up one specimen (and its types) first");
    if (c.dmg.on)
        return fail(LPM_ERR_ARG, "lpm_adjoint_forward: the adjoint does not model the damage stage "
                                 "(switch it off with lpm_set_damage)");
    auto t0 = std::chrono::steady_clock::now();
    const int n = c.n;
    std::vector<double> c11(n), c12(n), c44(n);
    for (int i = 0; i < n; i++) {  // src/lpmc_project.c:188-190
        const double e = E[i], v = nu[i];
        c11[i] = e * (1.0 - v) / (1.0 + v) / (1.0 - 2.0 * v);
        c12[i] = e * v / (1.0 + v) / (1.0 - 2.0 * v);
        c44[i] = e / 2.0 / (1.0 + v);
    }
    int rc = lpm_set_material(ctx, c11.data(), c12.data(), c44.data(), sigmay, H, 0.0, LPM_PL_J2);
    if (rc)
        return rc;
    if ((rc = lpm_init_state(ctx)))
        return rc;
    free_adjoint(c);
    c.adj = new AdjointState();
    AdjointState &A = *c.adj;
    lpm_default_adjoint_opts(&A.opts);
    if (opts)
        A.opts = *opts;
    A.opts.checkpoint_every = std::max(1, A.opts.checkpoint_every);
    A.opts.gmres_restart = std::max(1, std::min(A.opts.gmres_restart, 200));
    A.nsteps = nsteps;
    A.nbd = nbd;
    A.rtype = rtype;
    A.rcomp = rcomp;
    A.bcs.assign(bcs, bcs + (size_t)nsteps * nbd);
    A.R.assign(nsteps, 0.0);
    if ((rc = alloc_work(c, A)))
        return rc;
    LPM_CUDA(cudaMemcpy(A.w.E, E, n * sizeof(double), cudaMemcpyHostToDevice));
    LPM_CUDA(cudaMemcpy(A.w.nu, nu, n * sizeof(double), cudaMemcpyHostToDevice));
    const int every = A.opts.checkpoint_every;
    const int nck = (nsteps + every - 1) / every;
    A.ckpt.resize(nck);
    for (Snapshot &s : A.ckpt)
        if ((rc = snap_alloc(c, s)))
            return rc;
    if ((rc = snap_alloc(c, A.final_state)))
        return rc;
    A.seg.resize(every + 1);
    for (Snapshot &s : A.seg)
        if ((rc = snap_alloc(c, s)))
            return rc;
    if ((rc = snap_take(c, A.ckpt[0])))
        return rc;
    A.st = lpm_adjoint_stats();
    for (int k = 0; k < nsteps; k++) {
        lpm_step_stats st;
        if ((rc = lpm_load_step(ctx, nbd, A.bcs.data() + (size_t)k * nbd, 0, nullptr, &st)))
            return rc;
        if (st.newton_iters < 1)
            return fail(LPM_ERR_ARG, "lpm_adjoint_forward: load step " + std::to_string(k + 1) +
                                         " needed no Newton iteration; the adjoint needs one return map per step");
        A.st.status |= st.status;
        A.st.cg_iters += st.cg_iters;
        adj_reaction(c, rtype, rcomp, A.dots);
        LPM_CUDA(cudaMemcpyAsync(A.dots_h, A.dots, sizeof(double), cudaMemcpyDeviceToHost, c.stream));
        if ((rc = sync(c)))
            return rc;
        A.R[k] = A.dots_h[0];
        if ((k + 1) % every == 0 && (k + 1) < nsteps)
            if ((rc = snap_take(c, A.ckpt[(k + 1) / every])))
                return rc;
    }
    if ((rc = snap_take(c, A.final_state)) || (rc = sync(c)))
        return rc;
    A.st.steps = nsteps;
    A.st.checkpoints = nck;
    A.forward_done = true;
    A.st.ms_forward = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    if (R)
        std::memcpy(R, A.R.data(), nsteps * sizeof(double));
    return LPM_OK;
}

int lpm_adjoint_backward(lpm_ctx *ctx, const double *dLdR, double *gE, double *gnu, double *gsy, double *gH,
                         lpm_adjoint_stats *stats)
{
    if (!ctx || !dLdR)
        return fail(LPM_ERR_ARG, "lpm_adjoint_backward: bad argument");
    Ctx &c = ctx->c;
    if (!c.adj || !c.adj->forward_done)
        return fail(LPM_ERR_ARG, "lpm_adjoint_backward: run lpm_adjoint_forward first");
    AdjointState &A = *c.adj;
    auto t0 = std::chrono::steady_clock::now();
    const size_t n = c.n, nb = n * LPM_NN;
    const int every = A.opts.checkpoint_every, N = A.nsteps;
    A.st.gmres_iters = 0;
    A.st.recomputed_steps = 0;
    const int cg_fwd = A.st.cg_iters;
    A.st.cg_iters = 0;
    int rc;
    AdjBuffers &w = A.w;
    double *acc[] = {w.gE, w.gnu, w.gsy, w.gH};
    for (double *p : acc)
        LPM_CUDA(cudaMemsetAsync(p, 0, n * sizeof(double), c.stream));
    int cur = 0;  // mu ping-pong: mu_n in [cur]
    LPM_CUDA(cudaMemsetAsync(A.mu_dLp[cur], 0, nb * sizeof(double), c.stream));
    LPM_CUDA(cudaMemsetAsync(A.mu_alpha[cur], 0, n * sizeof(double), c.stream));
    const int nseg = (N + every - 1) / every;
    for (int sg = nseg - 1; sg >= 0; sg--) {
        const int start = sg * every, end = std::min(N, start + every);
        // recompute the segment from its checkpoint
        if ((rc = snap_put(c, A.ckpt[sg], false)))
            return rc;
        if ((rc = snap_take(c, A.seg[0])))
            return rc;
        for (int k = start; k < end; k++) {
            lpm_step_stats st;
            if ((rc = lpm_load_step(ctx, A.nbd, A.bcs.data() + (size_t)k * A.nbd, 0, nullptr, &st)))
                return rc;
            A.st.recomputed_steps++;
            if ((rc = snap_take(c, A.seg[k - start + 1])))
                return rc;
        }
        for (int k = end - 1; k >= start; k--) {
            // step k+1: u = seg[k-start+1].xyz, previous state = seg[k-start]
            const Snapshot &un = A.seg[k - start + 1], &qp = A.seg[k - start];
            LPM_CUDA(cudaMemcpyAsync(c.xyz, un.xyz, n * sizeof(dvec4), cudaMemcpyDeviceToDevice, c.stream));
            if ((rc = snap_put(c, qp, true)))
                return rc;
            // elastic tangent at u_n for the preconditioner, then the force
            // evaluation whose reverse is taken (it leaves q_{n-1} in slot 1)
            if ((rc = assemble(c)) || (rc = prepare_preconditioner(c)) || (rc = force_eval(c, LPM_PL_J2)))
                return rc;
            const double wn = -dLdR[k];  // R = -sum Pin: Pin-bar = -dL/dR on the reaction DOFs
            // rhs = -[VJP_u(seed, mu_n)]_free
            adj_reaction_seed(c, A.rtype, A.rcomp, wn, nullptr, A.Pbar);
            adj_vjp(c, A.Pbar, A.mu_dLp[cur], A.mu_alpha[cur], nullptr, nullptr, false, w);
            adj_gather(c, A.rhs, true, false, w);
            adj_axpby(c, 0.0, A.rhs, -1.0, A.rhs);
            if ((rc = gmres(c, A)))
                return rc;
            // full reverse pass with Pin-bar = lam + seed
            adj_reaction_seed(c, A.rtype, A.rcomp, wn, A.lam, A.Pbar);
            adj_vjp(c, A.Pbar, A.mu_dLp[cur], A.mu_alpha[cur], A.mu_dLp[1 - cur], A.mu_alpha[1 - cur], true, w);
            adj_gather(c, A.tmp, true, true, w);
            cur = 1 - cur;
        }
    }
    // leave the context at the end of the forward run
    if ((rc = snap_put(c, A.final_state, false)) || (rc = sync(c)))
        return rc;
    double *outs[] = {gE, gnu, gsy, gH};
    for (int k = 0; k < 4; k++)
        if (outs[k])
            LPM_CUDA(cudaMemcpy(outs[k], acc[k], n * sizeof(double), cudaMemcpyDeviceToHost));
    A.st.ms_backward = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    const int cg_bwd = A.st.cg_iters;
    A.st.cg_iters = cg_fwd;
    A.st.cg_iters_backward = cg_bwd;
    if (stats)
        *stats = A.st;
    return LPM_OK;
}

int lpm_force_vjp(lpm_ctx *ctx, const double *Pbar, const double *mu_dLp, const double *mu_alpha, double *xbar,
                  double *dLp_bar, double *alpha_bar, double *theta_bar)
{
    if (!ctx || !Pbar || !ctx->c.ready)
        return fail(LPM_ERR_ARG, "lpm_force_vjp: bad argument or uninitialised context");
    Ctx &c = ctx->c;
    const size_t n = c.n, nb = n * LPM_NN;
    AdjBuffers w;
    dvec4 *P = nullptr, *xb = nullptr;
    double *mud = nullptr, *mua = nullptr, *db = nullptr, *ab = nullptr;
    int rc = 0;
    auto cleanup = [&]() {
        double **ptrs[] = {&w.gx, &w.gy, &w.gz, &w.knbar, &w.tvbar, &w.Gbar, &w.sybar, &w.Hbar, &w.gsy,
                           &w.gH, &w.gC, &mud, &mua, &db, &ab};
        for (double **p : ptrs)
            afree(*p);
        afree(P);
        afree(xb);
    };
    if ((rc = aalloc(w.gx, nb)) || (rc = aalloc(w.gy, nb)) || (rc = aalloc(w.gz, nb)) || (rc = aalloc(w.knbar, nb)) ||
        (rc = aalloc(w.tvbar, nb)) || (rc = aalloc(w.Gbar, n)) || (rc = aalloc(w.sybar, n)) ||
        (rc = aalloc(w.Hbar, n)) || (rc = aalloc(w.gsy, n)) || (rc = aalloc(w.gH, n)) || (rc = aalloc(w.gC, 3 * n)) ||
        (rc = aalloc(mud, nb)) || (rc = aalloc(mua, n)) || (rc = aalloc(db, nb)) || (rc = aalloc(ab, n)) ||
        (rc = aalloc(P, n)) || (rc = aalloc(xb, n))) {
        cleanup();
        return rc;
    }
    std::vector<dvec4> hp(n);
    for (size_t i = 0; i < n; i++)
        hp[i] = make_dvec4(Pbar[3 * i], Pbar[3 * i + 1], Pbar[3 * i + 2], 0.0);
    std::vector<double> t(nb);
    cudaMemcpy(P, hp.data(), n * sizeof(dvec4), cudaMemcpyHostToDevice);
    if (mu_dLp) {  // [i][j] -> [j][i]
        for (size_t i = 0; i < n; i++)
            for (int j = 0; j < LPM_NN; j++)
                t[(size_t)j * n + i] = mu_dLp[i * LPM_NN + j];
        cudaMemcpy(mud, t.data(), nb * sizeof(double), cudaMemcpyHostToDevice);
    }
    if (mu_alpha)
        cudaMemcpy(mua, mu_alpha, n * sizeof(double), cudaMemcpyHostToDevice);
    adj_vjp(c, P, mu_dLp ? mud : nullptr, mu_alpha ? mua : nullptr, db, ab, true, w);
    adj_gather(c, xb, false, true, w);
    rc = sync(c);
    if (!rc) {
        cudaMemcpy(hp.data(), xb, n * sizeof(dvec4), cudaMemcpyDeviceToHost);
        if (xbar)
            for (size_t i = 0; i < n; i++) {
                xbar[3 * i] = hp[i].x;
                xbar[3 * i + 1] = hp[i].y;
                xbar[3 * i + 2] = hp[i].z;
            }
        if (dLp_bar) {
            cudaMemcpy(t.data(), db, nb * sizeof(double), cudaMemcpyDeviceToHost);
            for (size_t i = 0; i < n; i++)
                for (int j = 0; j < LPM_NN; j++)
                    dLp_bar[i * LPM_NN + j] = t[(size_t)j * n + i];
        }
        if (alpha_bar)
            cudaMemcpy(alpha_bar, ab, n * sizeof(double), cudaMemcpyDeviceToHost);
        if (theta_bar) {  // C11, C12, C44, sigmay, H per particle, [5][n]
            cudaMemcpy(theta_bar, w.gC, 3 * n * sizeof(double), cudaMemcpyDeviceToHost);
            cudaMemcpy(theta_bar + 3 * n, w.gsy, n * sizeof(double), cudaMemcpyDeviceToHost);
            cudaMemcpy(theta_bar + 4 * n, w.gH, n * sizeof(double), cudaMemcpyDeviceToHost);
        }
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess)
            rc = fail(LPM_ERR_CUDA, std::string("lpm_force_vjp: ") + cudaGetErrorString(e));
    }
    cleanup();
    return rc;
}

}  // extern "C"
