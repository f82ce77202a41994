// C ABI of the library (include/lpm_gpu.h): context lifetime, specimen setup,
// data exchange, and the host side of the load-step loop
// (src/lpmc_project.c:382-471) that sequences the device kernels.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>
#include "lpm_internal.h"
#include "damage_select.h"

namespace lpm {

thread_local std::string g_err;

int fail(int code, const std::string &msg)
{
    g_err = msg;
    return code;
}

template <typename T>
static int dalloc(T *&p, size_t count)
{
    if (p)
        cudaFree(p);
    p = nullptr;
    if (count == 0)
        count = 1;
    cudaError_t e = cudaMalloc((void **)&p, count * sizeof(T));
    if (e != cudaSuccess) {
        p = nullptr;
        return fail(LPM_ERR_NOMEM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
    }
    cudaMemset(p, 0, count * sizeof(T));
    return LPM_OK;
}

template <typename T>
static void dfree(T *&p)
{
    if (p)
        cudaFree(p);
    p = nullptr;
}

// Pinned host staging of at least `bytes`, grown when needed and kept by the
// context; null when pinned memory cannot be had.
static void *stage(Ctx &c, size_t bytes)
{
    if (bytes > c.stage_cap) {
        if (c.stage_h)
            cudaFreeHost(c.stage_h);
        c.stage_h = nullptr;
        c.stage_cap = 0;
        if (cudaMallocHost(&c.stage_h, bytes) != cudaSuccess) {
            cudaGetLastError();
            c.stage_h = nullptr;
            return nullptr;
        }
        c.stage_cap = bytes;
    }
    return c.stage_h;
}

// A host buffer for one exchange: the context's pinned staging, or an
// aligned pageable buffer of its own when pinning failed.
struct Staging {
    hvec<dvec4> own;
    char *p;
    Staging(Ctx &c, size_t bytes)
    {
        p = (char *)stage(c, bytes);
        if (!p) {
            own.resize((bytes + sizeof(dvec4) - 1) / sizeof(dvec4));
            p = (char *)own.data();
        }
    }
};

static void free_batch(Ctx &c)
{
    BatchCg &b = c.bcg;
    void *dev[] = {(void *)b.spec_of, (void *)b.off, (void *)b.seg_base, b.rz, b.rz_old, b.rr, b.rr_max,
                   b.tol2, b.alpha, b.beta, b.bscale, b.it, b.done, b.upd, b.nrel, b.active, b.partials,
                   b.counter, b.all_done, b.act_chunk, b.n_act, c.bh.norms_d, c.bh.bs, c.bh.bc_d};
    for (void *p : dev)
        if (p)
            cudaFree(p);
    void *host[] = {c.bh.norms_h, c.bh.bscale_h, c.bh.active_h, c.bh.it_h, c.bh.done_h, c.bh.nrel_h,
                    c.bh.all_done_h};
    for (void *p : host)
        if (p)
            cudaFreeHost(p);
    if (c.bh.graph)
        cudaGraphExecDestroy(c.bh.graph);
    c.bcg = BatchCg();
    c.bh = BatchHost();
    c.nspec = 0;
}

static void free_anderson(Ctx &c)
{
    dfree(c.acc.dU);
    dfree(c.acc.dF);
    dfree(c.acc.u_prev);
    dfree(c.acc.f_prev);
    dfree(c.acc.dots);
    if (c.acc.dots_h)
        cudaFreeHost(c.acc.dots_h);
    c.acc = Ctx::Anderson();
}

static void free_recycle(Ctx &c)
{
    dfree(c.rec.du);
    dfree(c.rec.b);
    dfree(c.rec.x0);
    dfree(c.rec.r0);
    dfree(c.rec.dots);
    if (c.rec.dots_h)
        cudaFreeHost(c.rec.dots_h);
    c.rec = Ctx::Recycle();
}

static void free_damage(Ctx &c)
{
    Ctx::Damage &d = c.dmg;
    dfree(d.brk);
    dfree(d.dw);
    dfree(d.D[0]);
    dfree(d.D[1]);
    dfree(d.dnl[0]);
    dfree(d.dnl[1]);
    dfree(d.dvis);
    dfree(d.nbc);
    dfree(d.opp);
    dfree(d.cstart);
    dfree(d.corder);
    dfree(d.list);
    dfree(d.lval);
    dfree(d.count);
    if (d.count_h)
        cudaFreeHost(d.count_h);
    c.dmg = Ctx::Damage();
}

Ctx::~Ctx()
{
    cudaSetDevice(device);
    free_writer(*this);
    free_batch(*this);
    free_adjoint(*this);
    free_anderson(*this);
    free_recycle(*this);
    free_damage(*this);
    free_amg(*this);
    void **all[] = {(void **)&xyz, (void **)&xyz0, (void **)&xyz_temp, (void **)&Pin, (void **)&Pex,
                    (void **)&res, (void **)&du, (void **)&mask, (void **)&type, (void **)&G, (void **)&sy,
                    (void **)&Hh, (void **)&stress, (void **)&strain, (void **)&dlambda, (void **)&nbr, (void **)&shell,
                    (void **)&rev, (void **)&nbv, (void **)&nconn_d, (void **)&L0, (void **)&Kn, (void **)&Tv,
                    (void **)&oppv, (void **)&dL, (void **)&csx, (void **)&csy, (void **)&csz, (void **)&F,
                    (void **)&F_prev, (void **)&S, (void **)&T, (void **)&ddL, (void **)&dS, (void **)&dT,
                    (void **)&Cab, (void **)&sch, (void **)&jact, (void **)&U, (void **)&W,
                    (void **)&rowoff, (void **)&npad, (void **)&cols, (void **)&Kd, (void **)&Kf,
                    (void **)&Pinv_d, (void **)&Pinv_f, (void **)&x_d, (void **)&r_d, (void **)&p_d,
                    (void **)&q_d, (void **)&z_d, (void **)&x_f, (void **)&r_f, (void **)&p_f, (void **)&q_f,
                    (void **)&z_f, (void **)&p_split, (void **)&Pinv_rf, (void **)&Krs, (void **)&Kh, (void **)&Kc, (void **)&kh_scale, (void **)&kh_max, (void **)&pl_flag, (void **)&b_d, (void **)&sc, (void **)&partials, (void **)&counter,
                    (void **)&norms, (void **)&status};
    for (void **p : all)
        if (*p) {
            cudaFree(*p);
            *p = nullptr;
        }
    for (int s = 0; s < 3; s++) {
        double **st[] = {&dLp[s], &alpha[s], &beta[s], &gy[s], &As[s], &A[s]};
        for (double **p : st)
            if (*p) {
                cudaFree(*p);
                *p = nullptr;
            }
    }
    if (sc_host)
        cudaFreeHost(sc_host);
    if (stage_h)
        cudaFreeHost(stage_h);
    if (norms_host)
        cudaFreeHost(norms_host);
    if (status_host)
        cudaFreeHost(status_host);
    if (graph_fp64)
        cudaGraphExecDestroy(graph_fp64);
    if (graph_fp32)
        cudaGraphExecDestroy(graph_fp32);
    if (ev_a)
        cudaEventDestroy(ev_a);
    if (ev_b)
        cudaEventDestroy(ev_b);
    if (own_stream && stream)
        cudaStreamDestroy(stream);
}

// ---- helpers -----------------------------------------------------------------

int sync(Ctx &c)
{
    cudaError_t e = cudaStreamSynchronize(c.stream);
    if (e != cudaSuccess)
        return fail(LPM_ERR_CUDA, std::string("kernel execution: ") + cudaGetErrorString(e));
    e = cudaGetLastError();
    if (e != cudaSuccess)
        return fail(LPM_ERR_CUDA, std::string("kernel launch: ") + cudaGetErrorString(e));
    return LPM_OK;
}

// read the residual / reaction norms written by the last force kernel
static int read_norms(Ctx &c, double &res, double &reac)
{
    LPM_CUDA(cudaMemcpyAsync(c.norms_host, c.norms, 4 * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
    int rc = sync(c);
    if (rc)
        return rc;
    res = std::sqrt(c.norms_host[0]);
    reac = std::sqrt(c.norms_host[1]);
    return LPM_OK;
}

static void copy_state(Ctx &c, int to, int from)
{
    const size_t n = c.n;
    cudaMemcpyAsync(c.dLp[to], c.dLp[from], n * LPM_NN * sizeof(double), cudaMemcpyDeviceToDevice, c.stream);
    cudaMemcpyAsync(c.alpha[to], c.alpha[from], n * sizeof(double), cudaMemcpyDeviceToDevice, c.stream);
    cudaMemcpyAsync(c.beta[to], c.beta[from], 6 * n * sizeof(double), cudaMemcpyDeviceToDevice, c.stream);
    if (c.nslip) {
        cudaMemcpyAsync(c.gy[to], c.gy[from], n * c.nslip * sizeof(double), cudaMemcpyDeviceToDevice, c.stream);
        cudaMemcpyAsync(c.As[to], c.As[from], n * c.nslip * sizeof(double), cudaMemcpyDeviceToDevice, c.stream);
        cudaMemcpyAsync(c.A[to], c.A[from], n * sizeof(double), cudaMemcpyDeviceToDevice, c.stream);
    }
}

// switchStateV (src/constitutive.c:10-85); damage_D and damage_nonlocal have
// slots 0 and 1 only and move with flags 0 and 1
void switch_state(Ctx &c, int flag)
{
    if (flag == 0)
        copy_state(c, 0, 1);
    else if (flag == 1)
        copy_state(c, 1, 0);
    else
        copy_state(c, 0, 2);
    if (c.dmg.on && flag != 2) {
        const int to = flag == 0 ? 0 : 1, from = 1 - to;
        cudaMemcpyAsync(c.dmg.D[to], c.dmg.D[from], (size_t)c.n * LPM_NN * sizeof(double), cudaMemcpyDeviceToDevice,
                        c.stream);
        cudaMemcpyAsync(c.dmg.dnl[to], c.dmg.dnl[from], (size_t)c.n * sizeof(double), cudaMemcpyDeviceToDevice,
                        c.stream);
    }
}

// transposes between host row-major [n][k] and device [k][n]
template <typename T>
static void to_slot_major(const T *src, T *dst, int n, int k)
{
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; i++)
        for (int j = 0; j < k; j++)
            dst[(size_t)j * n + i] = src[(size_t)i * k + j];
}

template <typename T>
static void from_slot_major(const T *src, T *dst, int n, int k)
{
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; i++)
        for (int j = 0; j < k; j++)
            dst[(size_t)i * k + j] = src[(size_t)j * n + i];
}

static int upload_particles(Ctx &c, dvec4 *dst, const double *src3)
{
    LPM_CUDA(cudaStreamSynchronize(c.stream));
    Staging sb(c, sizeof(dvec4) * (size_t)c.n);
    dvec4 *t = (dvec4 *)sb.p;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < c.n; i++)
        t[i] = make_dvec4(src3[3 * (size_t)i], src3[3 * (size_t)i + 1], src3[3 * (size_t)i + 2], 0.0);
    LPM_CUDA(cudaMemcpy(dst, t, sizeof(dvec4) * c.n, cudaMemcpyHostToDevice));
    return LPM_OK;
}

static int download_particles(Ctx &c, const dvec4 *src, double *dst3)
{
    Staging sb(c, sizeof(dvec4) * (size_t)c.n);
    const dvec4 *t = (const dvec4 *)sb.p;
    LPM_CUDA(cudaMemcpyAsync(sb.p, src, sizeof(dvec4) * c.n, cudaMemcpyDeviceToHost, c.stream));
    int rc = sync(c);
    if (rc)
        return rc;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < c.n; i++) {
        dst3[3 * i] = t[i].x;
        dst3[3 * i + 1] = t[i].y;
        dst3[3 * i + 2] = t[i].z;
    }
    return LPM_OK;
}

// ---- device allocation for a specimen ----------------------------------------

static int alloc_specimen(Ctx &c)
{
    const size_t n = c.n, nb = n * LPM_NN;
    int rc = 0;
#define A_(p, cnt)            \
    if ((rc = dalloc(p, cnt))) \
        return rc;
    A_(c.xyz, n) A_(c.xyz0, n) A_(c.xyz_temp, n) A_(c.Pin, n) A_(c.Pex, n) A_(c.res, n) A_(c.du, n)
    A_(c.mask, n) A_(c.type, n) A_(c.pl_flag, n) A_(c.G, n) A_(c.sy, n) A_(c.Hh, n) A_(c.stress, 6 * n) A_(c.strain, 6 * n) A_(c.dlambda, n)
    A_(c.nbr, nb) A_(c.shell, nb) A_(c.rev, nb) A_(c.nbv, n) A_(c.nconn_d, n) A_(c.L0, nb) A_(c.Kn, nb)
    A_(c.Tv, nb) A_(c.oppv, nb) A_(c.dL, nb) A_(c.csx, nb) A_(c.csy, nb) A_(c.csz, nb) A_(c.F, nb)
    A_(c.F_prev, nb) A_(c.S, n) A_(c.T, n) A_(c.ddL, nb) A_(c.dS, n) A_(c.dT, n) A_(c.U, 6 * n)
    A_(c.W, 6 * n) A_(c.Pinv_d, 9 * n) A_(c.Pinv_f, 9 * n)
    A_(c.x_d, n) A_(c.r_d, n) A_(c.p_d, n) A_(c.q_d, n) A_(c.z_d, n) A_(c.b_d, n)
    A_(c.x_f, n) A_(c.r_f, n) A_(c.p_f, n) A_(c.q_f, n) A_(c.z_f, n)
    A_(c.p_split, 2 * n) A_(c.Pinv_rf, 9 * n) A_(c.Krs, 9 * n) A_(c.kh_scale, 1) A_(c.kh_max, 1)
    c.krs_version = -1;
    for (int s = 0; s < 3; s++) {
        A_(c.dLp[s], nb) A_(c.alpha[s], n) A_(c.beta[s], 6 * n)
    }
    A_(c.sc, 1) A_(c.norms, 4) A_(c.status, 1) A_(c.counter, 1)
    int sms = 152;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c.device);
    c.tune.sms = sms;
    const size_t red = std::max<size_t>((n + 63) / 64 + 64, (size_t)sms * TUNE_MAX_PER_SM + 64);
    A_(c.partials, 4 * red)
    // block-CSR pattern
    const HostSetup &h = c.hs;
    c.nblk = h.rowoff[n];
    c.nblk_real = 0;
    for (int i = 0; i < c.n; i++)
        c.nblk_real += h.nconn[i];
    // row offsets padded past n + 1 with the total (empty rows): the streamed
    // product copies 18 offsets per tile of 16 rows
    const size_t nro = (n + 15) / 16 * 16 + 2;
    A_(c.rowoff, nro) A_(c.npad, n) A_(c.cols, (size_t)c.nblk)
#undef A_
    {
        std::vector<long long> ro(h.rowoff.begin(), h.rowoff.begin() + n + 1);
        ro.resize(nro, h.rowoff[n]);
        LPM_CUDA(cudaMemcpy(c.rowoff, ro.data(), sizeof(long long) * nro, cudaMemcpyHostToDevice));
        int max_npad = 0;
        for (size_t i = 0; i < n; i++)
            max_npad = std::max(max_npad, h.npad[i]);
        init_stream_product(c, max_npad);
        init_stream_smoother(c, max_npad);
    }
    LPM_CUDA(cudaMemcpy(c.npad, h.npad.data(), sizeof(int) * n, cudaMemcpyHostToDevice));
    LPM_CUDA(cudaMemcpy(c.cols, h.cols.data(), sizeof(int) * c.nblk, cudaMemcpyHostToDevice));
    if (!c.sc_host) {
        LPM_CUDA(cudaMallocHost((void **)&c.sc_host, sizeof(CgScalars)));
        LPM_CUDA(cudaMallocHost((void **)&c.norms_host, 4 * sizeof(double)));
        LPM_CUDA(cudaMallocHost((void **)&c.status_host, sizeof(int)));
    }
    return LPM_OK;
}

static int upload_setup(Ctx &c)
{
    const HostSetup &h = c.hs;
    const int n = c.n;
    const size_t nb = (size_t)n * LPM_NN;
    int rc = upload_particles(c, c.xyz, h.xyz.data());
    if (rc)
        return rc;
    rc = upload_particles(c, c.xyz0, h.xyz.data());
    if (rc)
        return rc;
    rc = upload_particles(c, c.xyz_temp, h.xyz.data());
    if (rc)
        return rc;
    hvec<int> ti(nb);
    hvec<int8_t> t8(nb);
    hvec<double> td(nb);
    to_slot_major(h.nbr.data(), ti.data(), n, LPM_NN);
    LPM_CUDA(cudaMemcpy(c.nbr, ti.data(), nb * sizeof(int), cudaMemcpyHostToDevice));
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; i++)
        for (int j = 0; j < LPM_NN; j++) {
            t8[(size_t)j * n + i] = (int8_t)h.shell[(size_t)i * LPM_NN + j];
        }
    LPM_CUDA(cudaMemcpy(c.shell, t8.data(), nb, cudaMemcpyHostToDevice));
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; i++)
        for (int j = 0; j < LPM_NN; j++)
            t8[(size_t)j * n + i] = (int8_t)h.rev[(size_t)i * LPM_NN + j];
    LPM_CUDA(cudaMemcpy(c.rev, t8.data(), nb, cudaMemcpyHostToDevice));
    std::vector<int8_t> v8(n);
    for (int i = 0; i < n; i++)
        v8[i] = (int8_t)h.nb[i];
    LPM_CUDA(cudaMemcpy(c.nbv, v8.data(), n, cudaMemcpyHostToDevice));
    for (int i = 0; i < n; i++)
        v8[i] = (int8_t)h.nconn[i];
    LPM_CUDA(cudaMemcpy(c.nconn_d, v8.data(), n, cudaMemcpyHostToDevice));
    to_slot_major(h.L0.data(), td.data(), n, LPM_NN);
    LPM_CUDA(cudaMemcpy(c.L0, td.data(), nb * sizeof(double), cudaMemcpyHostToDevice));
    to_slot_major(h.oppv.data(), td.data(), n, LPM_NN);
    LPM_CUDA(cudaMemcpy(c.oppv, td.data(), nb * sizeof(double), cudaMemcpyHostToDevice));
    std::vector<uint8_t> m(n, 7);
    LPM_CUDA(cudaMemcpy(c.mask, m.data(), n, cudaMemcpyHostToDevice));
    return LPM_OK;
}

static void drop_graphs(Ctx &c);

static int setup_common(Ctx &c, bool built = false)
{
    // everything sized for, or captured with, the previous specimen's arrays
    // (CUDA graphs hold the old device pointers) goes before reallocation
    free_writer(c);
    free_adjoint(c);
    free_anderson(c);
    free_recycle(c);
    free_damage(c);
    free_amg(c);
    drop_graphs(c);
    dfree(c.Kf);
    dfree(c.Kd);
    dfree(c.Kh);
    dfree(c.Kc);
    c.kf_cap = c.kd_cap = c.kh_cap = c.kc_cap = 0;
    c.kf_version = -1;
    c.kh_version = -1;
    c.kc_version = -1;
    c.vec64_fallback = false;
    c.amg_k64 = false;
    HostSetup &h = c.hs;
    if (!built) {
        const int brc = build_neighbors(h);
        if (brc < 0)
            return brc;
        build_afem(h);
        build_bond_tables(h);
        build_block_pattern(h);
    }
    c.n = h.n;
    c.ready = false;
    c.have_K = false;
    c.nslip = 0;
    int rc = alloc_specimen(c);
    if (rc)
        return rc;
    rc = upload_setup(c);
    if (rc)
        return rc;
    return c.n;
}

}  // namespace lpm

using namespace lpm;

// ---- C ABI -------------------------------------------------------------------

extern "C" {

const char *lpm_last_error(void) { return g_err.c_str(); }

void lpm_default_solver_opts(lpm_solver_opts *o)
{
    o->precision = LPM_PREC_FP64;
    o->newton_tol = 1e-8;
    o->newton_maxiter = 100;
    o->cg_rtol = 1e-10;
    o->cg_maxiter = 20000;
    o->inner_rtol = 0.1;
    o->refine_maxiter = 200;
    o->check_every = 16;
    o->use_graphs = 1;
    o->mixed_vectors = 32;
    o->newton_accel = 0;
    o->cg_forcing = 0.0;
    o->preconditioner = LPM_PRECOND_BJ;
    o->amg_spacing = 0.0;
    o->amg_rebuild = 2.5;
    o->amg_sweeps = 1;
    o->recycle = 0;
}

int lpm_create(lpm_ctx **out, int device)
{
    if (!out)
        return fail(LPM_ERR_ARG, "null output pointer");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= 0)
        return fail(LPM_ERR_CUDA, "no CUDA device available");
    if (device < 0 || device >= ndev)
        return fail(LPM_ERR_ARG, "device index out of range");
    lpm_ctx *x = new (std::nothrow) lpm_ctx;
    if (!x)
        return fail(LPM_ERR_NOMEM, "host allocation failed");
    Ctx &c = x->c;
    c.device = device;
    if (cudaSetDevice(device) != cudaSuccess || cudaStreamCreateWithFlags(&c.stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete x;
        return fail(LPM_ERR_CUDA, "stream creation failed");
    }
    c.own_stream = true;
    cudaEventCreate(&c.ev_a);
    cudaEventCreate(&c.ev_b);
    lpm_default_solver_opts(&c.opts);
    const char *tr = std::getenv("LPM_TRACE");
    c.trace = tr && tr[0] && std::strcmp(tr, "0") != 0;
    *out = x;
    return LPM_OK;
}

void lpm_destroy(lpm_ctx *ctx) { delete ctx; }

int lpm_set_stream(lpm_ctx *ctx, void *stream)
{
    if (!ctx)
        return fail(LPM_ERR_ARG, "null context");
    Ctx &c = ctx->c;
    if (c.graph_fp64) {
        cudaGraphExecDestroy(c.graph_fp64);
        c.graph_fp64 = nullptr;
    }
    if (c.graph_fp32) {
        cudaGraphExecDestroy(c.graph_fp32);
        c.graph_fp32 = nullptr;
    }
    if (stream) {
        if (c.own_stream && c.stream)
            cudaStreamDestroy(c.stream);
        c.stream = (cudaStream_t)stream;
        c.own_stream = false;
    } else if (!c.own_stream) {
        cudaStreamCreateWithFlags(&c.stream, cudaStreamNonBlocking);
        c.own_stream = true;
    }
    return LPM_OK;
}

int lpm_set_solver(lpm_ctx *ctx, const lpm_solver_opts *o)
{
    if (!ctx || !o)
        return fail(LPM_ERR_ARG, "null argument");
    if (o->precision != LPM_PREC_FP64 && o->precision != LPM_PREC_MIXED)
        return fail(LPM_ERR_ARG, "unknown precision");
    if (!(o->cg_rtol > 0) || o->cg_maxiter <= 0 || o->newton_maxiter < 0 || o->check_every <= 0 ||
        o->newton_accel < 0 || o->newton_accel > 16 || !(o->cg_forcing >= 0.0 && o->cg_forcing < 1.0) ||
        (o->preconditioner != LPM_PRECOND_BJ && o->preconditioner != LPM_PRECOND_AMG) ||
        !(o->amg_spacing >= 0.0) || !(o->amg_rebuild > 1.0) || o->amg_sweeps < 1 || o->amg_sweeps > 4 ||
        o->recycle < 0 || o->recycle > 8)
        return fail(LPM_ERR_ARG, "invalid solver options");
    Ctx &c = ctx->c;
    const bool prec_change = c.opts.precision != o->precision;
    if (c.amg && o->preconditioner != LPM_PRECOND_AMG)
        free_amg(c);  // graphs that use it are dropped below
    else if (c.amg && c.opts.amg_spacing != o->amg_spacing)
        c.amg->stale = true;
    c.opts = *o;
    c.vec64_fallback = false;
    c.amg_k64 = false;
    if (prec_change)
        c.have_K = false;
    if (c.graph_fp64) {
        cudaGraphExecDestroy(c.graph_fp64);
        c.graph_fp64 = nullptr;
    }
    if (c.graph_fp32) {
        cudaGraphExecDestroy(c.graph_fp32);
        c.graph_fp32 = nullptr;
    }
    return LPM_OK;
}

int lpm_setup_lattice(lpm_ctx *ctx, int lattice, double radius, const double box[6])
{
    if (!ctx || !box)
        return fail(LPM_ERR_ARG, "null argument");
    Ctx &c = ctx->c;
    cudaSetDevice(c.device);
    free_batch(c);
    c.hs = HostSetup();
    int rc = build_lattice(c.hs, lattice, radius, box);
    if (rc < 0)
        return rc;
    return setup_common(c);
}

int lpm_setup_particles(lpm_ctx *ctx, int lattice, double radius, int n, const double *xyz)
{
    if (!ctx)
        return fail(LPM_ERR_ARG, "null context");
    Ctx &c = ctx->c;
    cudaSetDevice(c.device);
    free_batch(c);
    c.hs = HostSetup();
    int rc = build_particles(c.hs, lattice, radius, n, xyz);
    if (rc < 0)
        return rc;
    return setup_common(c);
}

int lpm_nparticle(const lpm_ctx *ctx) { return ctx ? ctx->c.n : 0; }

int lpm_get_sizes(const lpm_ctx *ctx, int *n, int *nn, int *nslip, long long *nnzb)
{
    if (!ctx)
        return fail(LPM_ERR_ARG, "null context");
    if (n)
        *n = ctx->c.n;
    if (nn)
        *nn = LPM_NN;
    if (nslip)
        *nslip = ctx->c.nslip;
    if (nnzb)
        *nnzb = ctx->c.nblk_real;
    return LPM_OK;
}

int lpm_set_types(lpm_ctx *ctx, const int *type)
{
    if (!ctx || !type || ctx->c.n <= 0)
        return fail(LPM_ERR_ARG, "set up the specimen before its types");
    LPM_CUDA(cudaMemcpy(ctx->c.type, type, sizeof(int) * ctx->c.n, cudaMemcpyHostToDevice));
    return LPM_OK;
}

int lpm_set_material(lpm_ctx *ctx, const double *c11, const double *c12, const double *c44,
                     const double *sigmay, const double *hardening, double xi, int plmode)
{
    if (!ctx || !c11 || !c12 || !c44 || ctx->c.n <= 0)
        return fail(LPM_ERR_ARG, "set up the specimen and pass C11, C12, C44 per particle");
    Ctx &c = ctx->c;
    LPM_CUDA(cudaStreamSynchronize(c.stream));
    if (plmode != LPM_PL_J2 && plmode != LPM_PL_CP && plmode != LPM_PL_ELASTIC)
        return fail(LPM_ERR_ARG, "plmode must be 0 (J2), 1 (crystal plasticity) or 6 (elastic)");
    if (plmode == LPM_PL_CP && c.hs.lattice != 3)
        return fail(LPM_ERR_ARG, "crystal plasticity needs the FCC lattice (3)");
    const int n = c.n;
    const HostSetup &h = c.hs;
    std::vector<double> knt(3 * (size_t)n);
    kntv_per_particle(h.lattice, h.radius, c11, c12, c44, n, knt.data());
    std::vector<double> kn((size_t)n * LPM_NN, 0.0), tv((size_t)n * LPM_NN, 0.0);
    for (int i = 0; i < n; i++)
        for (int j = 0; j < h.nb[i]; j++) {
            const size_t b = (size_t)i * LPM_NN + j;
            const int p = h.nbr[b], s = h.shell[b];
            if (h.lattice == 2) {  // src/stiffness.c:192-200, averaged over the bond ends
                kn[b] = 0.5 * (knt[3 * i + s] + knt[3 * p + s]);
                tv[b] = 0.5 * (knt[3 * i + 2] + knt[3 * p + 2]);
            } else {               // src/stiffness.c:223-232, the particle's own values
                kn[b] = knt[3 * i + s];
                tv[b] = knt[3 * i + 2];
            }
        }
    std::vector<double> t((size_t)n * LPM_NN);
    to_slot_major(kn.data(), t.data(), n, LPM_NN);
    LPM_CUDA(cudaMemcpy(c.Kn, t.data(), t.size() * sizeof(double), cudaMemcpyHostToDevice));
    to_slot_major(tv.data(), t.data(), n, LPM_NN);
    LPM_CUDA(cudaMemcpy(c.Tv, t.data(), t.size() * sizeof(double), cudaMemcpyHostToDevice));
    LPM_CUDA(cudaMemcpy(c.G, c44, sizeof(double) * n, cudaMemcpyHostToDevice));
    std::vector<double> z(n, 0.0);
    LPM_CUDA(cudaMemcpy(c.sy, sigmay ? sigmay : z.data(), sizeof(double) * n, cudaMemcpyHostToDevice));
    LPM_CUDA(cudaMemcpy(c.Hh, hardening ? hardening : z.data(), sizeof(double) * n, cudaMemcpyHostToDevice));
    c.xi = xi;
    c.plmode = plmode;
    c.have_K = false;
    return LPM_OK;
}

int lpm_set_cp(lpm_ctx *ctx, const double cp[8])
{
    if (!ctx || !cp)
        return fail(LPM_ERR_ARG, "null argument");
    if (!(cp[3] > 0) || !(cp[7] > 0) || !(cp[1] > cp[0]))
        return fail(LPM_ERR_ARG, "crystal plasticity needs p > 0, dtime > 0 and taus > tau0");
    std::memcpy(ctx->c.cp, cp, sizeof(ctx->c.cp));
    return LPM_OK;
}

int lpm_init_state(lpm_ctx *ctx)
{
    if (!ctx || ctx->c.n <= 0)
        return fail(LPM_ERR_ARG, "set up the specimen first");
    Ctx &c = ctx->c;
    const size_t n = c.n, nb = n * LPM_NN;
    if (c.dmg.on) {
        // back to intact bonds: the setup's stress weights, no damage stage
        hvec<double> t(nb);
        to_slot_major(c.hs.oppv.data(), t.data(), c.n, LPM_NN);
        LPM_CUDA(cudaMemcpy(c.oppv, t.data(), nb * sizeof(double), cudaMemcpyHostToDevice));
        free_damage(c);
    }
    for (int s = 0; s < 3; s++) {
        LPM_CUDA(cudaMemsetAsync(c.dLp[s], 0, nb * sizeof(double), c.stream));
        LPM_CUDA(cudaMemsetAsync(c.alpha[s], 0, n * sizeof(double), c.stream));
        LPM_CUDA(cudaMemsetAsync(c.beta[s], 0, 6 * n * sizeof(double), c.stream));
    }
    LPM_CUDA(cudaMemsetAsync(c.F, 0, nb * sizeof(double), c.stream));
    LPM_CUDA(cudaMemsetAsync(c.F_prev, 0, nb * sizeof(double), c.stream));
    LPM_CUDA(cudaMemsetAsync(c.Pex, 0, n * sizeof(dvec4), c.stream));
    LPM_CUDA(cudaMemsetAsync(c.Pin, 0, n * sizeof(dvec4), c.stream));
    LPM_CUDA(cudaMemsetAsync(c.status, 0, sizeof(int), c.stream));
    LPM_CUDA(cudaMemsetAsync(c.pl_flag, 0, n * sizeof(int), c.stream));
    LPM_CUDA(cudaMemcpyAsync(c.xyz, c.xyz0, n * sizeof(dvec4), cudaMemcpyDeviceToDevice, c.stream));
    std::vector<uint8_t> m(n, 7);
    LPM_CUDA(cudaMemcpy(c.mask, m.data(), n, cudaMemcpyHostToDevice));
    // computedL (src/lpm_basic.c:252-291): stretches and unit vectors at rest
    launch_stretch(c, c.dLp[0], true);
    if (c.hs.lattice == 3 && c.plmode == LPM_PL_CP) {
        // slipSysDefine3D (src/initialization.c:565-637): 24 signed {111}<110>
        static const int pl[4][3] = {{1, 1, 1}, {-1, 1, 1}, {1, -1, 1}, {-1, -1, 1}};
        static const int dir[4][6][3] = {
            {{1, -1, 0}, {-1, 1, 0}, {-1, 0, 1}, {1, 0, -1}, {0, 1, -1}, {0, -1, 1}},
            {{1, 0, 1}, {-1, 0, -1}, {-1, -1, 0}, {1, 1, 0}, {0, 1, -1}, {0, -1, 1}},
            {{-1, 0, 1}, {1, 0, -1}, {0, -1, -1}, {0, 1, 1}, {1, 1, 0}, {-1, -1, 0}},
            {{-1, 1, 0}, {1, -1, 0}, {1, 0, 1}, {-1, 0, -1}, {0, -1, -1}, {0, 1, 1}}};
        const double a3 = 1 / std::sqrt(3.0), a2 = 1 / std::sqrt(2.0);
        std::vector<double> sch(6 * LPM_NSLIP);
        int m2 = 0;
        for (int p = 0; p < 4; p++)
            for (int d = 0; d < 6; d++, m2++) {
                double nv[3], sv[3];
                for (int k = 0; k < 3; k++) {
                    nv[k] = pl[p][k] * a3;
                    sv[k] = dir[p][d][k] * a2;
                }
                double *s = &sch[6 * m2];
                s[0] = nv[0] * sv[0];
                s[1] = nv[1] * sv[1];
                s[2] = nv[2] * sv[2];
                s[3] = nv[1] * sv[2] + nv[2] * sv[1];
                s[4] = nv[0] * sv[2] + nv[2] * sv[0];
                s[5] = nv[0] * sv[1] + nv[1] * sv[0];
            }
        c.nslip = LPM_NSLIP;
        int rc = 0;
        for (int s = 0; s < 3; s++) {
            if ((rc = dalloc(c.gy[s], n * LPM_NSLIP)) || (rc = dalloc(c.As[s], n * LPM_NSLIP)) ||
                (rc = dalloc(c.A[s], n)))
                return rc;
            std::vector<double> g0(n * LPM_NSLIP, c.cp[0]);  // cp_gy = tau0 (src/initialization.c:570)
            LPM_CUDA(cudaMemcpy(c.gy[s], g0.data(), g0.size() * sizeof(double), cudaMemcpyHostToDevice));
        }
        if ((rc = dalloc(c.Cab, n * LPM_NSLIP * LPM_NSLIP)) || (rc = dalloc(c.sch, 6 * LPM_NSLIP)) ||
            (rc = dalloc(c.jact, n)))
            return rc;
        LPM_CUDA(cudaMemcpy(c.sch, sch.data(), sch.size() * sizeof(double), cudaMemcpyHostToDevice));
        launch_cab(c);  // computeCab (src/constitutive.c:1864-1917)
    }
    c.ready = true;
    c.have_K = false;
    return sync(c);
}

}  // extern "C"

// ---- solver ------------------------------------------------------------------

namespace lpm {

enum PcgMode { PCG_FP64 = 0, PCG_FP32 = 1, PCG_FP32_K_FP64_VEC = 2, PCG_AMG_K64 = 3, PCG_AMG_K32 = 4 };

// One chunk of PCG iterations; the first SpMV of the chunk (which always does
// work: a chunk is only launched while the solve is running) carries the
// timing events when sampling is on.
static void issue_chunk(Ctx &c, int mode, int chunk)
{
    for (int k = 0; k < chunk; k++) {
        c.time_this = (k == 0);
        if (mode == PCG_FP64)
            launch_cg_iter_d(c);
        else if (mode == PCG_FP32)
            launch_cg_iter_f(c);
        else if (mode == PCG_FP32_K_FP64_VEC)
            launch_cg_iter_fx(c);
        else
            launch_amg_iter(c, mode == PCG_AMG_K32);
    }
    c.time_this = false;
}

// Run PCG iterations until the device marks the solve done; the host checks
// every opts.check_every iterations (one CUDA graph per chunk when enabled).
static int run_pcg(Ctx &c, int mode, int &iters, int &status)
{
    const int chunk = c.opts.check_every;
    cudaGraphExec_t &ge = mode == PCG_FP32 ? c.graph_fp32 : c.graph_fp64;
    bool use_graph = c.opts.use_graphs != 0;
    if (ge && (c.graph_timed != c.time_spmv || c.graph_chunk != chunk || c.graph_mode != mode)) {
        cudaGraphExecDestroy(ge);
        ge = nullptr;
    }
    if (use_graph && !ge) {
        cudaGraph_t g;
        if (cudaStreamBeginCapture(c.stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
            use_graph = false;
        } else {
            issue_chunk(c, mode, chunk);
            if (cudaStreamEndCapture(c.stream, &g) != cudaSuccess) {
                use_graph = false;
            } else {
                if (cudaGraphInstantiate(&ge, g, 0) != cudaSuccess) {
                    ge = nullptr;
                    use_graph = false;
                }
                cudaGraphDestroy(g);
                c.graph_chunk = chunk;
                c.graph_timed = c.time_spmv;
                c.graph_mode = mode;
            }
        }
        cudaGetLastError();
    }
    for (;;) {
        if (use_graph) {
            LPM_CUDA(cudaGraphLaunch(ge, c.stream));
        } else {
            issue_chunk(c, mode, chunk);
        }
        LPM_CUDA(cudaMemcpyAsync(c.sc_host, c.sc, sizeof(CgScalars), cudaMemcpyDeviceToHost, c.stream));
        if (c.time_spmv) {
            // one sampled SpMV launch per chunk (the last one issued)
            int rc = sync(c);
            if (rc)
                return rc;
            float ms = 0.f;
            if (cudaEventElapsedTime(&ms, c.ev_a, c.ev_b) == cudaSuccess) {
                c.spmv_ms_sum += ms;
                c.spmv_count++;
            }
        } else {
            int rc = sync(c);
            if (rc)
                return rc;
        }
        if (c.sc_host->done)
            break;
    }
    iters = c.sc_host->it;
    status = c.sc_host->done;
    return LPM_OK;
}

// Solve K x = b (b on the device, masked); x is written to c.du.
// The right-hand side is normalised by |b| so the iterates stay O(1) and
// squared residual norms 1e-10..1e-12 below the start cannot underflow (the
// reference's CG divides 0/0 there once forces are small).
// FP64: block-Jacobi PCG.  Mixed: FP32 PCG with reliable updates - when the
// FP32 recursive residual has fallen by the factor opts.inner_rtol since the
// last update (or meets the tolerance), x64 absorbs the FP32 increment, the
// true residual b - K32 x64 is recomputed with FP64 products and sums, and
// replaces the FP32 residual; the search direction is kept, so CG keeps its
// Krylov history.  Convergence is judged on the FP64 true residual.
// Multigrid-preconditioned CG (k_amg.cu) with FP64 vectors, the right-hand
// side normalised by |b| as below.  FP64: the recursive residual decides.
// Mixed: FP32 stiffness and products; at a reliable-update request or at
// convergence the true residual s b - K32 x is recomputed with FP64 sums and
// replaces r (p is kept), and convergence is judged on it.  A solve that
// needs more iterations per decade of residual reduction than opts.amg_rebuild
// times those of the first solve after the last build marks the hierarchy
// for a rebuild before the next solve.
static int solve_amg(Ctx &c, const dvec4 *b, double bn, lpm_step_stats *st)
{
    int rc;
    if (c.kf_version != c.k_version) {
        // FP64 stiffness assembled before the multigrid was switched on: the
        // smoother's FP32 copy
        if (!c.Kf || c.kf_cap != c.nblk) {
            drop_graphs(c);  // captured with the old Kf
            if ((rc = dalloc(c.Kf, 9 * (size_t)c.nblk)))
                return rc;
            c.kf_cap = c.nblk;
        }
        launch_amg_stiffness32(c);
        c.kf_version = c.k_version;
    }
    const int builds0 = c.amg ? c.amg->builds : 0;
    if ((rc = amg_prepare(c)))
        return rc;
    AmgDev &H = *c.amg;
    if (st && H.builds != builds0) {
        st->amg_builds += H.builds - builds0;
        st->ms_amg_build += H.build_ms;
    }
    const bool k32 = c.opts.precision == LPM_PREC_MIXED && !c.amg_k64;
    const double scale = 1.0 / bn;
    // The multigrid PCG gains a decade every one or two iterations, so a
    // reliable update per decade (inner_rtol 0.1) would cost a host round trip
    // every other iteration (measured on a GB300 at SC 10^3: 28 updates per
    // 53 iterations); one per three decades keeps the FP32-product drift of
    // the recursive residual far below the tolerance checks on the true one.
    const double delta = std::min(c.opts.inner_rtol, 1e-3);
    if (k32 && c.krs_version != c.kf_version) {
        launch_row_sums(c);  // for the difference-form product
        c.krs_version = c.kf_version;
    }
    if (c.kh_version != c.kf_version) {
        // the level-0 smoother's FP16 stiffness
        if (!c.Kh || c.kh_cap != c.nblk) {
            drop_graphs(c);
            // + 8 values: the streamed smoother copies whole 16-byte units
            if ((rc = dalloc(c.Kh, 9 * (size_t)c.nblk + 8)))
                return rc;
            c.kh_cap = c.nblk;
        }
        launch_amg_stiffness16(c);
        c.kh_version = c.kf_version;
    }
    if (k32 && c.kc_version != c.kf_version) {
        // the reliable updates' true residual reads an exact FP64 copy of
        // the FP32 stiffness (FP64 products without per-value conversions)
        if (!c.Kc || c.kc_cap != c.nblk) {
            drop_graphs(c);
            if ((rc = dalloc(c.Kc, 9 * (size_t)c.nblk)))
                return rc;
            c.kc_cap = c.nblk;
        }
        launch_stiffness64_of32(c);
        c.kc_version = c.kf_version;
    }
    launch_amg_init(c, b, scale, k32 ? delta * delta : 0.0, k32);
    int sweeps = 0, it = 0, done = 0;
    double rel = 1.0;
    for (;;) {
        if ((rc = run_pcg(c, k32 ? PCG_AMG_K32 : PCG_AMG_K64, it, done)))
            return rc;
        if (!k32) {
            rel = std::sqrt(c.sc_host->rr / std::max(c.sc_host->bnorm2, 1e-300));
            break;
        }
        launch_refine_residual(c, c.x_d, b, c.q_d, scale);
        LPM_CUDA(cudaMemcpyAsync(c.norms_host, c.norms, 4 * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
        if ((rc = sync(c)))
            return rc;
        rel = std::sqrt(c.norms_host[2]);
        sweeps++;
        if (rel <= solve_rtol(c) || done == 2 || done == 3 || !std::isfinite(rel) ||
            sweeps >= c.opts.refine_maxiter)
            break;
        launch_amg_reliable(c, c.q_d);
    }
    if (k32 && (done == 2 || done == 3 || !std::isfinite(rel))) {
        // FP32 products failed on this system (the FP32 rounding of an
        // ill-conditioned stiffness moves its smallest eigenvalues by as much
        // as they are): solve it again with the FP64 products of the FP64
        // assembly (Kd), and keep those for the rest of the context
        c.amg_k64 = true;
        if (c.trace)
            std::fprintf(stderr, "lpm: solve amg-fp32K failed (end %d, rel %.3e after %d iterations): FP64 "
                                 "products from now on\n",
                         done, rel, it);
        if (st) {
            st->cg_iters += it;
            st->spmv_calls += it + sweeps;
            st->refine_iters += sweeps;
            st->fp64_fallbacks++;
        }
        drop_graphs(c);
        return solve_amg(c, b, bn, st);
    }
    if (st) {
        st->cg_iters += it;
        st->spmv_calls += it + sweeps;
        st->refine_iters += sweeps;
        if (done == 2 || (k32 && rel > solve_rtol(c)))
            st->status |= std::isfinite(rel) ? LPM_STATUS_CG_MAXIT : LPM_STATUS_NAN;
        if (done == 3)
            st->status |= LPM_STATUS_NAN;
    }
    // iterations per decade of residual reduction against the first solve
    // after the build
    if (std::isfinite(rel) && rel > 0.0 && rel < 1.0 && it > 0) {
        const double per_decade = it / std::max(0.5, -std::log10(rel));
        if (H.ref_iters < 0)
            H.ref_iters = std::max(1, (int)std::lround(per_decade * 100.0));
        else if (per_decade * 100.0 > c.opts.amg_rebuild * H.ref_iters)
            H.stale = true;
    }
    if (c.trace)
        std::fprintf(stderr, "lpm: solve amg-%s |b| %.6e iters %d sweeps %d rel %.3e end %d%s\n",
                     k32 ? "fp32K" : "fp64", bn, it, sweeps, rel, done, H.stale ? " (rebuild next)" : "");
    launch_scale_copy(c, c.du, c.x_d, bn);
    return LPM_OK;
}

static int solve_plain(Ctx &c, const dvec4 *b, lpm_step_stats *st)
{
    int rc;
    launch_norm2(c, b, 2);
    LPM_CUDA(cudaMemcpyAsync(c.norms_host, c.norms, 4 * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
    if ((rc = sync(c)))
        return rc;
    const double bn = std::sqrt(c.norms_host[2]);
    if (!(bn > 0.0) || !std::isfinite(bn)) {
        LPM_CUDA(cudaMemsetAsync(c.du, 0, sizeof(dvec4) * c.n, c.stream));
        if (st && !std::isfinite(bn))
            st->status |= LPM_STATUS_NAN;
        return LPM_OK;
    }
    if (c.opts.preconditioner == LPM_PRECOND_AMG && c.nspec == 0)
        return solve_amg(c, b, bn, st);
    const double scale = 1.0 / bn;
    const double delta = c.opts.inner_rtol;
    if (c.opts.precision == LPM_PREC_MIXED && (c.opts.mixed_vectors == 64 || c.vec64_fallback)) {
        // FP32 stiffness and products, FP64 vectors (x in units of |b|);
        // reliable updates replace r by s b - K32 x computed with FP64 sums
        launch_cg_init_fx(c, b, scale, delta * delta);
        int sweeps = 0, it = 0, done = 0;
        double rel = 1.0;
        for (;;) {
            if ((rc = run_pcg(c, PCG_FP32_K_FP64_VEC, it, done)))
                return rc;
            launch_refine_residual(c, c.x_d, b, c.q_d, scale);
            LPM_CUDA(cudaMemcpyAsync(c.norms_host, c.norms, 4 * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
            if ((rc = sync(c)))
                return rc;
            rel = std::sqrt(c.norms_host[2]);
            sweeps++;
            if (rel <= solve_rtol(c) || done == 2 || done == 3 || !std::isfinite(rel) ||
                sweeps >= c.opts.refine_maxiter)
                break;
            launch_reliable_d(c, c.q_d);
        }
        if (st) {
            st->cg_iters += it;
            st->spmv_calls += it + sweeps;
            st->refine_iters += sweeps;
            if (rel > solve_rtol(c))
                st->status |= std::isfinite(rel) ? LPM_STATUS_CG_MAXIT : LPM_STATUS_NAN;
        }
        if (c.trace)
            std::fprintf(stderr, "lpm: solve fp32-K/fp64-vec |b| %.6e iters %d sweeps %d rel %.3e end %d\n", bn,
                         it, sweeps, rel, done);
        launch_scale_copy(c, c.du, c.x_d, bn);
        return LPM_OK;
    }
    if (c.opts.precision == LPM_PREC_FP64) {
        launch_cg_init_d(c, b, scale);
        int it = 0, done = 0;
        if ((rc = run_pcg(c, PCG_FP64, it, done)))
            return rc;
        if (st) {
            st->cg_iters += it;
            st->spmv_calls += it;
            if (done == 2)
                st->status |= LPM_STATUS_CG_MAXIT;
            if (done == 3)
                st->status |= LPM_STATUS_NAN;
        }
        if (c.trace)
            std::fprintf(stderr, "lpm: solve fp64 |b| %.6e iters %d end %d\n", bn, it, done);
        launch_scale_copy(c, c.du, c.x_d, bn);
        return LPM_OK;
    }
    LPM_CUDA(cudaMemsetAsync(c.x_d, 0, sizeof(dvec4) * c.n, c.stream));
    launch_cg_init_f(c, b, scale, solve_rtol(c), delta * delta);
    int sweeps = 0, it = 0, done = 0;
    double rn = bn;
    std::vector<double> hist;  // true residual after each reliable update
    bool stagnated = false;
    for (;;) {
        if ((rc = run_pcg(c, PCG_FP32, it, done)))
            return rc;
        launch_axpy_refine(c, scale);
        launch_refine_residual(c, c.x_d, b, c.r_d, 1.0);
        LPM_CUDA(cudaMemcpyAsync(c.norms_host, c.norms, 4 * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
        if ((rc = sync(c)))
            return rc;
        rn = std::sqrt(c.norms_host[2]);
        sweeps++;
        hist.push_back(rn);
        if (rn <= solve_rtol(c) * bn || done == 3 || !std::isfinite(rn) || sweeps >= c.opts.refine_maxiter)
            break;
        // FP32 vectors stagnate on very ill-conditioned systems: a healthy
        // sweep cuts the true residual by about inner_rtol, so three sweeps
        // that do not halve it (or the FP32 iteration cap) mean stagnation
        if (done == 2 || (sweeps > 3 && rn > 0.5 * hist[sweeps - 4])) {
            stagnated = true;
            break;
        }
        launch_reliable(c, c.r_d, scale);
    }
    if (st) {
        st->cg_iters += it;
        st->spmv_calls += it + sweeps;
        st->refine_iters += sweeps;
    }
    if (c.trace)
        std::fprintf(stderr, "lpm: solve fp32 |b| %.6e iters %d sweeps %d rel %.3e end %d%s\n", bn, it, sweeps,
                     rn / bn, done, stagnated ? " stagnated" : "");
    if (stagnated) {
        // redo this solve, and the context's later ones, with FP64 vectors
        // (the FP32 stiffness and products stay)
        c.vec64_fallback = true;
        return solve_plain(c, b, st);
    }
    if (st && rn > solve_rtol(c) * bn)
        st->status |= std::isfinite(rn) ? LPM_STATUS_CG_MAXIT : LPM_STATUS_NAN;
    LPM_CUDA(cudaMemcpyAsync(c.du, c.x_d, sizeof(dvec4) * c.n, cudaMemcpyDeviceToDevice, c.stream));
    return LPM_OK;
}

static bool spd_solve(std::vector<double> G, int h, int ld, std::vector<double> &x);

// r = b - K x (masked) in the precision of the solve, |r|^2 into norms[2]:
// the FP64 stiffness, or the exact FP64 copy of the FP32 one when there is
// one, else the FP32 values with FP64 products
static void true_residual(Ctx &c, const dvec4 *x, const dvec4 *b, dvec4 *r)
{
    if (c.opts.precision == LPM_PREC_FP64 || c.amg_k64)
        launch_refine_residual64(c, c.Kd, x, b, r);
    else
        launch_refine_residual(c, x, b, r, 1.0);
}

static int recycle_prepare(Ctx &c, int m)
{
    Ctx::Recycle &R = c.rec;
    if (R.m == m && R.du)
        return LPM_OK;
    free_recycle(c);
    int rc;
    const size_t n = c.n;
    if ((rc = dalloc(R.du, (size_t)m * n)) || (rc = dalloc(R.b, (size_t)m * n)) || (rc = dalloc(R.x0, n)) ||
        (rc = dalloc(R.r0, n)) || (rc = dalloc(R.dots, 16)))
        return rc;
    LPM_CUDA(cudaMallocHost((void **)&R.dots_h, 16 * sizeof(double)));
    R.m = m;
    R.G.assign((size_t)m * m, 0.0);
    return LPM_OK;
}

// dots_h[j] = A_j . w over the stored slots j (in slot order)
static int recycle_dots(Ctx &c, const dvec4 *const *A, int k, const dvec4 *w)
{
    adj_multidot(c, k, A, w, c.rec.dots);
    LPM_CUDA(cudaMemcpyAsync(c.rec.dots_h, c.rec.dots, k * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
    return sync(c);
}

// Solve K du = b (-> c.du) from the Galerkin combination of the load step's
// earlier solutions (opts.recycle): with K du_j = b_j, the guess
// x0 = sum_j c_j du_j with G c = (du_j . b) minimises the energy norm of its
// error over their span.  One true residual r0 = b - K x0 follows, the
// solver gains the remaining decades on r0, and (du, b) joins the store.
int solve_device(Ctx &c, const dvec4 *b, lpm_step_stats *st)
{
    const int m = std::min(c.opts.recycle, 8);
    if (m <= 0 || c.nspec != 0)
        return solve_plain(c, b, st);
    int rc;
    if ((rc = recycle_prepare(c, m)))
        return rc;
    Ctx::Recycle &R = c.rec;
    const size_t n = c.n;
    if (R.k_version != c.k_version) {  // a new stiffness: the stored pairs no longer apply
        R.count = 0;
        R.head = 0;
        R.k_version = c.k_version;
    }
    const dvec4 *slots_du[8], *slots_b[8];
    for (int j = 0; j < R.count; j++) {
        slots_du[j] = R.du + (size_t)j * n;
        slots_b[j] = R.b + (size_t)j * n;
    }
    bool guessed = false;
    const double rtol0 = c.cg_rtol_now;
    if (R.count > 0) {
        launch_norm2(c, b, 2);
        LPM_CUDA(cudaMemcpyAsync(c.norms_host, c.norms, 4 * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
        if ((rc = sync(c)))
            return rc;
        const double bn = std::sqrt(c.norms_host[2]);
        if ((rc = recycle_dots(c, slots_du, R.count, b)))
            return rc;
        std::vector<double> coef(R.dots_h, R.dots_h + R.count);
        if (bn > 0.0 && std::isfinite(bn) && spd_solve(R.G, R.count, R.m, coef)) {
            adj_axpby(c, coef[0], slots_du[0], 0.0, R.x0);
            for (int j = 1; j < R.count; j++)
                adj_axpby(c, coef[j], slots_du[j], 1.0, R.x0);
            true_residual(c, R.x0, b, R.r0);
            LPM_CUDA(cudaMemcpyAsync(c.norms_host, c.norms, 4 * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
            if ((rc = sync(c)))
                return rc;
            const double rn = std::sqrt(c.norms_host[2]);
            if (c.trace)
                std::fprintf(stderr, "lpm: recycled guess from %d solutions: |r0| / |b| = %.3e\n", R.count,
                             rn / bn);
            if (std::isfinite(rn) && rn < 0.5 * bn) {
                guessed = true;
                const double target = solve_rtol(c) * bn;  // the solve's tolerance, relative to |b|
                if (rn <= target) {
                    LPM_CUDA(cudaMemcpyAsync(c.du, R.x0, sizeof(dvec4) * n, cudaMemcpyDeviceToDevice, c.stream));
                } else {
                    c.cg_rtol_now = target / rn;
                    rc = solve_plain(c, R.r0, st);
                    c.cg_rtol_now = rtol0;
                    if (rc)
                        return rc;
                    adj_axpby(c, 1.0, R.x0, 1.0, c.du);
                }
            }
        }
    }
    if (!guessed && (rc = solve_plain(c, b, st)))
        return rc;
    // store (du, b): the newest pair replaces the oldest
    const int slot = R.head;
    dvec4 *du_s = R.du + (size_t)slot * n, *b_s = R.b + (size_t)slot * n;
    LPM_CUDA(cudaMemcpyAsync(du_s, c.du, sizeof(dvec4) * n, cudaMemcpyDeviceToDevice, c.stream));
    LPM_CUDA(cudaMemcpyAsync(b_s, b, sizeof(dvec4) * n, cudaMemcpyDeviceToDevice, c.stream));
    R.count = std::min(R.count + 1, R.m);
    R.head = (R.head + 1) % R.m;
    for (int j = 0; j < R.count; j++) {
        slots_du[j] = R.du + (size_t)j * n;
        slots_b[j] = R.b + (size_t)j * n;
    }
    // G row and column of the new slot: du_slot . b_j and du_j . b_slot, symmetrised
    if ((rc = recycle_dots(c, slots_b, R.count, du_s)))
        return rc;
    std::vector<double> row(R.dots_h, R.dots_h + R.count);
    if ((rc = recycle_dots(c, slots_du, R.count, b_s)))
        return rc;
    for (int j = 0; j < R.count; j++) {
        const double g = 0.5 * (row[j] + R.dots_h[j]);
        R.G[(size_t)slot * R.m + j] = g;
        R.G[(size_t)j * R.m + slot] = g;
    }
    return LPM_OK;
}

int assemble(Ctx &c)
{
    const bool amg = c.opts.preconditioner == LPM_PRECOND_AMG && c.nspec == 0;
    // FP32 assembly accumulates a block's contributions in FP32, so a block
    // and its transpose, summed in different rows, differ by rounding.  The
    // multigrid PCG needs a symmetric operator: there the FP32 stiffness is
    // the rounding of the FP64 assembly (one rounding per value, and K_ij,
    // K_ji agree to FP64 rounding before it), as it is for the FP64 path's
    // smoother.  The FP64 values are then replaced by an exact copy of the
    // FP32 ones for the reliable updates (solve_amg).
    const bool fp32 = c.opts.precision == LPM_PREC_MIXED && !amg;
    const bool smooth32 = amg;
    int rc;
    if ((fp32 || smooth32) && (!c.Kf || c.kf_cap != c.nblk)) {
        if ((rc = dalloc(c.Kf, 9 * (size_t)c.nblk)))
            return rc;
        c.kf_cap = c.nblk;
    }
    if (!fp32 && (!c.Kd || c.kd_cap != c.nblk)) {
        if ((rc = dalloc(c.Kd, 9 * (size_t)c.nblk)))
            return rc;
        c.kd_cap = c.nblk;
    }
    launch_tangent_geometry(c);
    launch_assemble(c, fp32);
    c.k_version++;
    if (fp32)
        c.kf_version = c.k_version;
    if (smooth32) {
        launch_amg_stiffness32(c);
        c.kf_version = c.k_version;
    }
    c.have_K = true;
    return LPM_OK;
}

int prepare_preconditioner(Ctx &c)
{
    launch_block_jacobi(c, c.opts.precision == LPM_PREC_MIXED);
    return LPM_OK;
}

int force_eval(Ctx &c, int plmode)
{
    switch (plmode) {
    case LPM_PL_PREDICTOR:
        launch_predictor(c);
        break;
    case LPM_PL_ELASTIC:
        launch_elastic_force(c);
        copy_state(c, 2, 0);
        break;
    case LPM_PL_J2:
        launch_j2(c);
        launch_final_force(c);
        break;
    case LPM_PL_CP:
        if (!c.Cab)
            return fail(LPM_ERR_ARG, "crystal plasticity state not initialised");
        launch_cp(c);
        launch_final_force(c);
        break;
    default:
        return fail(LPM_ERR_ARG, "unsupported plmode");
    }
    switch_state(c, 2);
    return LPM_OK;
}

static int apply_bc(Ctx &c, int nbd, const lpm_disp_bc *dbc, int nbf, const lpm_force_bc *fbc)
{
    if (nbd > 0) {
        if (!dbc)
            return fail(LPM_ERR_ARG, "null displacement BC array");
        launch_apply_disp_bc(c, nbd, dbc);
    }
    if (nbf > 0) {
        if (!fbc)
            return fail(LPM_ERR_ARG, "null force BC array");
        // particle counts per BC type (src/boundary.c:53-58)
        std::vector<int> types(c.n), counts(nbf, 0);
        LPM_CUDA(cudaMemcpyAsync(types.data(), c.type, sizeof(int) * c.n, cudaMemcpyDeviceToHost, c.stream));
        int rc = sync(c);
        if (rc)
            return rc;
        for (int k = 0; k < nbf; k++)
            for (int i = 0; i < c.n; i++)
                counts[k] += (types[i] == fbc[k].type);
        launch_apply_force_bc(c, nbf, fbc, counts.data());
    }
    return LPM_OK;
}

// updateDamageGeneral for the context's model (src/constitutive.c:149-164):
// ductile nonlocal damage for J2, brittle bond breaking for elastic bonds,
// nothing for crystal plasticity.  `broken` is its return value.  Broken
// bonds are logged as (particle, partner) in the order the reference writes
// its bond file.
static int damage_update(Ctx &c, int &broken)
{
    Ctx::Damage &d = c.dmg;
    const int n = c.n;
    broken = 0;
    auto read_list = [&](int &k) -> int {
        LPM_CUDA(cudaMemcpyAsync(d.count_h, d.count, sizeof(int), cudaMemcpyDeviceToHost, c.stream));
        int rc = sync(c);
        if (rc)
            return rc;
        k = *d.count_h;
        return LPM_OK;
    };
    if (c.plmode == LPM_PL_J2) {
        // updateDuctileDamagePwiseNonlocal (src/constitutive.c:1757-1862)
        launch_dmg_nonlocal(c);
        launch_dmg_ductile_break(c);
        launch_dmg_ductile_w(c);
        int k = 0, rc = read_list(k);
        if (rc)
            return rc;
        if (k > 0) {
            std::vector<int> b(k);
            LPM_CUDA(cudaMemcpy(b.data(), d.list, sizeof(int) * k, cudaMemcpyDeviceToHost));
            // scan order of the reference: particle, then bond slot
            std::sort(b.begin(), b.end(), [n](int x, int y) {
                const int ix = x % n, iy = y % n;
                return ix != iy ? ix < iy : x / n < y / n;
            });
            for (int v : b) {
                const int i = v % n, j = v / n;
                d.log.push_back(i);
                d.log.push_back(c.hs.nbr[(size_t)i * LPM_NN + j]);
            }
        }
        broken = k;
    } else if (c.plmode == LPM_PL_ELASTIC) {
        // updateBrittleDamage (src/constitutive.c:1437-1527)
        launch_dmg_brittle_cand(c);
        int k = 0, rc = read_list(k);
        if (rc)
            return rc;
        if (k > 0) {
            std::vector<int> b(k);
            std::vector<double> v(k);
            LPM_CUDA(cudaMemcpy(b.data(), d.list, sizeof(int) * k, cudaMemcpyDeviceToHost));
            LPM_CUDA(cudaMemcpy(v.data(), d.lval, sizeof(double) * k, cudaMemcpyDeviceToHost));
            const std::vector<int> chosen = brittle_select(b, v, n, d.opts.nbreak);
            if (!chosen.empty()) {
                LPM_CUDA(cudaMemcpyAsync(d.list, chosen.data(), sizeof(int) * chosen.size(), cudaMemcpyHostToDevice,
                                         c.stream));
                launch_dmg_break_list(c, d.list, (int)chosen.size());
            }
            for (int v2 : chosen) {
                const int i = v2 % n, j = v2 / n;
                d.log.push_back(i);
                d.log.push_back(c.hs.nbr[(size_t)i * LPM_NN + j]);
            }
        }
        broken = k;
    }
    return sync(c);
}

// updateCrack (src/constitutive.c:1399-1434): bond forces scaled by
// damage_w, internal forces and residual, intact-bond counts, visual damage;
// then the stress weights of the intact bonds.
static int damage_crack(Ctx &c)
{
    launch_crack(c);
    launch_dmg_oppv(c);
    return sync(c);
}

// The damage stage after a converged Newton pass (src/lpmc_project.c:466-470).
static int damage_pass(Ctx &c, int &broken)
{
    int rc = damage_update(c, broken);
    return rc ? rc : damage_crack(c);
}

struct Timer {
    cudaEvent_t a, b;
    cudaStream_t s;
    Timer(cudaStream_t st) : s(st)
    {
        cudaEventCreate(&a);
        cudaEventCreate(&b);
        cudaEventRecord(a, s);
    }
    double stop()
    {
        float ms = 0.f;
        cudaEventRecord(b, s);
        cudaEventSynchronize(b);
        cudaEventElapsedTime(&ms, a, b);
        return ms;
    }
    ~Timer()
    {
        cudaEventDestroy(a);
        cudaEventDestroy(b);
    }
};

}  // namespace lpm

extern "C" {

void lpm_default_damage_opts(lpm_damage_opts *o)
{
    o->enabled = 0;
    o->length = 0.5;             // damage_L, src/lpmc_project.c:244
    o->threshold = 0.9;          // damage_threshold, :243
    o->triax_coeff = 0.0;        // damagec_A, :242
    o->critical_bstrain = 1e-2;  // critical_bstrain, :240
    o->nbreak = 20;              // nbreak, :239
    o->max_passes = 1000;
}

int lpm_set_damage(lpm_ctx *ctx, const lpm_damage_opts *o)
{
    if (!ctx || !o)
        return fail(LPM_ERR_ARG, "null argument");
    Ctx &c = ctx->c;
    if (!c.ready)
        return fail(LPM_ERR_ARG, "call lpm_init_state first");
    if (c.nspec > 0)
        return fail(LPM_ERR_ARG, "the damage stage is not available for batches");
    if (c.adj)
        return fail(LPM_ERR_ARG, "the damage stage is not available with the adjoint");
    if (!o->enabled) {
        if (c.dmg.on) {
            hvec<double> t((size_t)c.n * LPM_NN);
            to_slot_major(c.hs.oppv.data(), t.data(), c.n, LPM_NN);
            LPM_CUDA(cudaMemcpy(c.oppv, t.data(), t.size() * sizeof(double), cudaMemcpyHostToDevice));
        }
        free_damage(c);
        return LPM_OK;
    }
    if (!(o->length > 0.0) || !std::isfinite(o->threshold) || !std::isfinite(o->triax_coeff) ||
        !(o->critical_bstrain > 0.0) || o->nbreak < 0 || o->max_passes < 1)
        return fail(LPM_ERR_ARG, "invalid damage options");
    if ((long long)c.n * LPM_NN > 2147483647LL)
        return fail(LPM_ERR_ARG, "too many bonds for the damage stage");
    free_damage(c);
    Ctx::Damage &d = c.dmg;
    const int n = c.n;
    const size_t nb = (size_t)n * LPM_NN;
    const HostSetup &h = c.hs;
    int rc = 0;
    if ((rc = dalloc(d.brk, nb)) || (rc = dalloc(d.dw, nb)) || (rc = dalloc(d.D[0], nb)) || (rc = dalloc(d.D[1], nb)) ||
        (rc = dalloc(d.dnl[0], n)) || (rc = dalloc(d.dnl[1], n)) || (rc = dalloc(d.dvis, n)) ||
        (rc = dalloc(d.nbc, n)) || (rc = dalloc(d.opp, nb)) || (rc = dalloc(d.list, nb)) ||
        (rc = dalloc(d.lval, nb)) || (rc = dalloc(d.count, 1))) {
        free_damage(c);
        return rc;
    }
    LPM_CUDA(cudaMallocHost((void **)&d.count_h, sizeof(int)));
    // initMatrices (src/initialization.c:1176-1181): intact bonds, no damage
    {
        hvec<double> ones(nb);
#pragma omp parallel for schedule(static)
        for (long long k = 0; k < (long long)nb; k++)
            ones[k] = 1.0;
        LPM_CUDA(cudaMemcpy(d.brk, ones.data(), nb * sizeof(double), cudaMemcpyHostToDevice));
        LPM_CUDA(cudaMemcpy(d.dw, ones.data(), nb * sizeof(double), cudaMemcpyHostToDevice));
    }
    LPM_CUDA(cudaMemset(d.D[0], 0, nb * sizeof(double)));
    LPM_CUDA(cudaMemset(d.D[1], 0, nb * sizeof(double)));
    LPM_CUDA(cudaMemset(d.dnl[0], 0, n * sizeof(double)));
    LPM_CUDA(cudaMemset(d.dnl[1], 0, n * sizeof(double)));
    LPM_CUDA(cudaMemset(d.dvis, 0, n * sizeof(double)));
    LPM_CUDA(cudaMemcpy(d.nbc, c.nbv, n, cudaMemcpyDeviceToDevice));
    // slot of each bond's opposite bond (the first match, as the reference's
    // opp_flag search over the initial unit vectors)
    {
        hvec<int8_t> op(nb);
#pragma omp parallel for schedule(static)
        for (int i = 0; i < n; i++) {
            for (int j = 0; j < LPM_NN; j++) {
                int m0 = -1;
                if (j < h.nb[i]) {
                    const double *cj = &h.cs0[3 * ((size_t)i * LPM_NN + j)];
                    for (int m = 0; m < h.nb[i]; m++) {
                        const double *cm = &h.cs0[3 * ((size_t)i * LPM_NN + m)];
                        if (std::fabs(cm[0] + cj[0]) < 1e-6 && std::fabs(cm[1] + cj[1]) < 1e-6 &&
                            std::fabs(cm[2] + cj[2]) < 1e-6) {
                            m0 = m;
                            break;
                        }
                    }
                }
                op[(size_t)j * n + i] = (int8_t)m0;
            }
        }
        LPM_CUDA(cudaMemcpy(d.opp, op.data(), nb, cudaMemcpyHostToDevice));
    }
    // cell list of the initial positions for the nonlocal sum (cells >= 3 L,
    // coarsened when a fine grid would hold far more cells than particles)
    {
        double lo[3], hi[3];
        for (int k = 0; k < 3; k++)
            lo[k] = hi[k] = h.xyz[k];
        for (int i = 0; i < n; i++)
            for (int k = 0; k < 3; k++) {
                lo[k] = std::min(lo[k], h.xyz[3 * (size_t)i + k]);
                hi[k] = std::max(hi[k], h.xyz[3 * (size_t)i + k]);
            }
        double cs = 3.0 * o->length * 1.0001;
        int g[3];
        for (;;) {
            for (int k = 0; k < 3; k++)
                g[k] = (int)((hi[k] - lo[k]) / cs) + 1;
            if ((double)g[0] * g[1] * g[2] <= 8.0 * n + 4096.0)
                break;
            cs *= 1.5;
        }
        const size_t ncell = (size_t)g[0] * g[1] * g[2];
        std::vector<int> cell(n), start(ncell + 1, 0), order(n);
        for (int i = 0; i < n; i++) {
            int cc[3];
            for (int k = 0; k < 3; k++)
                cc[k] = std::min(g[k] - 1, (int)((h.xyz[3 * (size_t)i + k] - lo[k]) / cs));
            cell[i] = (int)(((size_t)cc[2] * g[1] + cc[1]) * g[0] + cc[0]);
            start[cell[i] + 1]++;
        }
        for (size_t q = 0; q < ncell; q++)
            start[q + 1] += start[q];
        std::vector<int> fill(start.begin(), start.end() - 1);
        for (int i = 0; i < n; i++)
            order[fill[cell[i]]++] = i;
        if ((rc = dalloc(d.cstart, ncell + 1)) || (rc = dalloc(d.corder, n))) {
            free_damage(c);
            return rc;
        }
        LPM_CUDA(cudaMemcpy(d.cstart, start.data(), (ncell + 1) * sizeof(int), cudaMemcpyHostToDevice));
        LPM_CUDA(cudaMemcpy(d.corder, order.data(), n * sizeof(int), cudaMemcpyHostToDevice));
        for (int k = 0; k < 3; k++) {
            d.g[k] = g[k];
            d.lo[k] = lo[k];
        }
        d.cs = cs;
    }
    d.opts = *o;
    d.on = 1;
    return LPM_OK;
}

int lpm_damage_log(lpm_ctx *ctx, int *pairs, int capacity, int *count)
{
    if (!ctx || !count)
        return fail(LPM_ERR_ARG, "null argument");
    Ctx &c = ctx->c;
    const int k = (int)(c.dmg.log.size() / 2);
    *count = k;
    if (pairs) {
        if (capacity < k)
            return fail(LPM_ERR_ARG, "damage log: buffer too small");
        std::memcpy(pairs, c.dmg.log.data(), sizeof(int) * 2 * (size_t)k);
    }
    return LPM_OK;
}

int lpm_damage_update(lpm_ctx *ctx, int *broken)
{
    if (!ctx || !broken)
        return fail(LPM_ERR_ARG, "null argument");
    Ctx &c = ctx->c;
    if (!c.dmg.on)
        return fail(LPM_ERR_ARG, "lpm_damage_update: the damage stage is off (lpm_set_damage)");
    *broken = 0;
    return damage_update(c, *broken);
}

int lpm_damage_crack(lpm_ctx *ctx)
{
    if (!ctx)
        return fail(LPM_ERR_ARG, "null argument");
    Ctx &c = ctx->c;
    if (!c.dmg.on)
        return fail(LPM_ERR_ARG, "lpm_damage_crack: the damage stage is off (lpm_set_damage)");
    return damage_crack(c);
}

int lpm_damage_brittle_select(const int *bonds, const double *strain, int k, int n, int nbreak, int *chosen,
                              int *nchosen)
{
    if (k < 0 || n <= 0 || nbreak < 0 || !nchosen || (k > 0 && (!bonds || !strain || !chosen)))
        return fail(LPM_ERR_ARG, "lpm_damage_brittle_select: bad argument");
    const std::vector<int> c = brittle_select(std::vector<int>(bonds, bonds + k),
                                              std::vector<double>(strain, strain + k), n, nbreak);
    std::copy(c.begin(), c.end(), chosen);
    *nchosen = (int)c.size();
    return LPM_OK;
}

int lpm_begin_step(lpm_ctx *ctx)
{
    if (!ctx || !ctx->c.ready)
        return fail(LPM_ERR_ARG, "call lpm_init_state first");
    Ctx &c = ctx->c;
    // src/lpmc_project.c:387-389: xyz_temp = xyz, F_temp = F
    LPM_CUDA(cudaMemcpyAsync(c.xyz_temp, c.xyz, sizeof(dvec4) * c.n, cudaMemcpyDeviceToDevice, c.stream));
    LPM_CUDA(cudaMemcpyAsync(c.F_prev, c.F, sizeof(double) * LPM_NN * c.n, cudaMemcpyDeviceToDevice, c.stream));
    return LPM_OK;
}

int lpm_assemble_stiffness(lpm_ctx *ctx)
{
    if (!ctx || !ctx->c.ready)
        return fail(LPM_ERR_ARG, "call lpm_init_state first");
    int rc = assemble(ctx->c);
    if (rc)
        return rc;
    return sync(ctx->c);
}

int lpm_apply_bc(lpm_ctx *ctx, int nbd, const lpm_disp_bc *dbc, int nbf, const lpm_force_bc *fbc)
{
    if (!ctx || !ctx->c.ready)
        return fail(LPM_ERR_ARG, "call lpm_init_state first");
    int rc = apply_bc(ctx->c, nbd, dbc, nbf, fbc);
    if (rc)
        return rc;
    return sync(ctx->c);
}

int lpm_compute_force(lpm_ctx *ctx, int plmode, double norms[2])
{
    if (!ctx || !ctx->c.ready)
        return fail(LPM_ERR_ARG, "call lpm_init_state first");
    Ctx &c = ctx->c;
    int rc = force_eval(c, plmode);
    if (rc)
        return rc;
    double a = 0, b = 0;
    if ((rc = read_norms(c, a, b)))
        return rc;
    if (norms) {
        norms[0] = a;
        norms[1] = b;
    }
    return LPM_OK;
}

int lpm_compute_strain(lpm_ctx *ctx)
{
    if (!ctx || !ctx->c.ready)
        return fail(LPM_ERR_ARG, "call lpm_init_state first");
    launch_strain(ctx->c);
    return sync(ctx->c);
}

int lpm_switch_state(lpm_ctx *ctx, int flag)
{
    if (!ctx || !ctx->c.ready || flag < 0 || flag > 2)
        return fail(LPM_ERR_ARG, "bad switchStateV flag or uninitialised context");
    switch_state(ctx->c, flag);
    return sync(ctx->c);
}

int lpm_solve(lpm_ctx *ctx, lpm_step_stats *st)
{
    if (!ctx || !ctx->c.ready || !ctx->c.have_K)
        return fail(LPM_ERR_ARG, "assemble the stiffness first");
    Ctx &c = ctx->c;
    int rc = prepare_preconditioner(c);
    if (rc)
        return rc;
    if ((rc = solve_device(c, c.res, st)))
        return rc;
    launch_add_du(c);
    return sync(c);
}

int lpm_solve_rhs(lpm_ctx *ctx, const double *b, double *x, lpm_step_stats *st)
{
    if (!ctx || !ctx->c.ready || !ctx->c.have_K || !b || !x)
        return fail(LPM_ERR_ARG, "assemble the stiffness first; b and x must be non-null");
    Ctx &c = ctx->c;
    int rc = upload_particles(c, c.b_d, b);
    if (rc)
        return rc;
    if ((rc = prepare_preconditioner(c)) || (rc = solve_device(c, c.b_d, st)))
        return rc;
    return download_particles(c, c.du, x);
}

}  // extern "C"

namespace lpm {

// Anderson acceleration of the modified-Newton fixed point u <- u + K^-1 r(u)
// (Walker & Ni, SIAM J. Numer. Anal. 49 (2011), type II, mixing 1): with
// f_k = K^-1 r(u_k) and the last h differences dF_j = f_{j+1} - f_j,
// dU_j = u_{j+1} - u_j, gamma = argmin |f_k - dF gamma| and
// u_{k+1} = u_k + f_k - sum_j gamma_j (dU_j + dF_j).
struct AndersonRun {
    int m = 0, hist = 0, head = 0;
    bool have_prev = false;
    std::vector<double> G;  // Gram matrix of the stored dF, m x m
};

static int anderson_prepare(Ctx &c, int m)
{
    Ctx::Anderson &A = c.acc;
    if (A.m == m && A.dU)
        return LPM_OK;
    free_anderson(c);
    int rc;
    const size_t n = c.n;
    if ((rc = dalloc(A.dU, m * n)) || (rc = dalloc(A.dF, m * n)) || (rc = dalloc(A.u_prev, n)) ||
        (rc = dalloc(A.f_prev, n)) || (rc = dalloc(A.dots, 16)))
        return rc;
    LPM_CUDA(cudaMallocHost((void **)&A.dots_h, 16 * sizeof(double)));
    A.m = m;
    return LPM_OK;
}

// small SPD solve (Cholesky) of (G + reg I) x = b, h <= 16; false if not SPD
static bool spd_solve(std::vector<double> G, int h, int ld, std::vector<double> &x)
{
    double dmax = 0.0;
    for (int i = 0; i < h; i++)
        dmax = std::max(dmax, G[(size_t)i * ld + i]);
    if (!(dmax > 0.0))
        return false;
    for (int i = 0; i < h; i++)
        G[(size_t)i * ld + i] += 1e-12 * dmax;
    std::vector<double> L((size_t)h * h, 0.0);
    for (int i = 0; i < h; i++)
        for (int j = 0; j <= i; j++) {
            double s = G[(size_t)i * ld + j];
            for (int k = 0; k < j; k++)
                s -= L[(size_t)i * h + k] * L[(size_t)j * h + k];
            if (i == j) {
                if (!(s > 0.0))
                    return false;
                L[(size_t)i * h + i] = std::sqrt(s);
            } else {
                L[(size_t)i * h + j] = s / L[(size_t)j * h + j];
            }
        }
    for (int i = 0; i < h; i++) {
        double s = x[i];
        for (int k = 0; k < i; k++)
            s -= L[(size_t)i * h + k] * x[k];
        x[i] = s / L[(size_t)i * h + i];
    }
    for (int i = h - 1; i >= 0; i--) {
        double s = x[i];
        for (int k = i + 1; k < h; k++)
            s -= L[(size_t)k * h + i] * x[k];
        x[i] = s / L[(size_t)i * h + i];
    }
    return true;
}

// apply the step from c.du (= f_k) at c.xyz (= u_k)
static int anderson_step(Ctx &c, AndersonRun &R)
{
    Ctx::Anderson &A = c.acc;
    const size_t n = c.n;
    const int m = R.m;
    auto dU = [&](int j) { return A.dU + (size_t)j * n; };
    auto dF = [&](int j) { return A.dF + (size_t)j * n; };
    if (R.have_prev) {
        const int slot = R.head;
        R.head = (R.head + 1) % m;
        R.hist = std::min(R.hist + 1, m);
        LPM_CUDA(cudaMemcpyAsync(dF(slot), c.du, n * sizeof(dvec4), cudaMemcpyDeviceToDevice, c.stream));
        adj_axpby(c, -1.0, A.f_prev, 1.0, dF(slot));
        LPM_CUDA(cudaMemcpyAsync(dU(slot), c.xyz, n * sizeof(dvec4), cudaMemcpyDeviceToDevice, c.stream));
        adj_axpby(c, -1.0, A.u_prev, 1.0, dU(slot));
        std::vector<const dvec4 *> ptr(R.hist);
        for (int j = 0; j < R.hist; j++)
            ptr[j] = dF(j);
        adj_multidot(c, R.hist, ptr.data(), dF(slot), A.dots);
        LPM_CUDA(cudaMemcpyAsync(A.dots_h, A.dots, R.hist * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
        int rc = sync(c);
        if (rc)
            return rc;
        for (int j = 0; j < R.hist; j++)
            R.G[(size_t)slot * m + j] = R.G[(size_t)j * m + slot] = A.dots_h[j];
    }
    LPM_CUDA(cudaMemcpyAsync(A.u_prev, c.xyz, n * sizeof(dvec4), cudaMemcpyDeviceToDevice, c.stream));
    LPM_CUDA(cudaMemcpyAsync(A.f_prev, c.du, n * sizeof(dvec4), cudaMemcpyDeviceToDevice, c.stream));
    R.have_prev = true;
    adj_axpby(c, 1.0, c.du, 1.0, c.xyz);
    if (R.hist == 0)
        return LPM_OK;
    std::vector<const dvec4 *> ptr(R.hist);
    for (int j = 0; j < R.hist; j++)
        ptr[j] = dF(j);
    adj_multidot(c, R.hist, ptr.data(), c.du, A.dots);
    LPM_CUDA(cudaMemcpyAsync(A.dots_h, A.dots, R.hist * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
    int rc = sync(c);
    if (rc)
        return rc;
    std::vector<double> g(A.dots_h, A.dots_h + R.hist);
    if (!spd_solve(R.G, R.hist, m, g)) {  // degenerate history: plain step, restart
        R.hist = 0;
        R.head = 0;
        return LPM_OK;
    }
    for (int j = 0; j < R.hist; j++) {
        adj_axpby(c, -g[j], dU(j), 1.0, c.xyz);
        adj_axpby(c, -g[j], dF(j), 1.0, c.xyz);
    }
    return LPM_OK;
}

}  // namespace lpm

extern "C" {

int lpm_load_step(lpm_ctx *ctx, int nbd, const lpm_disp_bc *dbc, int nbf, const lpm_force_bc *fbc,
                  lpm_step_stats *stats)
{
    if (!ctx || !ctx->c.ready)
        return fail(LPM_ERR_ARG, "call lpm_init_state first");
    Ctx &c = ctx->c;
    lpm_step_stats st;
    std::memset(&st, 0, sizeof(st));
    int rc = lpm_begin_step(ctx);
    if (rc)
        return rc;
    {
        Timer t(c.stream);
        if ((rc = assemble(c)))  // calcStiffness3DFiniteDifference (src/lpmc_project.c:396)
            return rc;
        st.ms_stiffness = t.stop();
    }
    if ((rc = apply_bc(c, nbd, dbc, nbf, fbc)))  // setDispBC / setForceBC (:402-403)
        return rc;
    if ((rc = prepare_preconditioner(c)))  // BC-modified block diagonal (:440)
        return rc;
    double res = 0, reac = 0;
    {
        Timer t(c.stream);
        if ((rc = force_eval(c, LPM_PL_PREDICTOR)) || (rc = read_norms(c, res, reac)))  // :405-414
            return rc;
        st.ms_force += t.stop();
    }
    double tolm = std::max(res, reac);
    st.res0 = res;
    st.reac0 = reac;
    c.trace_step++;
    if (c.trace)
        std::fprintf(stderr, "lpm: step %lld res0 %.6e reac0 %.6e target %.6e stiffness %.1f ms\n", c.trace_step,
                     res, reac, c.opts.newton_tol * tolm, st.ms_stiffness);
    int ni = 0;
    AndersonRun ar;
    if (c.opts.newton_accel > 0) {
        if ((rc = anderson_prepare(c, c.opts.newton_accel)))
            return rc;
        ar.m = c.opts.newton_accel;
        ar.G.assign((size_t)ar.m * ar.m, 0.0);
    }
    // One Newton pass without the damage stage; with it, a pass per
    // label_broken_bond re-entry (src/lpmc_project.c:405, :528-546).
    int passes = 0;
    for (;;) {
        double res_best = res, res_prev = res, eta_prev = c.opts.cg_forcing;
        int nip = 0;
        ar.hist = 0;  // a pass starts without acceleration history
        ar.head = 0;
        ar.have_prev = false;
        while (res > c.opts.newton_tol * tolm && nip < c.opts.newton_maxiter) {  // :424
            if (!std::isfinite(res)) {
                st.status |= LPM_STATUS_NAN;
                break;
            }
            switch_state(c, 0);  // :428
            if (c.opts.cg_forcing > 0.0) {
                // inexact Newton (Eisenstat & Walker 1996, choice 2): solve only as
                // far as the outer iteration can use
                const double emax = c.opts.cg_forcing;
                double eta = emax;
                if (nip > 0) {
                    const double q = res / res_prev;
                    eta = 0.9 * q * q;
                    if (0.9 * eta_prev * eta_prev > 0.1)
                        eta = std::max(eta, 0.9 * eta_prev * eta_prev);
                }
                eta = std::max(eta, 0.5 * c.opts.newton_tol * tolm / res);
                eta = std::min(std::max(eta, c.opts.cg_rtol), emax);
                c.cg_rtol_now = eta;
                eta_prev = eta;
            }
            res_prev = res;
            {
                Timer t(c.stream);
                rc = solve_device(c, c.res, &st);  // :449 solverCG
                c.cg_rtol_now = 0.0;
                if (rc)
                    return rc;
                if (ar.m > 0) {
                    if ((rc = anderson_step(c, ar)))
                        return rc;
                } else {
                    launch_add_du(c);
                }
                st.ms_solve += t.stop();
            }
            {
                Timer t(c.stream);
                if ((rc = force_eval(c, c.plmode)) || (rc = read_norms(c, res, reac)))  // :454-463
                    return rc;
                st.ms_force += t.stop();
            }
            if (c.trace)
                std::fprintf(stderr, "lpm: step %lld newton %d res %.6e ratio %.3e step totals: cg %d sweeps %d solve %.1f ms force %.1f ms\n",
                             c.trace_step, ni + nip + 1, res, res / std::max(res_best, 1e-300), st.cg_iters,
                             st.refine_iters, st.ms_solve, st.ms_force);
            if (ar.m > 0 && res > 10.0 * res_best) {  // safeguard: drop the history
                ar.hist = 0;
                ar.head = 0;
            }
            res_best = std::min(res_best, res);
            nip++;
        }
        if (nip >= c.opts.newton_maxiter && res > c.opts.newton_tol * tolm)
            st.status |= LPM_STATUS_NEWTON_MAXIT;
        ni += nip;
        passes++;
        if (!c.dmg.on) {
            switch_state(c, 1);  // :471
            break;
        }
        // damage stage: updateDamageGeneral, updateCrack, switchStateV(1) (:466-471)
        int broken = 0;
        if ((rc = damage_pass(c, broken)))
            return rc;
        st.bonds_broken += broken;
        switch_state(c, 1);
        if (c.trace)
            std::fprintf(stderr, "lpm: step %lld damage pass %d: %d bonds reached the criterion\n", c.trace_step,
                         passes, broken);
        if (broken <= 0 || passes >= c.dmg.opts.max_passes)
            break;
        // bonds broke: new stiffness, and the elastic-law bond forces of the
        // current configuration that the reference's finite-difference sweep
        // leaves behind (src/stiffness.c:390-418) start the next pass
        {
            Timer t(c.stream);
            if ((rc = assemble(c)) || (rc = prepare_preconditioner(c)))
                return rc;
            st.ms_stiffness += t.stop();
        }
        launch_elastic_force(c);
        if ((rc = read_norms(c, res, reac)))
            return rc;
        tolm = std::max(res, reac);
    }
    st.damage_passes = c.dmg.on ? passes : 0;
    LPM_CUDA(cudaMemcpyAsync(c.status_host, c.status, sizeof(int), cudaMemcpyDeviceToHost, c.stream));
    if ((rc = sync(c)))
        return rc;
    st.status |= *c.status_host;
    st.newton_iters = ni;
    st.res_final = res;
    if (stats)
        *stats = st;
    return LPM_OK;
}

}  // extern "C"

// ---- batched specimens ---------------------------------------------------------

namespace lpm {

static int alloc_batch(Ctx &c, const std::vector<int> &off)
{
    const int ns = (int)off.size() - 1, n = c.n;
    BatchCg &b = c.bcg;
    b.n = n;
    b.nspec = ns;
    b.nchunk = (n + BATCH_TPB - 1) / BATCH_TPB;
    std::vector<int> spec(n), seg(b.nchunk + 1, 0);
    for (int s = 0; s < ns; s++)
        for (int i = off[s]; i < off[s + 1]; i++)
            spec[i] = s;
    for (int ch = 0; ch < b.nchunk; ch++) {
        const int first = ch * BATCH_TPB, last = std::min(n, first + BATCH_TPB) - 1;
        seg[ch + 1] = seg[ch] + spec[last] - spec[first] + 1;
    }
    b.nseg = seg[b.nchunk];
    int rc = 0;
    int *spec_of = nullptr, *offd = nullptr, *segd = nullptr;
#define A_(p, cnt)            \
    if ((rc = dalloc(p, cnt))) \
        return rc;
    A_(spec_of, n) A_(offd, ns + 1) A_(segd, b.nchunk + 1)
    A_(b.rz, ns) A_(b.rz_old, ns) A_(b.rr, ns) A_(b.rr_max, ns) A_(b.tol2, ns) A_(b.alpha, ns) A_(b.beta, ns)
    A_(b.bscale, ns) A_(b.it, ns) A_(b.done, ns) A_(b.upd, ns) A_(b.nrel, ns) A_(b.active, ns)
    A_(b.partials, 3 * (size_t)b.nseg) A_(b.counter, 1) A_(b.all_done, 1) A_(b.act_chunk, b.nchunk)
    A_(b.n_act, 1)
    A_(c.bh.norms_d, 2 * ns) A_(c.bh.bs, n)
#undef A_
    b.spec_of = spec_of;
    b.off = offd;
    b.seg_base = segd;
    LPM_CUDA(cudaMemcpy(spec_of, spec.data(), sizeof(int) * n, cudaMemcpyHostToDevice));
    LPM_CUDA(cudaMemcpy(offd, off.data(), sizeof(int) * (ns + 1), cudaMemcpyHostToDevice));
    LPM_CUDA(cudaMemcpy(segd, seg.data(), sizeof(int) * (b.nchunk + 1), cudaMemcpyHostToDevice));
    BatchHost &h = c.bh;
    LPM_CUDA(cudaMallocHost((void **)&h.norms_h, 2 * ns * sizeof(double)));
    LPM_CUDA(cudaMallocHost((void **)&h.bscale_h, ns * sizeof(double)));
    LPM_CUDA(cudaMallocHost((void **)&h.active_h, ns * sizeof(int)));
    LPM_CUDA(cudaMallocHost((void **)&h.it_h, ns * sizeof(int)));
    LPM_CUDA(cudaMallocHost((void **)&h.done_h, ns * sizeof(int)));
    LPM_CUDA(cudaMallocHost((void **)&h.nrel_h, ns * sizeof(int)));
    LPM_CUDA(cudaMallocHost((void **)&h.all_done_h, sizeof(int)));
    h.nspec = ns;
    h.off = off;
    c.nspec = ns;
    return LPM_OK;
}

// per-specimen |residual| and |reaction| after a force evaluation
static int read_batch_norms(Ctx &c, std::vector<double> &res, std::vector<double> &reac)
{
    launch_bnorm(c);
    LPM_CUDA(cudaMemcpyAsync(c.bh.norms_h, c.bh.norms_d, 2 * c.nspec * sizeof(double), cudaMemcpyDeviceToHost,
                             c.stream));
    int rc = sync(c);
    if (rc)
        return rc;
    for (int s = 0; s < c.nspec; s++) {
        res[s] = std::sqrt(c.bh.norms_h[2 * s]);
        reac[s] = std::sqrt(c.bh.norms_h[2 * s + 1]);
    }
    return LPM_OK;
}

static void issue_batch_chunk(Ctx &c, bool k32, int chunk)
{
    launch_bcg_compact(c);
    for (int k = 0; k < chunk; k++)
        launch_bcg_iter(c, k32);
    if (k32)
        launch_bcg_reliable(c);
}

// One linear solve of every active specimen (bh.active_h, bh.bscale_h set by
// the caller): K du = residual on each specimen's unconstrained DOFs, du = 0
// for the others.  The iterations run as CUDA graphs of opts.check_every
// iterations (plus the reliable-update step with an FP32 matrix); the host
// reads one flag per graph launch.
static int batch_solve(Ctx &c, std::vector<lpm_step_stats> &st)
{
    const bool k32 = c.opts.precision == LPM_PREC_MIXED;
    const int ns = c.nspec, chunk = std::max(1, c.opts.check_every);
    BatchCg &b = c.bcg;
    BatchHost &h = c.bh;
    const double d2 = k32 ? c.opts.inner_rtol * c.opts.inner_rtol : 0.0;
    const bool same = b.maxit == c.opts.cg_maxiter && b.maxrel == c.opts.refine_maxiter && b.upd_delta2 == d2;
    b.maxit = c.opts.cg_maxiter;
    b.maxrel = c.opts.refine_maxiter;
    b.upd_delta2 = d2;
    LPM_CUDA(cudaMemcpyAsync(b.bscale, h.bscale_h, ns * sizeof(double), cudaMemcpyHostToDevice, c.stream));
    LPM_CUDA(cudaMemcpyAsync(b.active, h.active_h, ns * sizeof(int), cudaMemcpyHostToDevice, c.stream));
    launch_bcg_init(c, c.res);
    // the kernels take BatchCg by value: a graph is valid for the options it
    // was captured with
    if (h.graph && (!same || h.graph_chunk != chunk || h.graph_k32 != (int)k32)) {
        cudaGraphExecDestroy(h.graph);
        h.graph = nullptr;
    }
    bool use_graph = c.opts.use_graphs != 0;
    if (use_graph && !h.graph) {
        cudaGraph_t g;
        if (cudaStreamBeginCapture(c.stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
            use_graph = false;
        } else {
            issue_batch_chunk(c, k32, chunk);
            if (cudaStreamEndCapture(c.stream, &g) != cudaSuccess) {
                use_graph = false;
            } else {
                if (cudaGraphInstantiate(&h.graph, g, 0) != cudaSuccess) {
                    h.graph = nullptr;
                    use_graph = false;
                }
                cudaGraphDestroy(g);
                h.graph_chunk = chunk;
                h.graph_k32 = (int)k32;
            }
        }
        cudaGetLastError();
    }
    const long long max_chunks = (long long)c.opts.cg_maxiter / chunk + c.opts.refine_maxiter + 4;
    long long chunks = 0;
    for (;;) {
        if (use_graph) {
            LPM_CUDA(cudaGraphLaunch(h.graph, c.stream));
        } else {
            issue_batch_chunk(c, k32, chunk);
        }
        LPM_CUDA(cudaMemcpyAsync(h.all_done_h, b.all_done, sizeof(int), cudaMemcpyDeviceToHost, c.stream));
        int rc = sync(c);
        if (rc)
            return rc;
        chunks++;
        if (*h.all_done_h || chunks >= max_chunks)
            break;
    }
    launch_bcg_finish(c);
    LPM_CUDA(cudaMemcpyAsync(h.it_h, b.it, ns * sizeof(int), cudaMemcpyDeviceToHost, c.stream));
    LPM_CUDA(cudaMemcpyAsync(h.done_h, b.done, ns * sizeof(int), cudaMemcpyDeviceToHost, c.stream));
    LPM_CUDA(cudaMemcpyAsync(h.nrel_h, b.nrel, ns * sizeof(int), cudaMemcpyDeviceToHost, c.stream));
    int rc = sync(c);
    if (rc)
        return rc;
    for (int s = 0; s < ns; s++) {
        if (!h.active_h[s])
            continue;
        st[s].cg_iters += h.it_h[s];
        st[s].refine_iters += h.nrel_h[s];
        st[s].spmv_calls += h.it_h[s] + h.nrel_h[s];
        const int d = h.done_h[s];
        if (d == 2 || d == 0 || (k32 && d == 1))
            st[s].status |= LPM_STATUS_CG_MAXIT;
        if (d == 3)
            st[s].status |= LPM_STATUS_NAN;
    }
    return LPM_OK;
}

}  // namespace lpm

extern "C" {

int lpm_setup_batch(lpm_ctx *ctx, int lattice, double radius, int nspec, const double *boxes)
{
    if (!ctx || !boxes || nspec <= 0)
        return fail(LPM_ERR_ARG, "lpm_setup_batch: null argument or no specimen");
    Ctx &c = ctx->c;
    cudaSetDevice(c.device);
    free_batch(c);
    c.hs = HostSetup();
    std::vector<int> off;
    int rc = build_batch(c.hs, lattice, radius, nspec, boxes, off);
    if (rc < 0)
        return rc;
    rc = setup_common(c, true);
    if (rc < 0)
        return rc;
    if ((rc = alloc_batch(c, off)))
        return rc;
    return c.n;
}

int lpm_batch_offsets(const lpm_ctx *ctx, int *offsets)
{
    if (!ctx)
        return fail(LPM_ERR_ARG, "null context");
    const Ctx &c = ctx->c;
    if (offsets)
        for (int s = 0; s <= c.nspec; s++)
            offsets[s] = c.bh.off[s];
    return c.nspec;
}

int lpm_batch_load_step(lpm_ctx *ctx, int nbd, const lpm_disp_bc *dbc, lpm_step_stats *stats)
{
    if (!ctx || !ctx->c.ready)
        return fail(LPM_ERR_ARG, "call lpm_init_state first");
    Ctx &c = ctx->c;
    if (c.nspec <= 0)
        return fail(LPM_ERR_ARG, "lpm_batch_load_step: the context holds no batch (lpm_setup_batch)");
    if (nbd < 0 || (nbd > 0 && !dbc))
        return fail(LPM_ERR_ARG, "lpm_batch_load_step: bad displacement BC list");
    const int ns = c.nspec;
    std::vector<lpm_step_stats> st(ns);
    std::memset(st.data(), 0, sizeof(lpm_step_stats) * ns);
    int rc = lpm_begin_step(ctx);
    if (rc)
        return rc;
    double ms_stiff = 0, ms_solve = 0, ms_force = 0;
    {
        Timer t(c.stream);
        if ((rc = assemble(c)))
            return rc;
        ms_stiff = t.stop();
    }
    if ((rc = launch_disp_bc_batch(c, nbd, dbc)))
        return rc;
    if ((rc = prepare_preconditioner(c)))
        return rc;
    std::vector<double> res(ns), reac(ns), tolm(ns);
    std::vector<int> ni(ns, 0), live(ns, 1);
    {
        Timer t(c.stream);
        if ((rc = force_eval(c, LPM_PL_PREDICTOR)) || (rc = read_batch_norms(c, res, reac)))
            return rc;
        ms_force += t.stop();
    }
    for (int s = 0; s < ns; s++) {
        tolm[s] = std::max(res[s], reac[s]);
        st[s].res0 = res[s];
        st[s].reac0 = reac[s];
    }
    for (;;) {
        // a specimen leaves the Newton loop for the rest of the step once its
        // test of src/lpmc_project.c:424 fails
        bool any = false;
        for (int s = 0; s < ns; s++) {
            if (live[s] && !std::isfinite(res[s])) {
                st[s].status |= LPM_STATUS_NAN;
                live[s] = 0;
            }
            if (live[s] && !(res[s] > c.opts.newton_tol * tolm[s] && ni[s] < c.opts.newton_maxiter))
                live[s] = 0;
            c.bh.active_h[s] = live[s];
            c.bh.bscale_h[s] = live[s] ? 1.0 / res[s] : 0.0;
            any = any || live[s];
        }
        if (!any)
            break;
        switch_state(c, 0);
        {
            Timer t(c.stream);
            if ((rc = batch_solve(c, st)))
                return rc;
            launch_add_du(c);
            ms_solve += t.stop();
        }
        {
            Timer t(c.stream);
            if ((rc = force_eval(c, c.plmode)) || (rc = read_batch_norms(c, res, reac)))
                return rc;
            ms_force += t.stop();
        }
        for (int s = 0; s < ns; s++)
            if (live[s])
                ni[s]++;
    }
    switch_state(c, 1);
    LPM_CUDA(cudaMemcpyAsync(c.status_host, c.status, sizeof(int), cudaMemcpyDeviceToHost, c.stream));
    if ((rc = sync(c)))
        return rc;
    for (int s = 0; s < ns; s++) {
        if (ni[s] >= c.opts.newton_maxiter && res[s] > c.opts.newton_tol * tolm[s])
            st[s].status |= LPM_STATUS_NEWTON_MAXIT;
        st[s].status |= *c.status_host;
        st[s].newton_iters = ni[s];
        st[s].res_final = res[s];
        st[s].ms_stiffness = ms_stiff;
        st[s].ms_solve = ms_solve;
        st[s].ms_force = ms_force;
    }
    if (stats)
        std::memcpy(stats, st.data(), sizeof(lpm_step_stats) * ns);
    return LPM_OK;
}

// ---- data exchange -------------------------------------------------------------

int lpm_get(lpm_ctx *ctx, const char *name, void *dst, size_t bytes)
{
    if (!ctx || !name || !dst)
        return fail(LPM_ERR_ARG, "null argument");
    Ctx &c = ctx->c;
    const int n = c.n;
    const size_t nb = (size_t)n * LPM_NN;
    std::string nm(name);
    auto need = [&](size_t b) { return bytes >= b; };
    auto particles = [&](const dvec4 *src) -> int {
        if (!need(3 * n * sizeof(double)))
            return fail(LPM_ERR_ARG, nm + ": buffer too small");
        return download_particles(c, src, (double *)dst);
    };
    auto bond_d = [&](const double *src) -> int {
        if (!need(nb * sizeof(double)))
            return fail(LPM_ERR_ARG, nm + ": buffer too small");
        Staging sb(c, nb * sizeof(double));
        LPM_CUDA(cudaMemcpy(sb.p, src, nb * sizeof(double), cudaMemcpyDeviceToHost));
        from_slot_major((const double *)sb.p, (double *)dst, n, LPM_NN);
        return LPM_OK;
    };
    auto rows_d = [&](const double *src, int k) -> int {
        if (!need((size_t)k * n * sizeof(double)))
            return fail(LPM_ERR_ARG, nm + ": buffer too small");
        Staging sb(c, (size_t)k * n * sizeof(double));
        LPM_CUDA(cudaMemcpy(sb.p, src, (size_t)k * n * sizeof(double), cudaMemcpyDeviceToHost));
        from_slot_major((const double *)sb.p, (double *)dst, n, k);
        return LPM_OK;
    };
    LPM_CUDA(cudaStreamSynchronize(c.stream));
    if (nm == "xyz") return particles(c.xyz);
    if (nm == "xyz_initial") return particles(c.xyz0);
    if (nm == "xyz_temp") return particles(c.xyz_temp);
    if (nm == "Pin") return particles(c.Pin);
    if (nm == "Pex") return particles(c.Pex);
    if (nm == "residual") return particles(c.res);
    if (nm == "disp") return particles(c.du);
    if (nm == "F") return bond_d(c.F);
    if (nm == "F_temp") return bond_d(c.F_prev);
    if (nm == "dL") return bond_d(c.dL);
    if (nm == "csx") return bond_d(c.csx);
    if (nm == "csy") return bond_d(c.csy);
    if (nm == "csz") return bond_d(c.csz);
    if (nm == "Kn") return bond_d(c.Kn);
    if (nm == "Tv") return bond_d(c.Tv);
    if (nm == "distance_initial") return bond_d(c.L0);
    if (nm == "dLp") return bond_d(c.dLp[1]);
    if (nm == "dLp0") return bond_d(c.dLp[0]);
    if (nm == "dLp2" || nm == "dLp_trial") return bond_d(c.dLp[2]);
    if (nm == "J2_alpha") return rows_d(c.alpha[1], 1);
    if (nm == "J2_alpha0") return rows_d(c.alpha[0], 1);
    if (nm == "J2_alpha2") return rows_d(c.alpha[2], 1);
    if (nm == "J2_beta") return rows_d(c.beta[1], 6);
    if (nm == "J2_beta2") return rows_d(c.beta[2], 6);
    if (nm == "J2_dlambda") return rows_d(c.dlambda, 1);
    if (nm == "stress_tensor") return rows_d(c.stress, 6);
    if (nm == "strain_tensor") return rows_d(c.strain, 6);
    if (nm == "cp_gy" && c.nslip) return rows_d(c.gy[1], c.nslip);
    if (nm == "cp_gy2" && c.nslip) return rows_d(c.gy[2], c.nslip);
    if (nm == "cp_A_single" && c.nslip) return rows_d(c.As[1], c.nslip);
    if (nm == "cp_A_single2" && c.nslip) return rows_d(c.As[2], c.nslip);
    if (nm == "cp_A" && c.nslip) return rows_d(c.A[1], 1);
    if (nm == "cp_A2" && c.nslip) return rows_d(c.A[2], 1);
    if (nm == "cp_Cab" && c.nslip) return rows_d(c.Cab, c.nslip * c.nslip);
    if (nm == "neighbors" || nm == "nsign") {
        if (!need(nb * sizeof(int)))
            return fail(LPM_ERR_ARG, nm + ": buffer too small");
        std::memcpy(dst, (nm == "neighbors" ? c.hs.nbr : c.hs.shell).data(), nb * sizeof(int));
        return LPM_OK;
    }
    if (nm == "nb" || nm == "nb_conn") {
        if (!need(n * sizeof(int)))
            return fail(LPM_ERR_ARG, nm + ": buffer too small");
        std::memcpy(dst, (nm == "nb" ? c.hs.nb : c.hs.nconn).data(), n * sizeof(int));
        return LPM_OK;
    }
    if (nm == "type" || nm == "pl_flag") {
        if (!need(n * sizeof(int)))
            return fail(LPM_ERR_ARG, nm + ": buffer too small");
        LPM_CUDA(cudaMemcpy(dst, nm == "type" ? c.type : c.pl_flag, n * sizeof(int), cudaMemcpyDeviceToHost));
        return LPM_OK;
    }
    if (nm == "conn") {
        if (!need((size_t)n * 61 * sizeof(int)))
            return fail(LPM_ERR_ARG, nm + ": buffer too small");
        std::memcpy(dst, c.hs.conn.data(), (size_t)n * 61 * sizeof(int));
        return LPM_OK;
    }
    if (nm == "K_pointer") {
        if (c.hs.kp1.empty())
            return fail(LPM_ERR_ARG, "K_pointer: this batch exceeds the reference's int32 CSR offsets");
        if (!need((size_t)(n + 1) * 2 * sizeof(int)))
            return fail(LPM_ERR_ARG, nm + ": buffer too small");
        int *o = (int *)dst;
        for (int i = 0; i <= n; i++) {
            o[2 * i] = c.hs.kp0[i];
            o[2 * i + 1] = c.hs.kp1[i];
        }
        return LPM_OK;
    }
    if (nm == "dispBC_index") {
        if (!need(3 * (size_t)n * sizeof(int)))
            return fail(LPM_ERR_ARG, nm + ": buffer too small");
        std::vector<uint8_t> m(n);
        LPM_CUDA(cudaMemcpy(m.data(), c.mask, n, cudaMemcpyDeviceToHost));
        int *o = (int *)dst;
        for (int i = 0; i < n; i++)
            for (int d = 0; d < 3; d++)
                o[3 * i + d] = (m[i] >> d) & 1;
        return LPM_OK;
    }
    if (nm == "cs_initial") {
        if (!need(nb * 3 * sizeof(double)))
            return fail(LPM_ERR_ARG, nm + ": buffer too small");
        std::memcpy(dst, c.hs.cs0.data(), nb * 3 * sizeof(double));
        return LPM_OK;
    }
    if (nm == "damage_broken" || nm == "damage_w" || nm == "damage_D" || nm == "damage_nonlocal" ||
        nm == "damage_D0" || nm == "damage_nonlocal0" || nm == "damage_visual" || nm == "nb_current") {
        if (!c.dmg.on)
            return fail(LPM_ERR_ARG, nm + ": the damage stage is off (lpm_set_damage)");
        if (nm == "damage_broken") return bond_d(c.dmg.brk);
        if (nm == "damage_w") return bond_d(c.dmg.dw);
        if (nm == "damage_D") return bond_d(c.dmg.D[1]);
        if (nm == "damage_D0") return bond_d(c.dmg.D[0]);
        if (nm == "damage_nonlocal") return rows_d(c.dmg.dnl[1], 1);
        if (nm == "damage_nonlocal0") return rows_d(c.dmg.dnl[0], 1);
        if (nm == "damage_visual") return rows_d(c.dmg.dvis, 1);
        if (!need(n * sizeof(int)))
            return fail(LPM_ERR_ARG, nm + ": buffer too small");
        std::vector<int8_t> t(n);
        LPM_CUDA(cudaMemcpy(t.data(), c.dmg.nbc, n, cudaMemcpyDeviceToHost));
        int *o = (int *)dst;
        for (int i = 0; i < n; i++)
            o[i] = t[i];
        return LPM_OK;
    }
    return fail(LPM_ERR_ARG, "unknown array name: " + nm);
}

int lpm_set(lpm_ctx *ctx, const char *name, const void *src, size_t bytes)
{
    if (!ctx || !name || !src)
        return fail(LPM_ERR_ARG, "null argument");
    Ctx &c = ctx->c;
    const int n = c.n;
    const size_t nb = (size_t)n * LPM_NN;
    std::string nm(name);
    LPM_CUDA(cudaStreamSynchronize(c.stream));
    auto particles = [&](dvec4 *d) -> int {
        if (bytes < 3 * (size_t)n * sizeof(double))
            return fail(LPM_ERR_ARG, nm + ": buffer too small");
        return upload_particles(c, d, (const double *)src);
    };
    auto bond_d = [&](double *d) -> int {
        if (bytes < nb * sizeof(double))
            return fail(LPM_ERR_ARG, nm + ": buffer too small");
        Staging sb(c, nb * sizeof(double));
        to_slot_major((const double *)src, (double *)sb.p, n, LPM_NN);
        LPM_CUDA(cudaMemcpy(d, sb.p, nb * sizeof(double), cudaMemcpyHostToDevice));
        return LPM_OK;
    };
    auto rows_d = [&](double *d, int k) -> int {
        if (bytes < (size_t)k * n * sizeof(double))
            return fail(LPM_ERR_ARG, nm + ": buffer too small");
        Staging sb(c, (size_t)k * n * sizeof(double));
        to_slot_major((const double *)src, (double *)sb.p, n, k);
        LPM_CUDA(cudaMemcpy(d, sb.p, (size_t)k * n * sizeof(double), cudaMemcpyHostToDevice));
        return LPM_OK;
    };
    if (nm == "xyz") return particles(c.xyz);
    if (nm == "xyz_temp") return particles(c.xyz_temp);
    if (nm == "Pex") return particles(c.Pex);
    if (nm == "residual") return particles(c.res);
    if (nm == "dL") return bond_d(c.dL);
    if (nm == "F") return bond_d(c.F);
    if (nm == "F_temp") return bond_d(c.F_prev);
    if (nm == "csx") return bond_d(c.csx);
    if (nm == "csy") return bond_d(c.csy);
    if (nm == "csz") return bond_d(c.csz);
    if (nm == "dLp0") return bond_d(c.dLp[0]);
    if (nm == "dLp" || nm == "dLp1") return bond_d(c.dLp[1]);
    if (nm == "J2_alpha0") return rows_d(c.alpha[0], 1);
    if (nm == "J2_alpha" || nm == "J2_alpha1") return rows_d(c.alpha[1], 1);
    if (nm == "J2_beta0") return rows_d(c.beta[0], 6);
    if (nm == "J2_beta" || nm == "J2_beta1") return rows_d(c.beta[1], 6);
    if (nm == "cp_gy0" && c.nslip) return rows_d(c.gy[0], c.nslip);
    if (nm == "cp_A_single0" && c.nslip) return rows_d(c.As[0], c.nslip);
    if (nm == "cp_A0" && c.nslip) return rows_d(c.A[0], 1);
    if ((nm == "cp_gy" || nm == "cp_gy1") && c.nslip) return rows_d(c.gy[1], c.nslip);
    if ((nm == "cp_A_single" || nm == "cp_A_single1") && c.nslip) return rows_d(c.As[1], c.nslip);
    if ((nm == "cp_A" || nm == "cp_A1") && c.nslip) return rows_d(c.A[1], 1);
    if (nm == "J2_dlambda") return rows_d(c.dlambda, 1);
    if (nm == "damage_broken" || nm == "damage_w" || nm == "damage_D" || nm == "damage_D0" ||
        nm == "damage_nonlocal" || nm == "damage_nonlocal0") {
        if (!c.dmg.on)
            return fail(LPM_ERR_ARG, nm + ": the damage stage is off (lpm_set_damage)");
        if (nm == "damage_broken") return bond_d(c.dmg.brk);
        if (nm == "damage_w") return bond_d(c.dmg.dw);
        if (nm == "damage_D") return bond_d(c.dmg.D[1]);
        if (nm == "damage_D0") return bond_d(c.dmg.D[0]);
        if (nm == "damage_nonlocal") return rows_d(c.dmg.dnl[1], 1);
        return rows_d(c.dmg.dnl[0], 1);
    }
    if (nm == "dispBC_index") {
        if (bytes < 3 * (size_t)n * sizeof(int))
            return fail(LPM_ERR_ARG, nm + ": buffer too small");
        const int *m = (const int *)src;
        std::vector<uint8_t> t(n);
        for (int i = 0; i < n; i++)
            t[i] = (uint8_t)((m[3 * i] ? 1 : 0) | (m[3 * i + 1] ? 2 : 0) | (m[3 * i + 2] ? 4 : 0));
        LPM_CUDA(cudaMemcpy(c.mask, t.data(), n, cudaMemcpyHostToDevice));
        return LPM_OK;
    }
    return fail(LPM_ERR_ARG, "unknown or read-only array name: " + nm);
}

int lpm_export_upper_csr(lpm_ctx *ctx, double *Kg, int *IK, int *JK, long long *nnz)
{
    if (!ctx)
        return fail(LPM_ERR_ARG, "null context");
    Ctx &c = ctx->c;
    const HostSetup &h = c.hs;
    const int n = c.n;
    if (h.kp1.empty())
        return fail(LPM_ERR_ARG, "export_upper_csr: this batch exceeds the reference's int32 CSR offsets");
    if (nnz)
        *nnz = h.kp1[n];
    if (!Kg && !IK && !JK)
        return LPM_OK;
    // layout of calcStiffness3DFiniteDifference (src/stiffness.c:431-515)
    if (!Kg) {
        export_upper_csr_host<double>(h, nullptr, Kg, IK, JK);
        return LPM_OK;
    }
    if (!c.have_K)
        return fail(LPM_ERR_ARG, "no stiffness assembled");
    const size_t cnt = 9 * (size_t)c.nblk;
    if (c.opts.precision == LPM_PREC_FP64) {
        Staging sb(c, cnt * sizeof(double));
        LPM_CUDA(cudaMemcpy(sb.p, c.Kd, cnt * sizeof(double), cudaMemcpyDeviceToHost));
        export_upper_csr_host<double>(h, (const double *)sb.p, Kg, IK, JK);
    } else {
        // FP32 values, widened exactly to double as they are written out
        Staging sb(c, cnt * sizeof(float));
        LPM_CUDA(cudaMemcpy(sb.p, c.Kf, cnt * sizeof(float), cudaMemcpyDeviceToHost));
        export_upper_csr_host<float>(h, (const float *)sb.p, Kg, IK, JK);
    }
    return LPM_OK;
}

int lpm_spmv(lpm_ctx *ctx, const double *x, double *y)
{
    if (!ctx || !ctx->c.have_K || !x || !y)
        return fail(LPM_ERR_ARG, "assemble the stiffness first; x and y must be non-null");
    Ctx &c = ctx->c;
    int rc = upload_particles(c, c.b_d, x);
    if (rc)
        return rc;
    if (c.opts.precision == LPM_PREC_FP64) {
        launch_spmv_d(c, c.b_d, c.q_d, false, false);
        return download_particles(c, c.q_d, y);
    }
    // FP32 product of an FP32 copy of x
    std::vector<float4> xf(c.n);
    for (int i = 0; i < c.n; i++)
        xf[i] = make_float4((float)x[3 * i], (float)x[3 * i + 1], (float)x[3 * i + 2], 0.f);
    LPM_CUDA(cudaMemcpy(c.p_f, xf.data(), sizeof(float4) * c.n, cudaMemcpyHostToDevice));
    launch_spmv_f(c, c.p_f, c.q_f, false, false);
    LPM_CUDA(cudaMemcpyAsync(xf.data(), c.q_f, sizeof(float4) * c.n, cudaMemcpyDeviceToHost, c.stream));
    if ((rc = sync(c)))
        return rc;
    for (int i = 0; i < c.n; i++) {
        y[3 * i] = xf[i].x;
        y[3 * i + 1] = xf[i].y;
        y[3 * i + 2] = xf[i].z;
    }
    return LPM_OK;
}

}  // extern "C"

// ---- autotuner -----------------------------------------------------------------

namespace lpm {

// cached CUDA graphs hold launch shapes: drop them when the shapes change
static void drop_graphs(Ctx &c)
{
    if (c.graph_fp64)
        cudaGraphExecDestroy(c.graph_fp64);
    if (c.graph_fp32)
        cudaGraphExecDestroy(c.graph_fp32);
    c.graph_fp64 = c.graph_fp32 = nullptr;
    if (c.bh.graph)
        cudaGraphExecDestroy(c.bh.graph);
    c.bh.graph = nullptr;
}

static void fill_tuning(const Ctx &c, lpm_tuning *t)
{
    t->spmv_variant = c.tune.spmv_variant;
    t->spmv_lanes = spmv_variant_lanes(c.tune.spmv_variant);
    t->spmv_blocks = spmv_variant_blocks(c.tune.spmv_variant);
    t->spmv_per_sm = c.tune.spmv_per_sm;
    t->cg_per_sm = c.tune.vec_per_sm;
    t->smooth_lanes =
        c.tune.smooth_stream ? 16 : (c.tune.smooth_variant == 1 ? 8 : (c.tune.smooth_variant == 2 ? 4 : 16));
    t->smooth_ms = 0.0;
    t->diff_stream = c.tune.diff_stream;
    t->smooth_stream = c.tune.smooth_stream;
}

}  // namespace lpm

extern "C" {

int lpm_get_tuning(const lpm_ctx *ctx, lpm_tuning *t)
{
    if (!ctx || !t)
        return fail(LPM_ERR_ARG, "null argument");
    fill_tuning(ctx->c, t);
    t->spmv_ms = t->spmv_ms_default = 0.0;
    return LPM_OK;
}

int lpm_set_tuning(lpm_ctx *ctx, const lpm_tuning *t)
{
    if (!ctx || !t)
        return fail(LPM_ERR_ARG, "null argument");
    auto ok_grid = [](int v) { return v >= 1 && v <= TUNE_MAX_PER_SM; };
    if (t->spmv_variant < 0 || t->spmv_variant > 3 || !ok_grid(t->spmv_per_sm) || !ok_grid(t->cg_per_sm) ||
        t->diff_stream < 0 || t->diff_stream > 3)
        return fail(LPM_ERR_ARG, "lpm_set_tuning: variant 0..3, blocks per SM 1.." +
                                     std::to_string(TUNE_MAX_PER_SM) + ", diff_stream 0..3");
    Ctx &c = ctx->c;
    if (t->smooth_stream < 0 || t->smooth_stream > 3)
        return fail(LPM_ERR_ARG, "lpm_set_tuning: smooth_stream 0..3");
    if (t->diff_stream > 0 && c.stream_stages[t->diff_stream - 1] < 2)
        return fail(LPM_ERR_ARG, "lpm_set_tuning: the streamed product's stages do not fit in shared memory");
    if (t->smooth_stream > 0 && c.smooth_stages[t->smooth_stream - 1] < 2)
        return fail(LPM_ERR_ARG, "lpm_set_tuning: the streamed smoother's stages do not fit in shared memory");
    c.tune.diff_stream = t->diff_stream;
    c.tune.smooth_stream = t->smooth_stream;
    c.tune.spmv_variant = t->spmv_variant;
    c.tune.spmv_per_sm = t->spmv_per_sm;
    c.tune.vec_per_sm = t->cg_per_sm;
    drop_graphs(c);
    return LPM_OK;
}

int lpm_autotune(lpm_ctx *ctx, lpm_tuning *out)
{
    if (!ctx || !ctx->c.have_K)
        return fail(LPM_ERR_ARG, "lpm_autotune: assemble the stiffness first");
    Ctx &c = ctx->c;
    const bool k32 = c.opts.precision == LPM_PREC_MIXED;
    const bool vec64 = !k32 || c.nspec > 0 || c.opts.mixed_vectors == 64 || c.vec64_fallback;
    const bool timed = c.time_spmv;
    c.time_spmv = false;
    // the multigrid path's products: the difference form under mixed
    // precision, and the level-0 smoother in either precision
    const bool amg = c.opts.preconditioner == LPM_PRECOND_AMG && c.nspec == 0 && c.amg && c.Kh &&
                     c.kh_version == c.kf_version;
    const bool diff = amg && k32 && c.krs_version == c.kf_version;
    // the difference-form product is timed in the form the PCG launches (with
    // p.q), on scratch CG scalars whose solve is never done
    CgScalars *sc_run = c.sc, *sc_tune = nullptr;
    if (diff) {
        int arc = dalloc(sc_tune, 1);
        if (arc)
            return arc;
    }
    auto spmv = [&]() {
        if (!k32) {
            launch_spmv_d(c, c.p_d, c.q_d, true, false);
        } else if (diff) {
            c.sc = sc_tune;
            launch_spmv_diff(c, c.q_d, true);
            c.sc = sc_run;
        } else if (vec64)
            launch_spmv_fx(c, c.p_d, c.q_d, true, false);
        else
            launch_spmv_f(c, c.p_f, c.q_f, true, false);
    };
    cudaEvent_t a, b;
    LPM_CUDA(cudaEventCreate(&a));
    LPM_CUDA(cudaEventCreate(&b));
    const int reps = 10;
    auto time_it = [&](auto &&launch, double &ms) -> int {
        for (int r = 0; r < 2; r++)
            launch();
        LPM_CUDA(cudaEventRecord(a, c.stream));
        for (int r = 0; r < reps; r++)
            launch();
        LPM_CUDA(cudaEventRecord(b, c.stream));
        LPM_CUDA(cudaEventSynchronize(b));
        float f = 0.f;
        LPM_CUDA(cudaEventElapsedTime(&f, a, b));
        ms = f / reps;
        return LPM_OK;
    };
    const Tune keep = c.tune;
    const int grids[] = {2, 4, 8, 16};
    Tune best = keep;
    double best_ms = 1e30, def_ms = 0.0;
    int rc = LPM_OK;
    c.tune.diff_stream = 0;
    for (int v = 0; v < 4 && !rc; v++)
        for (int g : grids) {
            c.tune.spmv_variant = v;
            c.tune.spmv_per_sm = g;
            double ms = 0.0;
            if ((rc = time_it(spmv, ms)))
                break;
            if (v == 0 && g == 8)
                def_ms = ms;
            if (ms < best_ms) {
                best_ms = ms;
                best.spmv_variant = v;
                best.spmv_per_sm = g;
            }
        }
    // the streamed difference-form product with 1 and 2 CTAs per SM
    best.diff_stream = 0;
    if (diff && !rc) {
        for (int ds = 1; ds <= 3 && !rc; ds++) {
            if (c.stream_stages[ds - 1] < 2)
                continue;
            c.tune.diff_stream = ds;
            double ms = 0.0;
            if ((rc = time_it(spmv, ms)))
                break;
            if (c.trace)
                std::fprintf(stderr, "lpm: autotune streamed product, variant %d, %d stages: %.4f ms "
                                     "(best so far %.4f ms)\n",
                             ds, c.stream_stages[ds - 1], ms, best_ms);
            if (ms < best_ms) {
                best_ms = ms;
                best.diff_stream = ds;
            }
        }
        c.tune.diff_stream = 0;
        if (!rc) {
            LPM_CUDA(cudaMemcpyAsync(c.status_host, c.status, sizeof(int), cudaMemcpyDeviceToHost, c.stream));
            if (!(rc = sync(c)) && (*c.status_host & LPM_STATUS_DEVICE_WAIT))
                rc = fail(LPM_ERR_DEVICE, "lpm_autotune: a wait of the streamed product ran out");
        }
    }
    double best_smooth = 0.0;
    if (amg && !rc) {
        best_smooth = 1e30;
        c.tune.smooth_stream = 0;
        for (int v = 0; v < 3 && !rc; v++) {
            c.tune.smooth_variant = v;
            double ms = 0.0;
            if ((rc = time_it([&]() { launch_amg_smoother_pass(c); }, ms)))
                break;
            if (ms < best_smooth) {
                best_smooth = ms;
                best.smooth_variant = v;
            }
        }
        // the streamed smoother with 1 and 2 CTAs per SM
        best.smooth_stream = 0;
        for (int ss = 1; ss <= 3 && !rc; ss++) {
            if (c.smooth_stages[ss - 1] < 2)
                continue;
            c.tune.smooth_stream = ss;
            double ms = 0.0;
            if ((rc = time_it([&]() { launch_amg_smoother_pass(c); }, ms)))
                break;
            if (c.trace)
                std::fprintf(stderr, "lpm: autotune streamed smoother, variant %d, %d stages: %.4f ms "
                                     "(best so far %.4f ms)\n",
                             ss, c.smooth_stages[ss - 1], ms, best_smooth);
            if (ms < best_smooth) {
                best_smooth = ms;
                best.smooth_stream = ss;
            }
        }
        c.tune.smooth_stream = 0;
        if (!rc) {
            LPM_CUDA(cudaMemcpyAsync(c.status_host, c.status, sizeof(int), cudaMemcpyDeviceToHost, c.stream));
            if (!(rc = sync(c)) && (*c.status_host & LPM_STATUS_DEVICE_WAIT))
                rc = fail(LPM_ERR_DEVICE, "lpm_autotune: a wait of the streamed smoother ran out");
        }
    }
    double best_vec = 1e30;
    for (int g : grids) {
        if (rc)
            break;
        c.tune.vec_per_sm = g;
        double ms = 0.0;
        if ((rc = time_it([&]() { launch_norm2(c, c.p_d, 3); }, ms)))
            break;
        if (ms < best_vec) {
            best_vec = ms;
            best.vec_per_sm = g;
        }
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    c.time_spmv = timed;
    if (sc_tune) {
        cudaStreamSynchronize(c.stream);
        dfree(sc_tune);
    }
    if (rc) {
        c.tune = keep;
        return rc;
    }
    c.tune = best;
    drop_graphs(c);
    if (out) {
        fill_tuning(c, out);
        out->spmv_ms = best_ms;
        out->spmv_ms_default = def_ms;
        out->smooth_ms = best_smooth;
    }
    return sync(c);
}

int lpm_spmv_timing(lpm_ctx *ctx, double *avg_ms, long long *count, int reset)
{
    if (!ctx)
        return fail(LPM_ERR_ARG, "null context");
    Ctx &c = ctx->c;
    if (avg_ms)
        *avg_ms = c.spmv_count ? c.spmv_ms_sum / c.spmv_count : 0.0;
    if (count)
        *count = c.spmv_count;
    if (reset) {
        c.spmv_ms_sum = 0;
        c.spmv_count = 0;
    }
    // reset > 1 also switches sampling on (reset == 2) or off (reset == 3)
    if (reset == 2)
        c.time_spmv = true;
    if (reset == 3)
        c.time_spmv = false;
    return LPM_OK;
}

double lpm_spmv_bytes(const lpm_ctx *ctx, int precision)
{
    if (!ctx)
        return 0.0;
    const Ctx &c = ctx->c;
    const double sv = precision == LPM_PREC_MIXED ? 4.0 : 8.0;
    // nnzb (9 s_v + 4) + 4 (N_b + 1) + 2 * 3 N_b * s_x
    return (double)c.nblk_real * (9.0 * sv + 4.0) + 4.0 * (c.n + 1) + 2.0 * 3.0 * c.n * sv;
}

}  // extern "C"
