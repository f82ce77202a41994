// Output writers in the reference's file formats (src/data_handler.c):
// writeDump (LAMMPS dump, :42-85), writeDisp (:278-306), writeReaction
// (:309-335), writeStress (:110-135) and writeStrain (:137-162).
//
// lpm_format_* write from host arrays in the reference's per-particle layout;
// the lpm_write_* entry points take a context: writeDump copies the device
// buffers into pinned host memory on the context's stream and formats the
// file on a host thread, so the next load step's kernels run while the file
// is written (lpm_write_wait joins it).  The text is byte-identical to the
// reference's for the same data: same printf formats and the same
// arithmetic (compiled without floating-point contraction).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <thread>
#include <vector>
#include "lpm_internal.h"

namespace lpm {

namespace {

constexpr double OUT_EPS = 1e-6;  // EPS of include/lpm.h:42

// computeStress (src/lpm_basic.c:102-111): equivalent and mean stress,
// triaxiality (kept at its previous value, here 0, when sigma_eq <= EPS)
void stress_scalars(const double *st, double &seq, double &sm, double &tri)
{
    seq = 0.0;
    for (int j = 0; j < 6; j++) {
        if (j < 3)
            seq += st[j] * st[j];
        else
            seq += 2.0 * st[j] * st[j];
    }
    seq = std::sqrt(3.0 / 2.0 * seq);
    sm = 1.0 / 3.0 * (st[0] + st[1] + st[2]);
    tri = seq > OUT_EPS ? sm / seq : 0.0;
}

int comp_of(char c) { return c == 'x' ? 0 : (c == 'y' ? 1 : 2); }

}  // namespace

// Snapshot of the arrays writeDump reads, in the reference's layout.
struct DumpData {
    int n = 0, plmode = 0, nslip = 0;
    double box[6] = {0, 0, 0, 0, 0, 0};
    std::vector<int> type, pl_flag;
    std::vector<double> xyz, xyz0, stress, alpha, As, A;  // n x 3, n x 3, n x 6, n, n x nslip, n
};

int format_dump(const char *path, int step, char flag, const DumpData &d)
{
    FILE *f = std::fopen(path, flag == 's' ? "w+" : "a+");
    if (!f)
        return fail(LPM_ERR_ARG, std::string("cannot open ") + path);
    std::fprintf(f, "ITEM: TIMESTEP\n");
    std::fprintf(f, "%d\n", step);
    std::fprintf(f, "ITEM: NUMBER OF ATOMS\n");
    std::fprintf(f, "%d\n", d.n);
    std::fprintf(f, "ITEM: BOX BOUNDS pp pp pp\n");
    std::fprintf(f, "%8.8f %8.8f\n", d.box[0], d.box[1]);
    std::fprintf(f, "%8.8f %8.8f\n", d.box[2], d.box[3]);
    std::fprintf(f, "%8.8f %8.8f\n", d.box[4], d.box[5]);
    if (d.plmode == 1) {
        static const int ms[8] = {1, 4, 10, 19, 9, 14, 17, 22};  // slip systems shown by the reference
        std::fprintf(f, "ITEM: ATOMS id type x y z dx dy dz s11 s22 s33 s23 s13 s12 gam11 gam12 gam13 gam14 gam21 "
                        "gam22 gam23 gam24 pl gam_total\n");
        for (int i = 0; i < d.n; i++) {
            const double *x = &d.xyz[3 * (size_t)i], *x0 = &d.xyz0[3 * (size_t)i], *s = &d.stress[6 * (size_t)i];
            double g[8];
            for (int k = 0; k < 8; k++)
                g[k] = ms[k] < d.nslip ? d.As[(size_t)i * d.nslip + ms[k]] : 0.0;
            std::fprintf(f,
                         "%d %d %.4e %.4e %.4e %.4e %.4e %.4e %.4e %.4e %.4e %.4e %.4e %.4e %.4e %.4e %.4e %.4e "
                         "%.4e %.4e %.4e %.4e %d %.4e\n",
                         i, d.type[i], x[0], x[1], x[2], x[0] - x0[0], x[1] - x0[1], x[2] - x0[2], s[0], s[1], s[2],
                         s[3], s[4], s[5], g[0], g[1], g[2], g[3], g[4], g[5], g[6], g[7], d.pl_flag[i], d.A[i]);
        }
    } else {
        std::fprintf(f, "ITEM: ATOMS id type x y z dx dy dz s11 s22 s33 s23 s13 s12 stress_eq strain_eq stress_m "
                        "stress_tri damage_local damage_nonlocal pl damage\n");
        for (int i = 0; i < d.n; i++) {
            const double *x = &d.xyz[3 * (size_t)i], *x0 = &d.xyz0[3 * (size_t)i], *s = &d.stress[6 * (size_t)i];
            double seq, sm, tri;
            stress_scalars(s, seq, sm, tri);
            // damage is not modelled: damage_local, damage_nonlocal and damage_visual are 0
            std::fprintf(f,
                         "%d %d %.4e %.4e %.4e %.4e %.4e %.4e %.4e %.4e %.4e %.4e %.4e %.4e %.4e %.4e %.4e %.4e "
                         "%.4e %.4e %d %.4e\n",
                         i, d.type[i], x[0], x[1], x[2], x[0] - x0[0], x[1] - x0[1], x[2] - x0[2], s[0], s[1], s[2],
                         s[3], s[4], s[5], seq, d.alpha[i], sm, tri, 0.0, 0.0, d.pl_flag[i], 0.0);
        }
    }
    std::fclose(f);
    return LPM_OK;
}

}  // namespace lpm

using namespace lpm;

extern "C" {

int lpm_format_dump(const char *path, int step, char flag, int n, const double box[6], int plmode, const int *type,
                    const double *xyz, const double *xyz0, const double *stress, const double *alpha,
                    const int *pl_flag, const double *cp_As, int nslip, const double *cp_A)
{
    if (!path || n < 0 || !box || !type || !xyz || !xyz0 || !stress || !pl_flag ||
        (plmode == 1 ? (!cp_As || !cp_A) : !alpha))
        return fail(LPM_ERR_ARG, "lpm_format_dump: null argument");
    DumpData d;
    d.n = n;
    d.plmode = plmode;
    d.nslip = nslip;
    std::memcpy(d.box, box, sizeof(d.box));
    d.type.assign(type, type + n);
    d.pl_flag.assign(pl_flag, pl_flag + n);
    d.xyz.assign(xyz, xyz + 3 * (size_t)n);
    d.xyz0.assign(xyz0, xyz0 + 3 * (size_t)n);
    d.stress.assign(stress, stress + 6 * (size_t)n);
    if (plmode == 1) {
        d.As.assign(cp_As, cp_As + (size_t)n * nslip);
        d.A.assign(cp_A, cp_A + n);
    } else {
        d.alpha.assign(alpha, alpha + n);
    }
    return format_dump(path, step, flag, d);
}

int lpm_format_disp(const char *path, char c, int t1, int tstep, int n, const int *type, const double *xyz,
                    const double *xyz0)
{
    if (!path || !type || !xyz || !xyz0)
        return fail(LPM_ERR_ARG, "lpm_format_disp: null argument");
    FILE *f = std::fopen(path, "a+");
    if (!f)
        return fail(LPM_ERR_ARG, std::string("cannot open ") + path);
    const int k = comp_of(c);
    int num = 0;
    double p = 0, p0 = 0;
    for (int i = 0; i < n; i++)
        if (type[i] == t1) {
            p += xyz[3 * (size_t)i + k];
            p0 += xyz0[3 * (size_t)i + k];
            num++;
        }
    std::fprintf(f, "%d %8.8e\n", tstep, (p - p0) / num);
    std::fclose(f);
    return LPM_OK;
}

int lpm_format_reaction(const char *path, char c, int t1, int tstep, int n, int nn, const int *type, const int *nb,
                        const double *csx, const double *csy, const double *csz, const double *F)
{
    if (!path || !type || !nb || !csx || !csy || !csz || !F)
        return fail(LPM_ERR_ARG, "lpm_format_reaction: null argument");
    FILE *f = std::fopen(path, "a+");
    if (!f)
        return fail(LPM_ERR_ARG, std::string("cannot open ") + path);
    double force = 0.;
    for (int i = 0; i < n; i++)
        if (type[i] == t1)
            for (int j = 0; j < nb[i]; j++) {
                const size_t b = (size_t)i * nn + j;
                if (c == 'x')
                    force += -csx[b] * F[b];
                else if (c == 'y')
                    force += -csy[b] * F[b];
                else if (c == 'z')
                    force += -csz[b] * F[b];
            }
    std::fprintf(f, "%d %8.8e \n", tstep, force);
    std::fclose(f);
    return LPM_OK;
}

static int format_type_average(const char *path, int t1, int tstep, int n, const int *type, const double *v)
{
    FILE *f = std::fopen(path, "a+");
    if (!f)
        return fail(LPM_ERR_ARG, std::string("cannot open ") + path);
    int num = 0;
    double ave[6] = {0, 0, 0, 0, 0, 0};
    for (int i = 0; i < n; i++)
        if (type[i] == t1) {
            num++;
            for (int j = 0; j < 6; j++)
                ave[j] += v[6 * (size_t)i + j];
        }
    std::fprintf(f, "%d ", tstep);
    for (int j = 0; j < 6; j++)
        std::fprintf(f, "%.6e ", ave[j] / num);
    std::fprintf(f, "\n");
    std::fclose(f);
    return LPM_OK;
}

int lpm_format_stress(const char *path, int t1, int tstep, int n, const int *type, const double *stress)
{
    if (!path || !type || !stress)
        return fail(LPM_ERR_ARG, "lpm_format_stress: null argument");
    return format_type_average(path, t1, tstep, n, type, stress);
}

// writeStrain (src/data_handler.c:137-162): same layout as writeStress
int lpm_format_strain(const char *path, int t1, int tstep, int n, const int *type, const double *strain)
{
    if (!path || !type || !strain)
        return fail(LPM_ERR_ARG, "lpm_format_strain: null argument");
    return format_type_average(path, t1, tstep, n, type, strain);
}

}  // extern "C"

// ---- context entry points -------------------------------------------------------

namespace lpm {

struct AsyncWriter {
    std::thread th;
    bool running = false;
    int rc = LPM_OK;
    std::string err;
    int cap = 0, cap_ns = 0;
    int *type = nullptr, *pl = nullptr;
    dvec4 *xyz = nullptr, *xyz0 = nullptr;
    double *stress = nullptr, *alpha = nullptr, *As = nullptr, *A = nullptr;
    cudaEvent_t ev = nullptr;
};

static void free_pinned(AsyncWriter &w)
{
    void *ps[] = {w.type, w.pl, w.xyz, w.xyz0, w.stress, w.alpha, w.As, w.A};
    for (void *p : ps)
        if (p)
            cudaFreeHost(p);
    w.type = w.pl = nullptr;
    w.xyz = w.xyz0 = nullptr;
    w.stress = w.alpha = w.As = w.A = nullptr;
    w.cap = w.cap_ns = 0;
}

static int writer_join(AsyncWriter &w)
{
    if (w.running) {
        w.th.join();
        w.running = false;
    }
    const int rc = w.rc;
    w.rc = LPM_OK;
    if (rc)
        return fail(rc, w.err);
    return LPM_OK;
}

void free_writer(Ctx &c)
{
    if (!c.writer)
        return;
    writer_join(*c.writer);
    free_pinned(*c.writer);
    if (c.writer->ev)
        cudaEventDestroy(c.writer->ev);
    delete c.writer;
    c.writer = nullptr;
}

}  // namespace lpm

extern "C" {

int lpm_write_wait(lpm_ctx *ctx)
{
    if (!ctx)
        return fail(LPM_ERR_ARG, "null context");
    return ctx->c.writer ? writer_join(*ctx->c.writer) : LPM_OK;
}

int lpm_write_dump(lpm_ctx *ctx, const char *path, int step, char flag, const double box[6])
{
    if (!ctx || !path || !box || !ctx->c.ready)
        return fail(LPM_ERR_ARG, "lpm_write_dump: bad argument or uninitialised context");
    Ctx &c = ctx->c;
    if (!c.writer)
        c.writer = new AsyncWriter();
    AsyncWriter &w = *c.writer;
    int rc = writer_join(w);
    if (rc)
        return rc;
    const int n = c.n, ns = c.nslip;
    if (w.cap < n || w.cap_ns < ns) {
        free_pinned(w);
        LPM_CUDA(cudaMallocHost((void **)&w.type, n * sizeof(int)));
        LPM_CUDA(cudaMallocHost((void **)&w.pl, n * sizeof(int)));
        LPM_CUDA(cudaMallocHost((void **)&w.xyz, n * sizeof(dvec4)));
        LPM_CUDA(cudaMallocHost((void **)&w.xyz0, n * sizeof(dvec4)));
        LPM_CUDA(cudaMallocHost((void **)&w.stress, 6 * (size_t)n * sizeof(double)));
        LPM_CUDA(cudaMallocHost((void **)&w.alpha, n * sizeof(double)));
        LPM_CUDA(cudaMallocHost((void **)&w.A, n * sizeof(double)));
        LPM_CUDA(cudaMallocHost((void **)&w.As, std::max(1, ns) * (size_t)n * sizeof(double)));
        w.cap = n;
        w.cap_ns = ns;
    }
    if (!w.ev)
        LPM_CUDA(cudaEventCreateWithFlags(&w.ev, cudaEventDisableTiming));
    cudaStream_t s = c.stream;
    const bool cp = c.plmode == LPM_PL_CP && ns > 0;
    LPM_CUDA(cudaMemcpyAsync(w.type, c.type, n * sizeof(int), cudaMemcpyDeviceToHost, s));
    LPM_CUDA(cudaMemcpyAsync(w.pl, c.pl_flag, n * sizeof(int), cudaMemcpyDeviceToHost, s));
    LPM_CUDA(cudaMemcpyAsync(w.xyz, c.xyz, n * sizeof(dvec4), cudaMemcpyDeviceToHost, s));
    LPM_CUDA(cudaMemcpyAsync(w.xyz0, c.xyz0, n * sizeof(dvec4), cudaMemcpyDeviceToHost, s));
    LPM_CUDA(cudaMemcpyAsync(w.stress, c.stress, 6 * (size_t)n * sizeof(double), cudaMemcpyDeviceToHost, s));
    LPM_CUDA(cudaMemcpyAsync(w.alpha, c.alpha[1], n * sizeof(double), cudaMemcpyDeviceToHost, s));
    if (cp) {
        LPM_CUDA(cudaMemcpyAsync(w.As, c.As[1], (size_t)ns * n * sizeof(double), cudaMemcpyDeviceToHost, s));
        LPM_CUDA(cudaMemcpyAsync(w.A, c.A[1], n * sizeof(double), cudaMemcpyDeviceToHost, s));
    }
    LPM_CUDA(cudaEventRecord(w.ev, s));
    const std::string p(path);
    double bx[6];
    std::memcpy(bx, box, sizeof(bx));
    const int dev = c.device, plmode = cp ? 1 : 0;
    w.running = true;
    w.th = std::thread([&w, p, step, flag, bx, n, ns, dev, plmode]() {
        cudaSetDevice(dev);
        cudaError_t e = cudaEventSynchronize(w.ev);
        if (e != cudaSuccess) {
            w.rc = LPM_ERR_CUDA;
            w.err = std::string("lpm_write_dump: ") + cudaGetErrorString(e);
            return;
        }
        // device layouts -> the reference's per-particle layout
        DumpData d;
        d.n = n;
        d.plmode = plmode;
        d.nslip = ns;
        std::memcpy(d.box, bx, sizeof(d.box));
        d.type.assign(w.type, w.type + n);
        d.pl_flag.assign(w.pl, w.pl + n);
        d.xyz.resize(3 * (size_t)n);
        d.xyz0.resize(3 * (size_t)n);
        d.stress.resize(6 * (size_t)n);
        for (int i = 0; i < n; i++) {
            d.xyz[3 * (size_t)i] = w.xyz[i].x;
            d.xyz[3 * (size_t)i + 1] = w.xyz[i].y;
            d.xyz[3 * (size_t)i + 2] = w.xyz[i].z;
            d.xyz0[3 * (size_t)i] = w.xyz0[i].x;
            d.xyz0[3 * (size_t)i + 1] = w.xyz0[i].y;
            d.xyz0[3 * (size_t)i + 2] = w.xyz0[i].z;
            for (int k = 0; k < 6; k++)
                d.stress[6 * (size_t)i + k] = w.stress[(size_t)k * n + i];
        }
        if (plmode == 1) {
            d.As.resize((size_t)n * ns);
            for (int i = 0; i < n; i++)
                for (int m = 0; m < ns; m++)
                    d.As[(size_t)i * ns + m] = w.As[(size_t)m * n + i];
            d.A.assign(w.A, w.A + n);
        } else {
            d.alpha.assign(w.alpha, w.alpha + n);
        }
        w.rc = format_dump(p.c_str(), step, flag, d);
        if (w.rc)
            w.err = g_err;
    });
    return LPM_OK;
}

int lpm_write_disp(lpm_ctx *ctx, const char *path, char c, int t1, int tstep)
{
    if (!ctx || !ctx->c.ready)
        return fail(LPM_ERR_ARG, "lpm_write_disp: uninitialised context");
    const int n = ctx->c.n;
    std::vector<int> type(n);
    std::vector<double> xyz(3 * (size_t)n), xyz0(3 * (size_t)n);
    int rc;
    if ((rc = lpm_get(ctx, "type", type.data(), type.size() * sizeof(int))) ||
        (rc = lpm_get(ctx, "xyz", xyz.data(), xyz.size() * sizeof(double))) ||
        (rc = lpm_get(ctx, "xyz_initial", xyz0.data(), xyz0.size() * sizeof(double))))
        return rc;
    return lpm_format_disp(path, c, t1, tstep, n, type.data(), xyz.data(), xyz0.data());
}

int lpm_write_reaction(lpm_ctx *ctx, const char *path, char c, int t1, int tstep)
{
    if (!ctx || !ctx->c.ready)
        return fail(LPM_ERR_ARG, "lpm_write_reaction: uninitialised context");
    const int n = ctx->c.n, nn = LPM_NN;
    std::vector<int> type(n), nb(n);
    std::vector<double> cs[3], F((size_t)n * nn);
    const char *names[3] = {"csx", "csy", "csz"};
    int rc;
    if ((rc = lpm_get(ctx, "type", type.data(), type.size() * sizeof(int))) ||
        (rc = lpm_get(ctx, "nb", nb.data(), nb.size() * sizeof(int))) ||
        (rc = lpm_get(ctx, "F", F.data(), F.size() * sizeof(double))))
        return rc;
    for (int k = 0; k < 3; k++) {
        cs[k].resize((size_t)n * nn);
        if ((rc = lpm_get(ctx, names[k], cs[k].data(), cs[k].size() * sizeof(double))))
            return rc;
    }
    return lpm_format_reaction(path, c, t1, tstep, n, nn, type.data(), nb.data(), cs[0].data(), cs[1].data(),
                               cs[2].data(), F.data());
}

int lpm_write_strain(lpm_ctx *ctx, const char *path, int t1, int tstep)
{
    if (!ctx || !ctx->c.ready)
        return fail(LPM_ERR_ARG, "lpm_write_strain: uninitialised context");
    const int n = ctx->c.n;
    std::vector<int> type(n);
    std::vector<double> e(6 * (size_t)n);
    int rc;
    if ((rc = lpm_get(ctx, "type", type.data(), type.size() * sizeof(int))) ||
        (rc = lpm_get(ctx, "strain_tensor", e.data(), e.size() * sizeof(double))))
        return rc;
    return lpm_format_strain(path, t1, tstep, n, type.data(), e.data());
}

int lpm_write_stress(lpm_ctx *ctx, const char *path, int t1, int tstep)
{
    if (!ctx || !ctx->c.ready)
        return fail(LPM_ERR_ARG, "lpm_write_stress: uninitialised context");
    const int n = ctx->c.n;
    std::vector<int> type(n);
    std::vector<double> st(6 * (size_t)n);
    int rc;
    if ((rc = lpm_get(ctx, "type", type.data(), type.size() * sizeof(int))) ||
        (rc = lpm_get(ctx, "stress_tensor", st.data(), st.size() * sizeof(double))))
        return rc;
    return lpm_format_stress(path, t1, tstep, n, type.data(), st.data());
}

}  // extern "C"
