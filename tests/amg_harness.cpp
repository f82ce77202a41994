// Test helper: runs lpm::amg_build on a stiffness given in the device
// block-CSR layout (binary files in a directory) and writes the hierarchy
// back as binary files, for tests/test_amg_setup.py.  When DIR holds r.bin
// (a level-0 vector, 4 doubles per particle), it also applies the device's
// V-cycle to it: the launch sequence of launch_amg_vcycle (k_amg.cu), each
// kernel's rows computed one after another by the same per-row functions
// (amg_rows.h), all in FP64 (z.bin) and all in FP32 as the device runs it
// (z32.bin; the device keeps the level-0 smoother's stiffness as scaled FP16
// values and multiplies them in FP32, which changes the values, not the index
// arithmetic this emulation checks).
//   amg_harness DIR AGG_SPACING [SWEEPS]
#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>
#include "amg.h"
#include "amg_rows.h"

template <typename T>
static std::vector<T> rd(const std::string &path, size_t count)
{
    std::vector<T> v(count);
    FILE *f = std::fopen(path.c_str(), "rb");
    if (!f || std::fread(v.data(), sizeof(T), count, f) != count) {
        std::fprintf(stderr, "cannot read %s\n", path.c_str());
        std::exit(2);
    }
    std::fclose(f);
    return v;
}

template <typename V>
static void wr(const std::string &path, const V &v)
{
    FILE *f = std::fopen(path.c_str(), "wb");
    std::fwrite(v.data(), sizeof(v[0]), v.size(), f);
    std::fclose(f);
}

static void wr_bsr(FILE *f, const std::string &p, const lpm::Bsr &A)
{
    std::fprintf(f, " %d %d %d %d", A.nbr, A.nbc, A.R, A.C);
    wr(p + "_ptr.bin", A.ptr);
    wr(p + "_col.bin", A.col);
    wr(p + "_val.bin", A.val);
}

template <typename T>
struct Level0 {
    int n;
    const uint8_t *mask;
    const long long *rowoff;
    const int *npad, *cols;
    const T *Pinv;
};

// one launch of k_amg_k0, rows one after another (V: stiffness values and
// products, T: vectors and epilogue)
template <typename V, typename T, typename O>
static void k0(const Level0<T> &z0, const V *val, int mode, T omega, const T *x, const T *b, O *out)
{
    for (int row = 0; row < z0.n; row++) {
        V y0 = 0, y1 = 0, y2 = 0;
        lpm::k0_row_partial<V, T>(z0.rowoff, z0.npad, z0.cols, val, x, row, 0, 1, y0, y1, y2);
        T P[9];
        for (int k = 0; k < 9; k++)
            P[k] = z0.Pinv[(size_t)k * z0.n + row];
        lpm::k0_epilogue<T, O>(mode, row, z0.mask[row], P, omega, x, b, out, (T)y0, (T)y1, (T)y2);
    }
}

template <int R, int C, int MODE, typename T>
static void bsr(int nbr, const lpm::Bsr &M, const T *val, const T *x, int SX, T *out, int SY, const T *b = nullptr,
                const T *dinv = nullptr, T omega = 0)
{
    for (int row = 0; row < nbr; row++) {
        T y[R] = {};
        lpm::bsr_row_partial<R, C, T>(M.ptr.data(), M.col.data(), val, x, SX, row, 0, 1, y);
        lpm::bsr_epilogue<R, MODE, T>(row, y, x, SX, out, SY, b, dinv, omega);
    }
}

template <typename T, typename S>
static std::vector<T> conv(const S &v) { return std::vector<T>(v.begin(), v.end()); }

template <typename BT, typename OT>
static void dense(const lpm::AmgHierarchy &H, const BT *b, OT *out, int B, int S)
{
    for (int k = 0; k < H.coarse_n; k++)
        out[(size_t)(k / B) * S + k % B] = (OT)lpm::dense_row_partial<BT>(H.coarse_n, H.coarse_inv.data(), b, B, S, k,
                                                                          0, 1);
}

// z = V(r), in the order and with the buffers of launch_amg_vcycle (nu
// sweeps before and after each coarse correction); V: stiffness values, T:
// everything else (the device runs V = T = float)
template <typename V, typename T>
static void vcycle(const lpm::AmgHierarchy &H, const Level0<T> &z0, const V *val, const double *r, double *z, int nu)
{
    const int L = (int)H.levels.size();
    if (L == 0) {
        dense<double, double>(H, r, z, 3, 4);
        return;
    }
    const size_t n4 = 4 * (size_t)z0.n;
    std::vector<T> bt(n4, T(0)), xa(n4, T(0)), qa(n4, T(0));
    std::vector<std::vector<T>> b(L), x(L), y(L), P(L), Pt(L), A(L), D(L);
    for (int l = 0; l < L; l++) {
        const lpm::AmgLevel &v = H.levels[l];
        P[l] = conv<T>(v.P.val);
        Pt[l] = conv<T>(v.Pt.val);
        if (l > 0) {
            const size_t m = 6 * (size_t)v.nblock;
            b[l].assign(m, T(0));
            x[l].assign(m, T(0));
            y[l].assign(m, T(0));
            A[l] = conv<T>(v.A.val);
            D[l] = conv<T>(v.Dinv);
        }
    }
    std::vector<T> cb(H.coarse_n), cx(H.coarse_n);
    for (int l = 0; l < L; l++) {
        const lpm::AmgLevel &v = H.levels[l];
        const T om = (T)v.omega;
        T *bnext = (l + 1 < L) ? b[l + 1].data() : cb.data();
        if (l == 0) {
            T *it = xa.data(), *ot = qa.data();
            for (int i = 0; i < z0.n; i++)
                lpm::jacobi0_row<T, T, double>(z0.n, i, z0.mask[i], z0.Pinv, om, r, bt.data(), it);
            for (int s = 1; s < nu; s++) {
                k0<V, T, T>(z0, val, lpm::SM_SMOOTH, om, it, bt.data(), ot);
                std::swap(it, ot);
            }
            k0<V, T, T>(z0, val, lpm::SM_RESID, om, it, bt.data(), ot);
            bsr<6, 3, lpm::BM_SET, T>(v.P.nbc, v.Pt, Pt[l].data(), ot, 4, bnext, 6);
        } else {
            T *it = x[l].data(), *ot = y[l].data();
            for (int i = 0; i < v.nblock; i++)
                lpm::jacobi6_row<T>(i, D[l].data(), om, b[l].data(), it);
            for (int s = 1; s < nu; s++) {
                bsr<6, 6, lpm::BM_SMOOTH, T>(v.nblock, v.A, A[l].data(), it, 6, ot, 6, b[l].data(), D[l].data(), om);
                std::swap(it, ot);
            }
            bsr<6, 6, lpm::BM_RESID, T>(v.nblock, v.A, A[l].data(), it, 6, ot, 6, b[l].data());
            bsr<6, 6, lpm::BM_SET, T>(v.P.nbc, v.Pt, Pt[l].data(), ot, 6, bnext, 6);
        }
    }
    dense<T, T>(H, cb.data(), cx.data(), 6, 6);
    for (int l = L - 1; l >= 0; l--) {
        const lpm::AmgLevel &v = H.levels[l];
        const T om = (T)v.omega;
        const T *e = (l + 1 < L) ? y[l + 1].data() : cx.data();
        if (l == 0) {
            T *it = (nu % 2 == 1) ? xa.data() : qa.data(), *ot = (nu % 2 == 1) ? qa.data() : xa.data();
            bsr<3, 6, lpm::BM_ADD, T>(v.nblock, v.P, P[l].data(), e, 6, it, 4);
            for (int s = 0; s < nu; s++) {
                if (s == nu - 1) {
                    k0<V, T, double>(z0, val, lpm::SM_SMOOTH, om, it, bt.data(), z);
                } else {
                    k0<V, T, T>(z0, val, lpm::SM_SMOOTH, om, it, bt.data(), ot);
                    std::swap(it, ot);
                }
            }
        } else {
            T *it = (nu % 2 == 1) ? x[l].data() : y[l].data(), *ot = (nu % 2 == 1) ? y[l].data() : x[l].data();
            bsr<6, 6, lpm::BM_ADD, T>(v.nblock, v.P, P[l].data(), e, 6, it, 6);
            for (int s = 0; s < nu; s++) {
                bsr<6, 6, lpm::BM_SMOOTH, T>(v.nblock, v.A, A[l].data(), it, 6, ot, 6, b[l].data(), D[l].data(), om);
                std::swap(it, ot);
            }
        }
    }
}

int main(int argc, char **argv)
{
    if (argc < 3)
        return 2;
    const std::string d(argv[1]);
    int n = 0;
    {
        FILE *f = std::fopen((d + "/n.txt").c_str(), "r");
        if (!f || std::fscanf(f, "%d", &n) != 1)
            return 2;
        std::fclose(f);
    }
    auto xyz = rd<double>(d + "/xyz.bin", 3 * (size_t)n);
    auto mask = rd<uint8_t>(d + "/mask.bin", n);
    auto rowoff = rd<long long>(d + "/rowoff.bin", (size_t)n + 1);
    auto npad = rd<int>(d + "/npad.bin", n);
    auto nconn = rd<int>(d + "/nconn.bin", n);
    auto cols = rd<int>(d + "/cols.bin", (size_t)rowoff[n]);
    auto val = rd<double>(d + "/val.bin", 9 * (size_t)rowoff[n]);
    lpm::AmgInput in;
    in.n = n;
    in.xyz = xyz.data();
    in.mask = mask.data();
    in.rowoff = rowoff.data();
    in.npad = npad.data();
    in.nconn = nconn.data();
    in.cols = cols.data();
    in.val = val.data();
    std::vector<int> group;
    if (FILE *fg = std::fopen((d + "/group.bin").c_str(), "rb")) {
        std::fclose(fg);
        group = rd<int>(d + "/group.bin", n);
        in.group = group.data();
    }
    lpm::AmgOptions opt;
    opt.agg_spacing = std::atof(argv[2]);
    lpm::AmgHierarchy H;
    const auto t0 = std::chrono::steady_clock::now();
    const int L = lpm::amg_build(in, H, opt);
    const double sec = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    std::fprintf(stderr, "amg_build %.3f s\n", sec);
    FILE *f = std::fopen((d + "/levels.txt").c_str(), "w");
    std::fprintf(f, "%d %d\n", L, H.coarse_n);
    for (size_t l = 0; l < H.levels.size(); l++) {
        const lpm::AmgLevel &lv = H.levels[l];
        std::fprintf(f, "%d %d %.17g", lv.nblock, lv.bs, lv.omega);
        const std::string p = d + "/L" + std::to_string(l);
        wr_bsr(f, p + "_A", lv.A);
        wr_bsr(f, p + "_P", lv.P);
        wr_bsr(f, p + "_Pt", lv.Pt);
        std::fprintf(f, "\n");
        wr(p + "_Dinv.bin", lv.Dinv);
    }
    wr_bsr(f, d + "/coarse_A", H.coarse_A);
    std::fprintf(f, "\n");
    std::fclose(f);
    wr(d + "/coarse_chol.bin", H.coarse_chol);
    wr(d + "/coarse_inv.bin", H.coarse_inv);
    if (L >= 0) {
        FILE *fr = std::fopen((d + "/r.bin").c_str(), "rb");
        if (fr) {
            std::fclose(fr);
            auto r = rd<double>(d + "/r.bin", 4 * (size_t)n);
            // the block-Jacobi inverse [9][n] as the device keeps it
            std::vector<double> Pinv(9 * (size_t)n);
            if (L > 0)
                for (int i = 0; i < n; i++)
                    for (int k = 0; k < 9; k++)
                        Pinv[(size_t)k * n + i] = H.levels[0].Dinv[(size_t)i * 9 + k];
            const Level0<double> z0{n, mask.data(), rowoff.data(), npad.data(), cols.data(), Pinv.data()};
            std::vector<double> z(4 * (size_t)n, 0.0);
            const int nu = argc > 3 ? std::atoi(argv[3]) : 1;
            vcycle<double, double>(H, z0, val.data(), r.data(), z.data(), nu);
            wr(d + "/z.bin", z);
            // as the device runs it: everything in FP32
            std::vector<float> vf(val.begin(), val.end()), Pf(Pinv.begin(), Pinv.end());
            const Level0<float> z0f{n, mask.data(), rowoff.data(), npad.data(), cols.data(), Pf.data()};
            std::fill(z.begin(), z.end(), 0.0);
            vcycle<float, float>(H, z0f, vf.data(), r.data(), z.data(), nu);
            wr(d + "/z32.bin", z);
        }
    }
    return L >= 0 ? 0 : 1;
}
