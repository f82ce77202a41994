// Host-side build of a smoothed-aggregation multigrid hierarchy for the
// stiffness (the multigrid preconditioner of the PCG, k_amg.cu).
//
// Level 0 is the stiffness itself, read in place from the device block-CSR
// layout (rows padded to a multiple of 4 blocks, values component-major per
// row) with the boundary-condition mask (bit d of mask[i] set = DOF d free);
// constrained DOFs are removed, i.e. their rows and columns count as zero.
// Aggregates are boxes of 3 x 3 x 3 lattice spacings of the initial
// positions; above level 0, boxes of 3 x 3 x 3 aggregates of the level
// below.  The tentative prolongator T of an aggregate spans the six
// rigid-body modes of its free DOFs (translations, rotations about the
// aggregate's centroid), orthonormalised by Householder QR, whose R becomes
// the near-nullspace of the next level; rank-deficient columns stay zero and
// the next level decouples them with a unit diagonal.  The prolongator is
// smoothed by one damped block-Jacobi step, P = (I - 4/3 D^-1 A / rho) T with
// rho = rho(D^-1 A) from power iteration, and the coarse operator is the
// Galerkin product P^T (A P).  The coarsest level is factored densely.
//
// Everything is kept in blocks (3 x 3 and 3 x 6 on level 0, 6 x 6 above), so
// the products are small dense block products with compile-time sizes; rows
// run in parallel with per-thread column markers, and every output is laid
// out by a counting pass first, so the result does not depend on the thread
// count.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <vector>
#include <omp.h>
#include "amg.h"

namespace lpm {

namespace {

// Operator with BS x BS blocks in block-CSR.
template <int NB>
struct OpB {
    const Bsr &A;
    static constexpr int BS = NB;
    int nbr() const { return A.nbr; }
    template <typename F>
    void row(int I, F f) const
    {
        for (long long k = A.ptr[I]; k < A.ptr[I + 1]; k++)
            f(A.col[k], &A.val[(size_t)k * NB * NB]);
    }
};

// The level-0 operator: the stiffness of the device layout with the
// constrained rows and columns zeroed, as 3 x 3 row-major blocks without the
// padding.
Bsr level0(const AmgInput &in)
{
    const int n = in.n;
    Bsr A;
    A.nbr = A.nbc = n;
    A.R = A.C = 3;
    A.ptr.assign((size_t)n + 1, 0);
    for (int i = 0; i < n; i++)
        A.ptr[i + 1] = A.ptr[i] + in.nconn[i];
    A.col.resize((size_t)A.ptr[n]);
    A.val.resize((size_t)A.ptr[n] * 9);
#pragma omp parallel for schedule(dynamic, 256)
    for (int i = 0; i < n; i++) {
        const long long off = in.rowoff[i];
        const int np = in.npad[i], nc = in.nconn[i];
        const unsigned mi = in.mask[i];
        const double *v = in.val + 9 * off;
        for (int b = 0; b < nc; b++) {
            const long long k = A.ptr[i] + b;
            const int j = in.cols[off + b];
            const unsigned mj = in.mask[j];
            A.col[k] = j;
            for (int r = 0; r < 3; r++)
                for (int c = 0; c < 3; c++)
                    A.val[(size_t)k * 9 + 3 * r + c] =
                        (((mi >> r) & (mj >> c)) & 1u) ? v[(size_t)(3 * r + c) * np + b] : 0.0;
        }
    }
    return A;
}

// inverse of an n x n matrix (Gauss-Jordan, partial pivoting); rows and
// columns that are entirely zero are decoupled with a unit diagonal
template <int N>
void invert_block(const double *in, double *out)
{
    double m[N * N], inv[N * N];
    std::memcpy(m, in, sizeof(m));
    for (int r = 0; r < N; r++)
        for (int c = 0; c < N; c++)
            inv[r * N + c] = r == c ? 1.0 : 0.0;
    for (int r = 0; r < N; r++) {
        bool zero = true;
        for (int c = 0; c < N; c++)
            zero = zero && m[r * N + c] == 0.0 && m[c * N + r] == 0.0;
        if (zero)
            m[r * N + r] = 1.0;
    }
    for (int k = 0; k < N; k++) {
        int piv = k;
        for (int r = k + 1; r < N; r++)
            if (std::fabs(m[r * N + k]) > std::fabs(m[piv * N + k]))
                piv = r;
        if (piv != k)
            for (int c = 0; c < N; c++) {
                std::swap(m[k * N + c], m[piv * N + c]);
                std::swap(inv[k * N + c], inv[piv * N + c]);
            }
        const double d = m[k * N + k];
        const double id = d != 0.0 ? 1.0 / d : 0.0;
        for (int c = 0; c < N; c++) {
            m[k * N + c] *= id;
            inv[k * N + c] *= id;
        }
        for (int r = 0; r < N; r++)
            if (r != k) {
                const double f = m[r * N + k];
                if (f != 0.0)
                    for (int c = 0; c < N; c++) {
                        m[r * N + c] -= f * m[k * N + c];
                        inv[r * N + c] -= f * inv[k * N + c];
                    }
            }
    }
    std::memcpy(out, inv, sizeof(inv));
}

// C (R x Q) += A (R x K) * B (K x Q), all row-major
template <int R, int K, int Q>
inline void gemm_acc(const double *A, const double *B, double *C)
{
    for (int r = 0; r < R; r++)
        for (int k = 0; k < K; k++) {
            const double a = A[r * K + k];
            for (int q = 0; q < Q; q++)
                C[r * Q + q] += a * B[k * Q + q];
        }
}

// Householder QR of an m x k block (m rows of k columns, row-major): Q
// (m x k, orthonormal columns) and R (k x k, upper triangular).
void small_qr(std::vector<double> B, int m, int k, std::vector<double> &Q, std::vector<double> &R)
{
    std::vector<double> V((size_t)m * k, 0.0), beta(k, 0.0);
    for (int j = 0; j < k && j < m; j++) {
        double nx = 0.0;
        for (int i = j; i < m; i++)
            nx += B[(size_t)i * k + j] * B[(size_t)i * k + j];
        nx = std::sqrt(nx);
        if (nx == 0.0)
            continue;
        const double a = B[(size_t)j * k + j] >= 0.0 ? -nx : nx;
        double vn = 0.0;
        for (int i = j; i < m; i++) {
            V[(size_t)i * k + j] = B[(size_t)i * k + j] - (i == j ? a : 0.0);
            vn += V[(size_t)i * k + j] * V[(size_t)i * k + j];
        }
        if (vn == 0.0)
            continue;
        beta[j] = 2.0 / vn;
        for (int c = j; c < k; c++) {
            double s = 0.0;
            for (int i = j; i < m; i++)
                s += V[(size_t)i * k + j] * B[(size_t)i * k + c];
            s *= beta[j];
            for (int i = j; i < m; i++)
                B[(size_t)i * k + c] -= s * V[(size_t)i * k + j];
        }
    }
    R.assign((size_t)k * k, 0.0);
    for (int r = 0; r < k && r < m; r++)
        for (int c = r; c < k; c++)
            R[(size_t)r * k + c] = B[(size_t)r * k + c];
    // Q = H_0 H_1 ... applied to the first k unit columns
    Q.assign((size_t)m * k, 0.0);
    for (int c = 0; c < k && c < m; c++)
        Q[(size_t)c * k + c] = 1.0;
    for (int j = std::min(k, m) - 1; j >= 0; j--) {
        if (beta[j] == 0.0)
            continue;
        for (int c = 0; c < k; c++) {
            double s = 0.0;
            for (int i = j; i < m; i++)
                s += V[(size_t)i * k + j] * Q[(size_t)i * k + c];
            s *= beta[j];
            for (int i = j; i < m; i++)
                Q[(size_t)i * k + c] -= s * V[(size_t)i * k + j];
        }
    }
}

// Per-thread map from column to slot of the current row.
struct Marker {
    std::vector<int> slot;
    std::vector<int> used;
    explicit Marker(int ncol) : slot(ncol, -1) {}
    int find_or_add(int c)
    {
        int &s = slot[c];
        if (s < 0) {
            s = (int)used.size();
            used.push_back(c);
        }
        return s;
    }
    void reset()
    {
        for (int c : used)
            slot[c] = -1;
        used.clear();
    }
};

// Exclusive prefix sum of counts into ptr (size n + 1).
void prefix(const std::vector<long long> &cnt, avec<long long> &ptr)
{
    ptr.assign(cnt.size() + 1, 0);
    for (size_t i = 0; i < cnt.size(); i++)
        ptr[i + 1] = ptr[i] + cnt[i];
}

// Transpose of a block-CSR matrix; rows of the result list their columns in
// ascending order.  Column counts per contiguous chunk of rows give every
// block its place, so the chunks fill in parallel (any number of threads).
Bsr transpose(const Bsr &A)
{
    Bsr T;
    T.nbr = A.nbc;
    T.nbc = A.nbr;
    T.R = A.C;
    T.C = A.R;
    const int nt = omp_get_max_threads();
    const int bsz = A.R * A.C;
    std::vector<std::vector<long long>> cnt(nt, std::vector<long long>(A.nbc, 0));
    std::vector<int> lo(nt + 1);
    for (int t = 0; t <= nt; t++)
        lo[t] = (int)((long long)A.nbr * t / nt);
#pragma omp parallel for schedule(static, 1)
    for (int t = 0; t < nt; t++)
        for (int i = lo[t]; i < lo[t + 1]; i++)
            for (long long k = A.ptr[i]; k < A.ptr[i + 1]; k++)
                cnt[t][A.col[k]]++;
    T.ptr.assign((size_t)A.nbc + 1, 0);
    for (int c = 0; c < A.nbc; c++) {
        long long s = 0;
        for (int t = 0; t < nt; t++)
            s += cnt[t][c];
        T.ptr[c + 1] = T.ptr[c] + s;
    }
    // per-thread start of each column
    for (int c = 0; c < A.nbc; c++) {
        long long p = T.ptr[c];
        for (int t = 0; t < nt; t++) {
            const long long k = cnt[t][c];
            cnt[t][c] = p;
            p += k;
        }
    }
    T.col.resize((size_t)T.ptr[A.nbc]);
    T.val.resize((size_t)T.ptr[A.nbc] * bsz);
#pragma omp parallel for schedule(static, 1)
    for (int t = 0; t < nt; t++)
        for (int i = lo[t]; i < lo[t + 1]; i++)
            for (long long k = A.ptr[i]; k < A.ptr[i + 1]; k++) {
                const long long q = cnt[t][A.col[k]]++;
                T.col[q] = i;
                const double *s = &A.val[(size_t)k * bsz];
                double *d = &T.val[(size_t)q * bsz];
                for (int r = 0; r < A.R; r++)
                    for (int c = 0; c < A.C; c++)
                        d[c * A.R + r] = s[r * A.C + c];
            }
    return T;
}

template <class Op>
std::vector<double> diag_inverse(const Op &A)
{
    constexpr int BS = Op::BS;
    const int nb = A.nbr();
    std::vector<double> out((size_t)nb * BS * BS);
#pragma omp parallel for schedule(dynamic, 256)
    for (int I = 0; I < nb; I++) {
        double d[BS * BS] = {};
        A.row(I, [&](int J, const double *blk) {
            if (J == I)
                for (int k = 0; k < BS * BS; k++)
                    d[k] += blk[k];
        });
        invert_block<BS>(d, &out[(size_t)I * BS * BS]);
    }
    return out;
}

// rho(D^-1 A) by power iteration from a fixed start vector; the sums run over
// per-row partials in row order, so the estimate does not depend on the
// thread count
template <class Op>
double spectral_radius(const Op &A, const std::vector<double> &Dinv, int iters)
{
    constexpr int BS = Op::BS;
    const int nb = A.nbr();
    const size_t nd = (size_t)nb * BS;
    std::vector<double> v(nd), z(nd), part(nb);
    for (size_t i = 0; i < nd; i++)
        v[i] = 1.0 + 0.5 * std::sin(0.731 * (double)i);
    double lam = 1e-300;
    for (int it = 0; it < iters; it++) {
#pragma omp parallel for schedule(static)
        for (int I = 0; I < nb; I++) {
            double s = 0.0;
            for (int r = 0; r < BS; r++)
                s += v[(size_t)I * BS + r] * v[(size_t)I * BS + r];
            part[I] = s;
        }
        double nv = 0.0;
        for (int I = 0; I < nb; I++)
            nv += part[I];
        nv = std::sqrt(nv);
        if (!(nv > 0.0))
            return 1.0;
#pragma omp parallel for schedule(dynamic, 256)
        for (int I = 0; I < nb; I++) {
            double y[BS] = {};
            A.row(I, [&](int J, const double *blk) {
                for (int r = 0; r < BS; r++)
                    for (int c = 0; c < BS; c++)
                        y[r] += blk[r * BS + c] * v[(size_t)J * BS + c];
            });
            const double *D = &Dinv[(size_t)I * BS * BS];
            double num = 0.0;
            for (int r = 0; r < BS; r++) {
                double s = 0.0;
                for (int c = 0; c < BS; c++)
                    s += D[r * BS + c] * y[c];
                z[(size_t)I * BS + r] = s / nv;
                num += v[(size_t)I * BS + r] * s;
            }
            part[I] = num;
        }
        double num = 0.0;
        for (int I = 0; I < nb; I++)
            num += part[I];
        lam = num / (nv * nv);
        v.swap(z);
    }
    return std::max(lam, 1e-300);
}

// One coarsening step from an operator with BS x BS blocks.
struct CoarseOut {
    Bsr Ac;
    std::vector<double> Bc;  // coarse near-nullspace, 6 x 6 per aggregate (row-major)
    std::vector<int> gidx;   // integer box coordinates of the aggregates
    std::vector<int> grp;    // specimen of each aggregate
    std::vector<double> cen; // aggregate centroids
};

template <class Op>
bool coarsen(const Op &A, const uint8_t *mask, const std::vector<int> &gidx, const std::vector<int> &grp,
             const std::vector<double> &pos,
             const std::vector<double> &Bl, const AmgOptions &opt, AmgLevel &L, CoarseOut &out)
{
    constexpr int BS = Op::BS;
    const int nb = A.nbr();
    // aggregates: boxes of the integer grid
    int gmax[3] = {0, 0, 0};
    for (int I = 0; I < nb; I++)
        for (int d = 0; d < 3; d++)
            gmax[d] = std::max(gmax[d], gidx[3 * (size_t)I + d]);
    // boxes never join block rows of different specimens (grp), so every
    // level stays block-diagonal over the specimens of a batch
    std::vector<long long> key(nb);
    for (int I = 0; I < nb; I++)
        key[I] = (((long long)grp[I] * (gmax[2] + 1) + gidx[3 * (size_t)I + 2]) * (gmax[1] + 1) +
                  gidx[3 * (size_t)I + 1]) * (gmax[0] + 1) +
                 gidx[3 * (size_t)I];
    std::vector<long long> uk(key);
    std::sort(uk.begin(), uk.end());
    uk.erase(std::unique(uk.begin(), uk.end()), uk.end());
    const int nagg = (int)uk.size();
    if (nagg >= nb)
        return false;
    std::vector<int> agg(nb);
#pragma omp parallel for schedule(static)
    for (int I = 0; I < nb; I++)
        agg[I] = (int)(std::lower_bound(uk.begin(), uk.end(), key[I]) - uk.begin());
    std::vector<long long> mcnt(nagg, 0);
    avec<long long> mptr;
    for (int I = 0; I < nb; I++)
        mcnt[agg[I]]++;
    prefix(mcnt, mptr);
    std::vector<int> mem(nb);
    {
        std::vector<long long> fill(mptr.begin(), mptr.end() - 1);
        for (int I = 0; I < nb; I++)
            mem[fill[agg[I]]++] = I;
    }
    out.cen.assign(3 * (size_t)nagg, 0.0);
    for (int a = 0; a < nagg; a++) {
        for (long long q = mptr[a]; q < mptr[a + 1]; q++)
            for (int d = 0; d < 3; d++)
                out.cen[3 * (size_t)a + d] += pos[3 * (size_t)mem[q] + d];
        for (int d = 0; d < 3; d++)
            out.cen[3 * (size_t)a + d] /= (double)(mptr[a + 1] - mptr[a]);
    }
    // near-nullspace on level 0: translations and rotations about the centroid
    std::vector<double> B0;
    const std::vector<double> *B = &Bl;
    if (mask) {
        B0.assign((size_t)nb * BS * 6, 0.0);
#pragma omp parallel for schedule(static)
        for (int i = 0; i < nb; i++) {
            const double *c = &out.cen[3 * (size_t)agg[i]];
            const double x = pos[3 * (size_t)i] - c[0], y = pos[3 * (size_t)i + 1] - c[1],
                         z = pos[3 * (size_t)i + 2] - c[2];
            const double rot[3][3] = {{-y, 0.0, z}, {x, -z, 0.0}, {0.0, y, -x}};  // rows: x, y, z comps
            for (int d = 0; d < 3; d++) {
                if (!((mask[i] >> d) & 1u))
                    continue;
                double *row = &B0[((size_t)i * BS + d) * 6];
                row[d] = 1.0;
                row[3] = rot[d][0];
                row[4] = rot[d][1];
                row[5] = rot[d][2];
            }
        }
        B = &B0;
    }
    // tentative prolongator: one BS x 6 block per block row
    std::vector<double> T((size_t)nb * BS * 6, 0.0);
    out.Bc.assign((size_t)nagg * 36, 0.0);
    std::vector<char> dropped((size_t)nagg * 6, 0);
#pragma omp parallel for schedule(dynamic, 16)
    for (int a = 0; a < nagg; a++) {
        const int cnt = (int)(mptr[a + 1] - mptr[a]);
        const int m = cnt * BS;
        std::vector<double> Bm((size_t)m * 6), Q, R;
        for (int q = 0; q < cnt; q++)
            std::memcpy(&Bm[(size_t)q * BS * 6], &(*B)[(size_t)mem[mptr[a] + q] * BS * 6], sizeof(double) * BS * 6);
        small_qr(Bm, m, 6, Q, R);
        double rmax = 0.0;
        for (double v : R)
            rmax = std::max(rmax, std::fabs(v));
        for (int c = 0; c < 6; c++)
            if (!(std::fabs(R[(size_t)c * 6 + c]) > 1e-10 * std::max(1.0, rmax))) {
                dropped[(size_t)a * 6 + c] = 1;
                for (int r = 0; r < m; r++)
                    Q[(size_t)r * 6 + c] = 0.0;
                for (int c2 = 0; c2 < 6; c2++)
                    R[(size_t)c * 6 + c2] = 0.0;
            }
        for (int q = 0; q < cnt; q++)
            std::memcpy(&T[(size_t)mem[mptr[a] + q] * BS * 6], &Q[(size_t)q * BS * 6], sizeof(double) * BS * 6);
        std::memcpy(&out.Bc[(size_t)a * 36], R.data(), sizeof(double) * 36);
    }
    // smoother data
    L.nblock = nb;
    L.bs = BS;
    L.Dinv = diag_inverse(A);
    const double rho = spectral_radius(A, L.Dinv, opt.power_iters);
    L.omega = 4.0 / 3.0 / rho;  // 13 % fewer PCG iterations than 1 / rho on the CPU checks
    const double wp = 4.0 / 3.0 / rho;
    // smoothed prolongator P = T - wp D^-1 A T, BS x 6 blocks; the row of a
    // block row lists the aggregates of its operator row, its own first
    Bsr &P = L.P;
    P.nbr = nb;
    P.nbc = nagg;
    P.R = BS;
    P.C = 6;
    {
        std::vector<long long> cnt(nb);
#pragma omp parallel
        {
            Marker mk(nagg);
#pragma omp for schedule(dynamic, 256)
            for (int I = 0; I < nb; I++) {
                mk.find_or_add(agg[I]);
                A.row(I, [&](int J, const double *) { mk.find_or_add(agg[J]); });
                cnt[I] = (long long)mk.used.size();
                mk.reset();
            }
        }
        prefix(cnt, P.ptr);
    }
    P.col.resize((size_t)P.ptr[nb]);
    P.val.resize((size_t)P.ptr[nb] * BS * 6);  // every value written below
#pragma omp parallel
    {
        Marker mk(nagg);
        std::vector<double> acc;
#pragma omp for schedule(dynamic, 256)
        for (int I = 0; I < nb; I++) {
            const long long p0 = P.ptr[I];
            const int ns = (int)(P.ptr[I + 1] - p0);
            acc.assign((size_t)ns * BS * 6, 0.0);
            mk.find_or_add(agg[I]);
            A.row(I, [&](int J, const double *blk) {
                const int s = mk.find_or_add(agg[J]);
                gemm_acc<BS, BS, 6>(blk, &T[(size_t)J * BS * 6], &acc[(size_t)s * BS * 6]);
            });
            const double *D = &L.Dinv[(size_t)I * BS * BS];
            for (int s = 0; s < ns; s++) {
                P.col[p0 + s] = mk.used[s];
                double *pv = &P.val[(size_t)(p0 + s) * BS * 6];
                double da[BS * 6] = {};
                gemm_acc<BS, BS, 6>(D, &acc[(size_t)s * BS * 6], da);
                for (int k = 0; k < BS * 6; k++)
                    pv[k] = (s == 0 ? T[(size_t)I * BS * 6 + k] : 0.0) - wp * da[k];
                if (mask)  // constrained level-0 DOFs stay out of the prolongation
                    for (int r = 0; r < BS; r++)
                        if (!((mask[I] >> r) & 1u))
                            for (int c = 0; c < 6; c++)
                                pv[r * 6 + c] = 0.0;
            }
            mk.reset();
        }
    }
    L.Pt = transpose(P);
    // W = A P (BS x 6 blocks)
    Bsr W;
    W.nbr = nb;
    W.nbc = nagg;
    W.R = BS;
    W.C = 6;
    {
        std::vector<long long> cnt(nb);
#pragma omp parallel
        {
            Marker mk(nagg);
#pragma omp for schedule(dynamic, 256)
            for (int I = 0; I < nb; I++) {
                A.row(I, [&](int J, const double *) {
                    for (long long k = P.ptr[J]; k < P.ptr[J + 1]; k++)
                        mk.find_or_add(P.col[k]);
                });
                cnt[I] = (long long)mk.used.size();
                mk.reset();
            }
        }
        prefix(cnt, W.ptr);
    }
    W.col.resize((size_t)W.ptr[nb]);
    W.val.resize((size_t)W.ptr[nb] * BS * 6);  // zeroed row by row below
#pragma omp parallel
    {
        Marker mk(nagg);
#pragma omp for schedule(dynamic, 256)
        for (int I = 0; I < nb; I++) {
            const long long w0 = W.ptr[I];
            std::fill(W.val.begin() + (size_t)w0 * BS * 6, W.val.begin() + (size_t)W.ptr[I + 1] * BS * 6, 0.0);
            A.row(I, [&](int J, const double *blk) {
                for (long long k = P.ptr[J]; k < P.ptr[J + 1]; k++) {
                    const int s = mk.find_or_add(P.col[k]);
                    gemm_acc<BS, BS, 6>(blk, &P.val[(size_t)k * BS * 6], &W.val[(size_t)(w0 + s) * BS * 6]);
                }
            });
            for (size_t s = 0; s < mk.used.size(); s++)
                W.col[w0 + s] = mk.used[s];
            mk.reset();
        }
    }
    // Ac = P^T W (6 x 6 blocks); every row holds its diagonal block
    Bsr &Ac = out.Ac;
    Ac.nbr = Ac.nbc = nagg;
    Ac.R = Ac.C = 6;
    const Bsr &Pt = L.Pt;
    {
        std::vector<long long> cnt(nagg);
#pragma omp parallel
        {
            Marker mk(nagg);
#pragma omp for schedule(dynamic, 16)
            for (int a = 0; a < nagg; a++) {
                mk.find_or_add(a);
                for (long long k = Pt.ptr[a]; k < Pt.ptr[a + 1]; k++) {
                    const int I = Pt.col[k];
                    for (long long q = W.ptr[I]; q < W.ptr[I + 1]; q++)
                        mk.find_or_add(W.col[q]);
                }
                cnt[a] = (long long)mk.used.size();
                mk.reset();
            }
        }
        prefix(cnt, Ac.ptr);
    }
    Ac.col.resize((size_t)Ac.ptr[nagg]);
    Ac.val.resize((size_t)Ac.ptr[nagg] * 36);  // zeroed row by row below
#pragma omp parallel
    {
        Marker mk(nagg);
#pragma omp for schedule(dynamic, 16)
        for (int a = 0; a < nagg; a++) {
            const long long a0 = Ac.ptr[a];
            std::fill(Ac.val.begin() + (size_t)a0 * 36, Ac.val.begin() + (size_t)Ac.ptr[a + 1] * 36, 0.0);
            mk.find_or_add(a);
            for (long long k = Pt.ptr[a]; k < Pt.ptr[a + 1]; k++) {
                const int I = Pt.col[k];
                // Pt block (6 x BS) is the transpose of P's (BS x 6)
                const double *pt = &Pt.val[(size_t)k * 6 * BS];
                for (long long q = W.ptr[I]; q < W.ptr[I + 1]; q++) {
                    const int s = mk.find_or_add(W.col[q]);
                    gemm_acc<6, BS, 6>(pt, &W.val[(size_t)q * BS * 6], &Ac.val[(size_t)(a0 + s) * 36]);
                }
            }
            for (size_t s = 0; s < mk.used.size(); s++)
                Ac.col[a0 + s] = mk.used[s];
            // coarse DOFs without a prolongation column: unit diagonal
            for (int c = 0; c < 6; c++)
                if (dropped[(size_t)a * 6 + c])
                    Ac.val[(size_t)a0 * 36 + c * 6 + c] = 1.0;
            mk.reset();
        }
    }
    // next level's grid
    out.grp.assign(nagg, 0);
    for (int I = 0; I < nb; I++)
        out.grp[agg[I]] = grp[I];
    out.gidx.assign(3 * (size_t)nagg, 0);
    for (int I = 0; I < nb; I++)
        for (int d = 0; d < 3; d++)
            out.gidx[3 * (size_t)agg[I] + d] = gidx[3 * (size_t)I + d] / 3;
    return true;
}

}  // namespace

int amg_build(const AmgInput &in, AmgHierarchy &H, const AmgOptions &opt)
{
    H = AmgHierarchy();
    const int n = in.n;
    const double h = opt.agg_spacing;
    double lo[3] = {in.xyz[0], in.xyz[1], in.xyz[2]};
    for (int i = 0; i < n; i++)
        for (int d = 0; d < 3; d++)
            lo[d] = std::min(lo[d], in.xyz[3 * (size_t)i + d]);
    std::vector<int> gidx(3 * (size_t)n);
    for (int i = 0; i < n; i++)
        for (int d = 0; d < 3; d++)
            gidx[3 * (size_t)i + d] = (int)std::floor((in.xyz[3 * (size_t)i + d] - lo[d]) / h + 1e-9);
    std::vector<double> pos(in.xyz, in.xyz + 3 * (size_t)n);
    std::vector<int> grp(n, 0);
    if (in.group)
        grp.assign(in.group, in.group + n);
    Bsr A = level0(in);  // the operator of the level being coarsened
    std::vector<double> Bnull;
    if (n > opt.coarse_blocks && opt.max_levels > 0) {
        AmgLevel L;
        CoarseOut co;
        if (coarsen(OpB<3>{A}, in.mask, gidx, grp, pos, Bnull, opt, L, co)) {
            H.levels.push_back(std::move(L));
            A = std::move(co.Ac);
            Bnull = std::move(co.Bc);
            gidx = std::move(co.gidx);
            grp = std::move(co.grp);
            pos = std::move(co.cen);
        }
    }
    while (!H.levels.empty() && (int)H.levels.size() < opt.max_levels && A.nbr > opt.coarse_blocks) {
        AmgLevel L;
        CoarseOut co;
        if (!coarsen(OpB<6>{A}, nullptr, gidx, grp, pos, Bnull, opt, L, co))
            break;
        L.A = std::move(A);
        H.levels.push_back(std::move(L));
        A = std::move(co.Ac);
        Bnull = std::move(co.Bc);
        gidx = std::move(co.gidx);
        grp = std::move(co.grp);
        pos = std::move(co.cen);
    }
    // coarsest level: dense Cholesky (lower factor, row-major) and inverse
    const int bs = A.R;
    const int nc = A.nbr * bs;
    if (nc > opt.max_coarse_dofs)
        return -2;  // the lattice did not coarsen (aggregate boxes below the particle spacing)
    H.coarse_n = nc;
    H.coarse_chol.assign((size_t)nc * nc, 0.0);
    std::vector<double> &Lc = H.coarse_chol;
    for (int I = 0; I < A.nbr; I++)
        for (long long k = A.ptr[I]; k < A.ptr[I + 1]; k++)
            for (int r = 0; r < bs; r++)
                for (int c = 0; c < bs; c++)
                    Lc[(size_t)(I * bs + r) * nc + A.col[k] * bs + c] += A.val[(size_t)k * bs * bs + r * bs + c];
    for (int r = 0; r < nc; r++) {
        bool zero = true;
        for (int c = 0; c < nc && zero; c++)
            zero = Lc[(size_t)r * nc + c] == 0.0;
        if (zero)
            Lc[(size_t)r * nc + r] = 1.0;  // decoupled (constrained) DOF
    }
    for (int j = 0; j < nc; j++) {
        double d = Lc[(size_t)j * nc + j];
        for (int k = 0; k < j; k++)
            d -= Lc[(size_t)j * nc + k] * Lc[(size_t)j * nc + k];
        if (!(d > 0.0))
            return -1;  // not positive definite
        d = std::sqrt(d);
        Lc[(size_t)j * nc + j] = d;
#pragma omp parallel for schedule(static)
        for (int i = j + 1; i < nc; i++) {
            double s = Lc[(size_t)i * nc + j];
            for (int k = 0; k < j; k++)
                s -= Lc[(size_t)i * nc + k] * Lc[(size_t)j * nc + k];
            Lc[(size_t)i * nc + j] = s / d;
        }
    }
    for (int i = 0; i < nc; i++)
        for (int j = i + 1; j < nc; j++)
            Lc[(size_t)i * nc + j] = 0.0;
    // inverse: solve L L^T X = I column by column
    H.coarse_inv.assign((size_t)nc * nc, 0.0);
#pragma omp parallel
    {
        std::vector<double> y(nc);
#pragma omp for schedule(dynamic, 8)
        for (int col = 0; col < nc; col++) {
            for (int i = 0; i < nc; i++) {
                double s = i == col ? 1.0 : 0.0;
                for (int k = 0; k < i; k++)
                    s -= Lc[(size_t)i * nc + k] * y[k];
                y[i] = s / Lc[(size_t)i * nc + i];
            }
            for (int i = nc - 1; i >= 0; i--) {
                double s = y[i];
                for (int k = i + 1; k < nc; k++)
                    s -= Lc[(size_t)k * nc + i] * y[k];
                y[i] = s / Lc[(size_t)i * nc + i];
            }
            for (int i = 0; i < nc; i++)
                H.coarse_inv[(size_t)i * nc + col] = y[i];
        }
    }
    H.coarse_A = std::move(A);
    return (int)H.levels.size();
}

}  // namespace lpm
