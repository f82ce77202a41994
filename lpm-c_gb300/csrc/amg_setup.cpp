// Host-side build of a smoothed-aggregation multigrid hierarchy for the
// stiffness (the preconditioner planned to replace block-Jacobi in the PCG).
//
// Level 0 is the stiffness itself, given in the device block-CSR layout
// (rows padded to a multiple of 4 blocks, values component-major per row),
// with the boundary-condition mask (bit d of mask[i] set = DOF d free).
// Aggregates are boxes of 3 x 3 x 3 lattice spacings of the initial
// positions; above level 0, boxes of 3 x 3 x 3 aggregates of the level
// below.  The tentative prolongator of an aggregate spans the six rigid-body
// modes of its free DOFs (translations, rotations about the aggregate's
// centroid), orthonormalised by Householder QR, whose R becomes the
// near-nullspace of the next level; rank-deficient columns stay zero and the
// next level decouples them with a unit diagonal.  The prolongator is smoothed
// by one damped block-Jacobi step, P = (I - 4/3 D^-1 A / rho(D^-1 A)) T, and
// the coarse operator is the Galerkin product P^T A P.  The coarsest level is
// factored densely (Cholesky).
//
// Matrices are kept as scalar CSR (double) during the build; the sparse
// products run row-parallel with a dense accumulator per thread.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <vector>
#include <omp.h>
#include "amg.h"

namespace lpm {

namespace {

// C = A * B (scalar CSR), rows in parallel: a symbolic pass counts each
// row's distinct columns, a numeric pass fills them in ascending order.
Csr spgemm(const Csr &A, const Csr &B)
{
    Csr C;
    C.nrow = A.nrow;
    C.ncol = B.ncol;
    C.ptr.assign((size_t)A.nrow + 1, 0);
    const int nt = omp_get_max_threads();
    std::vector<std::vector<int>> mark(nt, std::vector<int>(B.ncol, -1));
#pragma omp parallel for schedule(dynamic, 256)
    for (int i = 0; i < A.nrow; i++) {
        std::vector<int> &mk = mark[omp_get_thread_num()];
        long long cnt = 0;
        for (long long a = A.ptr[i]; a < A.ptr[i + 1]; a++) {
            const int k = A.col[a];
            for (long long b = B.ptr[k]; b < B.ptr[k + 1]; b++) {
                const int j = B.col[b];
                if (mk[j] != i) {
                    mk[j] = i;
                    cnt++;
                }
            }
        }
        C.ptr[i + 1] = cnt;
    }
    for (int i = 0; i < A.nrow; i++)
        C.ptr[i + 1] += C.ptr[i];
    C.col.resize((size_t)C.ptr[A.nrow]);
    C.val.resize((size_t)C.ptr[A.nrow]);
    std::vector<std::vector<double>> acc(nt, std::vector<double>(B.ncol, 0.0));
    for (auto &m : mark)
        std::fill(m.begin(), m.end(), -1);
#pragma omp parallel for schedule(dynamic, 256)
    for (int i = 0; i < A.nrow; i++) {
        const int t = omp_get_thread_num();
        std::vector<int> &mk = mark[t];
        std::vector<double> &ac = acc[t];
        long long p = C.ptr[i];
        for (long long a = A.ptr[i]; a < A.ptr[i + 1]; a++) {
            const int k = A.col[a];
            const double av = A.val[a];
            for (long long b = B.ptr[k]; b < B.ptr[k + 1]; b++) {
                const int j = B.col[b];
                if (mk[j] != i) {
                    mk[j] = i;
                    C.col[p++] = j;
                    ac[j] = 0.0;
                }
                ac[j] += av * B.val[b];
            }
        }
        const long long p0 = C.ptr[i];
        std::sort(C.col.begin() + p0, C.col.begin() + p);
        for (long long q = p0; q < p; q++)
            C.val[q] = ac[C.col[q]];
    }
    return C;
}

Csr transpose(const Csr &A)
{
    Csr T;
    T.nrow = A.ncol;
    T.ncol = A.nrow;
    T.ptr.assign((size_t)A.ncol + 1, 0);
    for (long long a = 0; a < A.ptr[A.nrow]; a++)
        T.ptr[A.col[a] + 1]++;
    for (int j = 0; j < A.ncol; j++)
        T.ptr[j + 1] += T.ptr[j];
    T.col.resize((size_t)T.ptr[A.ncol]);
    T.val.resize((size_t)T.ptr[A.ncol]);
    std::vector<long long> fill(T.ptr.begin(), T.ptr.end() - 1);
    for (int i = 0; i < A.nrow; i++)
        for (long long a = A.ptr[i]; a < A.ptr[i + 1]; a++) {
            const long long q = fill[A.col[a]]++;
            T.col[q] = i;
            T.val[q] = A.val[a];
        }
    return T;
}

// y = A x
void spmv(const Csr &A, const std::vector<double> &x, std::vector<double> &y)
{
    y.assign(A.nrow, 0.0);
#pragma omp parallel for schedule(static)
    for (int i = 0; i < A.nrow; i++) {
        double s = 0.0;
        for (long long a = A.ptr[i]; a < A.ptr[i + 1]; a++)
            s += A.val[a] * x[A.col[a]];
        y[i] = s;
    }
}

// Inverse of each bs x bs diagonal block (Gauss-Jordan with partial
// pivoting); a block row with a zero row/column is decoupled: its inverse
// has a unit diagonal there.
std::vector<double> block_diag_inverse(const Csr &A, int bs)
{
    const int nb = A.nrow / bs;
    std::vector<double> out((size_t)nb * bs * bs, 0.0);
#pragma omp parallel for schedule(static)
    for (int I = 0; I < nb; I++) {
        double m[36], inv[36];
        for (int r = 0; r < bs; r++)
            for (int c = 0; c < bs; c++) {
                m[r * bs + c] = 0.0;
                inv[r * bs + c] = r == c ? 1.0 : 0.0;
            }
        for (int r = 0; r < bs; r++) {
            const int row = I * bs + r;
            for (long long a = A.ptr[row]; a < A.ptr[row + 1]; a++) {
                const int c = A.col[a] - I * bs;
                if (c >= 0 && c < bs)
                    m[r * bs + c] = A.val[a];
            }
        }
        // decouple empty rows
        for (int r = 0; r < bs; r++) {
            bool zero = true;
            for (int c = 0; c < bs; c++)
                zero = zero && m[r * bs + c] == 0.0 && m[c * bs + r] == 0.0;
            if (zero)
                m[r * bs + r] = 1.0;
        }
        for (int k = 0; k < bs; k++) {
            int piv = k;
            for (int r = k + 1; r < bs; r++)
                if (std::fabs(m[r * bs + k]) > std::fabs(m[piv * bs + k]))
                    piv = r;
            if (piv != k)
                for (int c = 0; c < bs; c++) {
                    std::swap(m[k * bs + c], m[piv * bs + c]);
                    std::swap(inv[k * bs + c], inv[piv * bs + c]);
                }
            const double d = m[k * bs + k];
            const double id = d != 0.0 ? 1.0 / d : 0.0;
            for (int c = 0; c < bs; c++) {
                m[k * bs + c] *= id;
                inv[k * bs + c] *= id;
            }
            for (int r = 0; r < bs; r++)
                if (r != k) {
                    const double f = m[r * bs + k];
                    if (f != 0.0)
                        for (int c = 0; c < bs; c++) {
                            m[r * bs + c] -= f * m[k * bs + c];
                            inv[r * bs + c] -= f * inv[k * bs + c];
                        }
                }
        }
        std::memcpy(&out[(size_t)I * bs * bs], inv, sizeof(double) * bs * bs);
    }
    return out;
}

void apply_block_diag(const std::vector<double> &Dinv, int bs, const std::vector<double> &x, std::vector<double> &y)
{
    const int nb = (int)(x.size() / bs);
    y.resize(x.size());
#pragma omp parallel for schedule(static)
    for (int I = 0; I < nb; I++)
        for (int r = 0; r < bs; r++) {
            double s = 0.0;
            for (int c = 0; c < bs; c++)
                s += Dinv[(size_t)I * bs * bs + r * bs + c] * x[(size_t)I * bs + c];
            y[(size_t)I * bs + r] = s;
        }
}

// rho(D^-1 A) by power iteration from a fixed start vector
double spectral_radius(const Csr &A, const std::vector<double> &Dinv, int bs)
{
    std::vector<double> v(A.nrow), w, z;
    for (int i = 0; i < A.nrow; i++)
        v[i] = 1.0 + 0.5 * std::sin(0.731 * i);
    double lam = 0.0;
    for (int it = 0; it < 20; it++) {
        double nv = 0.0;
        for (double t : v)
            nv += t * t;
        nv = std::sqrt(nv);
        if (!(nv > 0.0))
            return 1.0;
        for (double &t : v)
            t /= nv;
        spmv(A, v, w);
        apply_block_diag(Dinv, bs, w, z);
        double num = 0.0;
        for (int i = 0; i < A.nrow; i++)
            num += v[i] * z[i];
        lam = num;
        v.swap(z);
    }
    return std::max(lam, 1e-300);
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

}  // namespace

int amg_build(const AmgInput &in, AmgHierarchy &H, const AmgOptions &opt)
{
    H = AmgHierarchy();
    const int n = in.n;
    // ---- level 0 operator, scalar CSR, constrained rows and columns removed
    Csr A;
    A.nrow = A.ncol = 3 * n;
    A.ptr.assign((size_t)3 * n + 1, 0);
    auto freedof = [&](int i, int d) { return ((in.mask[i] >> d) & 1u) != 0; };
    for (int i = 0; i < n; i++)
        for (int r = 0; r < 3; r++)
            A.ptr[3 * (size_t)i + r + 1] = freedof(i, r) ? 3LL * in.nconn[i] : 0;
    for (int k = 0; k < 3 * n; k++)
        A.ptr[k + 1] += A.ptr[k];
    A.col.resize((size_t)A.ptr[3 * n]);
    A.val.resize((size_t)A.ptr[3 * n]);
#pragma omp parallel for schedule(dynamic, 256)
    for (int i = 0; i < n; i++) {
        const long long off = in.rowoff[i];
        const int np = in.npad[i], nc = in.nconn[i];
        for (int r = 0; r < 3; r++) {
            if (!freedof(i, r))
                continue;
            long long q = A.ptr[3 * (size_t)i + r];
            for (int b = 0; b < nc; b++) {
                const int j = in.cols[off + b];
                for (int c = 0; c < 3; c++) {
                    A.col[q] = 3 * j + c;
                    A.val[q] = freedof(j, c) ? in.val[9 * off + (size_t)(3 * r + c) * np + b] : 0.0;
                    q++;
                }
            }
        }
    }
    // ---- near-nullspace of level 0 and the aggregation grid
    const double h = opt.agg_spacing;
    double lo[3] = {in.xyz[0], in.xyz[1], in.xyz[2]};
    for (int i = 0; i < n; i++)
        for (int d = 0; d < 3; d++)
            lo[d] = std::min(lo[d], in.xyz[3 * (size_t)i + d]);
    std::vector<int> gidx(3 * (size_t)n);  // integer box coordinates of each block row
    for (int i = 0; i < n; i++)
        for (int d = 0; d < 3; d++)
            gidx[3 * (size_t)i + d] = (int)std::floor((in.xyz[3 * (size_t)i + d] - lo[d]) / h + 1e-9);
    std::vector<double> pos(in.xyz, in.xyz + 3 * (size_t)n);  // block-row positions
    int nrow_blocks = n, bs = 3;
    std::vector<double> Bnull;  // near-nullspace rows (bs * nrow_blocks) x 6
    for (int lev = 0; lev < opt.max_levels; lev++) {
        const int nd = nrow_blocks * bs;
        if (nrow_blocks <= opt.coarse_blocks)
            break;
        // aggregates: boxes of the integer grid (coarsened by 3 above level 0)
        std::vector<long long> key(nrow_blocks);
        int gmax[3] = {0, 0, 0};
        for (int I = 0; I < nrow_blocks; I++)
            for (int d = 0; d < 3; d++)
                gmax[d] = std::max(gmax[d], gidx[3 * (size_t)I + d]);
        for (int I = 0; I < nrow_blocks; I++)
            key[I] = ((long long)gidx[3 * (size_t)I + 2] * (gmax[1] + 1) + gidx[3 * (size_t)I + 1]) * (gmax[0] + 1) +
                     gidx[3 * (size_t)I];
        std::vector<long long> uk(key);
        std::sort(uk.begin(), uk.end());
        uk.erase(std::unique(uk.begin(), uk.end()), uk.end());
        const int nagg = (int)uk.size();
        if (nagg >= nrow_blocks)
            break;  // no coarsening left
        std::vector<int> agg(nrow_blocks);
        for (int I = 0; I < nrow_blocks; I++)
            agg[I] = (int)(std::lower_bound(uk.begin(), uk.end(), key[I]) - uk.begin());
        std::vector<double> cen(3 * (size_t)nagg, 0.0);
        std::vector<int> cnt(nagg, 0);
        for (int I = 0; I < nrow_blocks; I++) {
            for (int d = 0; d < 3; d++)
                cen[3 * (size_t)agg[I] + d] += pos[3 * (size_t)I + d];
            cnt[agg[I]]++;
        }
        for (int a = 0; a < nagg; a++)
            for (int d = 0; d < 3; d++)
                cen[3 * (size_t)a + d] /= cnt[a];
        // near-nullspace of this level's DOFs (zero rows where A has none)
        std::vector<double> Bl((size_t)nd * 6, 0.0);
        if (lev == 0) {
            for (int i = 0; i < n; i++) {
                const double x = pos[3 * (size_t)i] - cen[3 * (size_t)agg[i]],
                             y = pos[3 * (size_t)i + 1] - cen[3 * (size_t)agg[i] + 1],
                             z = pos[3 * (size_t)i + 2] - cen[3 * (size_t)agg[i] + 2];
                const double rot[3][3] = {{-y, 0.0, z}, {x, -z, 0.0}, {0.0, y, -x}};  // rows: x, y, z comps
                for (int d = 0; d < 3; d++) {
                    if (!freedof(i, d))
                        continue;
                    double *row = &Bl[(3 * (size_t)i + d) * 6];
                    row[d] = 1.0;
                    row[3] = rot[d][0];
                    row[4] = rot[d][1];
                    row[5] = rot[d][2];
                }
            }
        } else {
            Bl = Bnull;
        }
        // tentative prolongator T (nd x 6 nagg) and the next near-nullspace
        std::vector<std::vector<int>> members(nagg);
        for (int I = 0; I < nrow_blocks; I++)
            members[agg[I]].push_back(I);
        Csr T;
        T.nrow = nd;
        T.ncol = 6 * nagg;
        T.ptr.assign((size_t)nd + 1, 0);
        std::vector<double> Bc((size_t)nagg * 36, 0.0);
        std::vector<double> tv((size_t)nd * 6, 0.0);
#pragma omp parallel for schedule(dynamic, 16)
        for (int a = 0; a < nagg; a++) {
            const std::vector<int> &mem = members[a];
            const int m = (int)mem.size() * bs;
            std::vector<double> B((size_t)m * 6), Q, R;
            for (size_t q = 0; q < mem.size(); q++)
                for (int d = 0; d < bs; d++)
                    for (int c = 0; c < 6; c++)
                        B[(q * bs + d) * 6 + c] = Bl[((size_t)mem[q] * bs + d) * 6 + c];
            small_qr(B, m, 6, Q, R);
            // drop columns the aggregate cannot represent
            double rmax = 0.0;
            for (double v : R)
                rmax = std::max(rmax, std::fabs(v));
            for (int c = 0; c < 6; c++)
                if (!(std::fabs(R[(size_t)c * 6 + c]) > 1e-10 * std::max(1.0, rmax))) {
                    for (int r = 0; r < m; r++)
                        Q[(size_t)r * 6 + c] = 0.0;
                    for (int c2 = 0; c2 < 6; c2++)
                        R[(size_t)c * 6 + c2] = 0.0;
                }
            for (size_t q = 0; q < mem.size(); q++)
                for (int d = 0; d < bs; d++)
                    for (int c = 0; c < 6; c++)
                        tv[((size_t)mem[q] * bs + d) * 6 + c] = Q[(q * bs + d) * 6 + c];
            std::memcpy(&Bc[(size_t)a * 36], R.data(), sizeof(double) * 36);
        }
        for (int r = 0; r < nd; r++)
            T.ptr[r + 1] = T.ptr[r] + 6;
        T.col.resize((size_t)nd * 6);
        T.val = tv;
        for (int r = 0; r < nd; r++)
            for (int c = 0; c < 6; c++)
                T.col[(size_t)r * 6 + c] = 6 * agg[r / bs] + c;
        // smoothed prolongator P = T - omega D^-1 A T
        const std::vector<double> Dinv = block_diag_inverse(A, bs);
        const double rho = spectral_radius(A, Dinv, bs);
        const double omega = 4.0 / 3.0 / rho;
        Csr AT = spgemm(A, T);
        // D^-1 (A T): block rows of AT mixed by the bs x bs inverse
        Csr P;
        {
            Csr DAT;
            DAT.nrow = nd;
            DAT.ncol = AT.ncol;
            DAT.ptr.assign((size_t)nd + 1, 0);
            // the union pattern of the bs rows of a block row, for every row of it
            std::vector<std::vector<int>> pat(nrow_blocks);
#pragma omp parallel for schedule(dynamic, 256)
            for (int I = 0; I < nrow_blocks; I++) {
                std::vector<int> &pt = pat[I];
                for (int r = 0; r < bs; r++)
                    for (long long a2 = AT.ptr[I * bs + r]; a2 < AT.ptr[I * bs + r + 1]; a2++)
                        pt.push_back(AT.col[a2]);
                for (int c = 0; c < 6; c++)  // T's own columns too
                    pt.push_back(6 * agg[I] + c);
                std::sort(pt.begin(), pt.end());
                pt.erase(std::unique(pt.begin(), pt.end()), pt.end());
            }
            for (int I = 0; I < nrow_blocks; I++)
                for (int r = 0; r < bs; r++)
                    DAT.ptr[I * bs + r + 1] = (long long)pat[I].size();
            for (int k = 0; k < nd; k++)
                DAT.ptr[k + 1] += DAT.ptr[k];
            DAT.col.resize((size_t)DAT.ptr[nd]);
            DAT.val.assign((size_t)DAT.ptr[nd], 0.0);
#pragma omp parallel for schedule(dynamic, 256)
            for (int I = 0; I < nrow_blocks; I++) {
                const std::vector<int> &pt = pat[I];
                for (int r = 0; r < bs; r++) {
                    const long long base = DAT.ptr[I * bs + r];
                    for (size_t q = 0; q < pt.size(); q++)
                        DAT.col[base + q] = pt[q];
                    // T part
                    for (int c = 0; c < 6; c++) {
                        const size_t q = std::lower_bound(pt.begin(), pt.end(), 6 * agg[I] + c) - pt.begin();
                        DAT.val[base + q] += tv[((size_t)I * bs + r) * 6 + c];
                    }
                    // - omega D^-1 A T part
                    for (int s = 0; s < bs; s++) {
                        const double dv = Dinv[(size_t)I * bs * bs + r * bs + s];
                        if (dv == 0.0)
                            continue;
                        for (long long a2 = AT.ptr[I * bs + s]; a2 < AT.ptr[I * bs + s + 1]; a2++) {
                            const size_t q = std::lower_bound(pt.begin(), pt.end(), AT.col[a2]) - pt.begin();
                            DAT.val[base + q] -= omega * dv * AT.val[a2];
                        }
                    }
                }
            }
            P = std::move(DAT);
        }
        // rows of constrained level-0 DOFs stay out of the prolongation
        if (lev == 0)
            for (int i = 0; i < n; i++)
                for (int d = 0; d < 3; d++)
                    if (!freedof(i, d))
                        for (long long q = P.ptr[3 * (size_t)i + d]; q < P.ptr[3 * (size_t)i + d + 1]; q++)
                            P.val[q] = 0.0;
        Csr Pt = transpose(P);
        Csr AP = spgemm(A, P);
        Csr Ac = spgemm(Pt, AP);
        // decouple coarse DOFs whose prolongation column is empty
        {
            std::vector<char> empty(Ac.nrow, 1);
            for (long long q = 0; q < P.ptr[P.nrow]; q++)
                if (P.val[q] != 0.0)
                    empty[P.col[q]] = 0;
            // rebuild rows of empty DOFs as a unit diagonal
            Csr B2;
            B2.nrow = B2.ncol = Ac.nrow;
            B2.ptr.assign((size_t)Ac.nrow + 1, 0);
            for (int r = 0; r < Ac.nrow; r++) {
                long long c = 0;
                if (empty[r]) {
                    c = 1;
                } else {
                    for (long long q = Ac.ptr[r]; q < Ac.ptr[r + 1]; q++)
                        c += !empty[Ac.col[q]];
                }
                B2.ptr[r + 1] = B2.ptr[r] + c;
            }
            B2.col.resize((size_t)B2.ptr[Ac.nrow]);
            B2.val.resize((size_t)B2.ptr[Ac.nrow]);
            for (int r = 0; r < Ac.nrow; r++) {
                long long p = B2.ptr[r];
                if (empty[r]) {
                    B2.col[p] = r;
                    B2.val[p] = 1.0;
                    continue;
                }
                for (long long q = Ac.ptr[r]; q < Ac.ptr[r + 1]; q++)
                    if (!empty[Ac.col[q]]) {
                        B2.col[p] = Ac.col[q];
                        B2.val[p] = Ac.val[q];
                        p++;
                    }
            }
            Ac = std::move(B2);
        }
        AmgLevel L;
        L.nblock = nrow_blocks;
        L.bs = bs;
        L.A = std::move(A);
        L.Dinv = Dinv;
        L.omega = 1.0 / rho;
        L.P = std::move(P);
        L.Pt = std::move(Pt);
        H.levels.push_back(std::move(L));
        // next level: aggregates as block rows of 6 DOFs
        A = std::move(Ac);
        Bnull = Bc;  // R factors: the coarse near-nullspace, 6 x 6 per aggregate
        {
            // Bc is per aggregate 6 x 6 (rows = coarse DOFs of the aggregate)
            std::vector<double> Bn((size_t)nagg * 6 * 6);
            for (int a = 0; a < nagg; a++)
                for (int r = 0; r < 6; r++)
                    for (int c = 0; c < 6; c++)
                        Bn[((size_t)a * 6 + r) * 6 + c] = Bc[(size_t)a * 36 + r * 6 + c];
            Bnull.swap(Bn);
        }
        std::vector<int> g2(3 * (size_t)nagg);
        for (int I = 0; I < nrow_blocks; I++)
            for (int d = 0; d < 3; d++)
                g2[3 * (size_t)agg[I] + d] = gidx[3 * (size_t)I + d] / 3;
        gidx.swap(g2);
        pos.swap(cen);
        nrow_blocks = nagg;
        bs = 6;
    }
    // coarsest level: dense Cholesky (lower factor, row-major)
    const int nc = A.nrow;
    H.coarse_n = nc;
    H.coarse_chol.assign((size_t)nc * nc, 0.0);
    std::vector<double> &Lc = H.coarse_chol;
    for (int r = 0; r < nc; r++)
        for (long long q = A.ptr[r]; q < A.ptr[r + 1]; q++)
            Lc[(size_t)r * nc + A.col[q]] = A.val[q];
    for (int r = 0; r < nc; r++)
        if (Lc[(size_t)r * nc + r] == 0.0)
            Lc[(size_t)r * nc + r] = 1.0;  // decoupled DOF
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
    H.coarse_A = std::move(A);
    return (int)H.levels.size();
}

}  // namespace lpm
