// Host-side specimen setup: lattice generation, two-shell bond lists, AFEM
// connectivity, bond tables and the block-CSR stiffness pattern.  This is the
// once-per-specimen part of the reference (src/initialization.c,
// src/neighbor.c, src/stiffness.c:145-235); its outputs must be bit-identical
// to the reference's, so it is compiled without floating-point contraction
// and evaluates every expression in the reference's order.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>
#include <omp.h>
#include "lpm_internal.h"

namespace lpm {

static void lattice_constants(HostSetup &h)
{
    const double r = h.radius;
    h.cut1 = 2.0 * r;                 // neighbor1_cutoff
    h.cut2 = 2.0 * std::sqrt(2.0) * r;  // neighbor2_cutoff
    if (h.lattice == 2) {            // src/initialization.c:251-259
        h.nn1 = 6;
        h.nn2 = 12;
        h.vol = std::pow(2 * r, 3);
    } else {                         // src/initialization.c:336-345
        h.nn1 = 12;
        h.nn2 = 6;
        h.vol = 4.0 * std::sqrt(2.0) * std::pow(r, 3);
    }
}

// createCuboid for the identity orientation (all Euler angles zero): the
// rotation of src/initialization.c:287-313 maps every point to itself.
int build_lattice(HostSetup &h, int lattice, double radius, const double *box)
{
    if (lattice != 2 && lattice != 3)
        return fail(LPM_ERR_ARG, "lattice must be 2 (simple cubic) or 3 (FCC)");
    if (!(radius > 0.0))
        return fail(LPM_ERR_ARG, "radius must be positive");
    h.lattice = lattice;
    h.radius = radius;
    lattice_constants(h);
    const double bx = box[1] - box[0], by = box[3] - box[2], bz = box[5] - box[4];
    const double a = std::sqrt(bx * bx + by * by + bz * bz);
    const double t0 = -a, t1 = a;
    h.xyz.clear();
    auto keep = [&](double x, double y, double z) {
        if (x >= box[0] && x <= box[1] && y >= box[2] && y <= box[3] && z >= box[4] && z <= box[5]) {
            h.xyz.push_back(x);
            h.xyz.push_back(y);
            h.xyz.push_back(z);
        }
    };
    if (lattice == 2) {  // src/initialization.c:241-284
        const double s = 2 * radius;
        const int nx = 1 + (int)std::floor((t1 - t0) / s);
        for (int k = 1; k <= nx; k++) {
            const double z = t0 + s * (k - 1);
            for (int j = 1; j <= nx; j++) {
                const double y = t0 + s * (j - 1);
                for (int i = 1; i <= nx; i++)
                    keep(box[0] + s * (i - 1), y, z);
            }
        }
    } else {  // src/initialization.c:326-426 (alternating full / shifted rows)
        const double s = 4 * radius / std::sqrt(2.0);
        const int nx = 1 + (int)std::floor((t1 - t0) / s);
        const int ny = 1 + (int)std::floor((t1 - t0) / (s / 2.0));
        for (int k = 1; k <= ny; k++) {
            const double z = t0 + s / 2.0 * (k - 1);
            for (int j = 1; j <= ny; j++) {
                const double y = t0 + s / 2.0 * (j - 1);
                if ((k % 2 == 1) == (j % 2 == 1)) {
                    for (int i = 1; i <= nx; i++)
                        keep(t0 + s * (i - 1), y, z);
                } else {
                    for (int i = 1; i <= nx - 1; i++)
                        keep(t0 + s * (i - 1) + s / 2.0, y, z);
                }
            }
        }
    }
    h.n = (int)(h.xyz.size() / 3);
    if (h.n <= 0)
        return fail(LPM_ERR_ARG, "the box holds no lattice site");
    return h.n;
}

int build_particles(HostSetup &h, int lattice, double radius, int n, const double *xyz)
{
    if (lattice != 2 && lattice != 3)
        return fail(LPM_ERR_ARG, "lattice must be 2 (simple cubic) or 3 (FCC)");
    if (n <= 0 || !xyz)
        return fail(LPM_ERR_ARG, "no particles");
    h.lattice = lattice;
    h.radius = radius;
    lattice_constants(h);
    h.xyz.assign(xyz, xyz + 3 * (size_t)n);
    h.n = n;
    return n;
}

// searchNormalNeighbor (src/neighbor.c:9-46).  A uniform cell grid replaces
// the all-pairs loop; every candidate is tested with the reference's
// distance expression and cut-offs, and bonds are kept in ascending j.
// A particle with more bonds than the LPM_NN slots (the reference writes past
// the end of its row then) fails the setup: returns LPM_ERR_ARG with the
// particle named in the error, LPM_OK otherwise.
int build_neighbors(HostSetup &h)
{
    const int n = h.n;
    const double c1 = 1.01 * h.cut1, c2 = 1.01 * h.cut2;
    double lo[3], hi[3];
    for (int d = 0; d < 3; d++) {
        lo[d] = hi[d] = h.xyz[d];
    }
    for (int i = 0; i < n; i++)
        for (int d = 0; d < 3; d++) {
            lo[d] = std::min(lo[d], h.xyz[3 * i + d]);
            hi[d] = std::max(hi[d], h.xyz[3 * i + d]);
        }
    const double cs = c2 * 1.0001;
    int g[3];
    for (int d = 0; d < 3; d++)
        g[d] = (int)((hi[d] - lo[d]) / cs) + 1;
    const size_t ncell = (size_t)g[0] * g[1] * g[2];
    std::vector<int> cell(n), start(ncell + 1, 0), order(n);
    for (int i = 0; i < n; i++) {
        int c[3];
        for (int d = 0; d < 3; d++)
            c[d] = std::min(g[d] - 1, (int)((h.xyz[3 * i + d] - lo[d]) / cs));
        cell[i] = (c[2] * g[1] + c[1]) * g[0] + c[0];
        start[cell[i] + 1]++;
    }
    for (size_t c = 0; c < ncell; c++)
        start[c + 1] += start[c];
    {
        std::vector<int> fill(start.begin(), start.end() - 1);
        for (int i = 0; i < n; i++)
            order[fill[cell[i]]++] = i;
    }
    // sized without a fill: the loop below writes every slot of its row
    h.nbr.resize((size_t)n * LPM_NN);
    h.shell.resize((size_t)n * LPM_NN);
    h.nb.resize(n);
    h.L0.resize((size_t)n * LPM_NN);
    h.cs0.resize((size_t)n * LPM_NN * 3);
    const double *X = h.xyz.data();
    constexpr int MAXCAND = 96;
    int over = n;  // lowest particle with too many bonds
#pragma omp parallel for schedule(dynamic, 512) reduction(min : over)
    for (int i = 0; i < n; i++) {
        int cand[MAXCAND];
        double cd[MAXCAND];
        int nc = 0, found = 0;
        const int ci = cell[i];
        const int cx = ci % g[0], cy = (ci / g[0]) % g[1], cz = ci / (g[0] * g[1]);
        for (int dz = -1; dz <= 1; dz++)
            for (int dy = -1; dy <= 1; dy++)
                for (int dx = -1; dx <= 1; dx++) {
                    const int x = cx + dx, y = cy + dy, z = cz + dz;
                    if (x < 0 || y < 0 || z < 0 || x >= g[0] || y >= g[1] || z >= g[2])
                        continue;
                    const size_t c = ((size_t)z * g[1] + y) * g[0] + x;
                    for (int q = start[c]; q < start[c + 1]; q++) {
                        const int j = order[q];
                        const double ex = X[3 * j] - X[3 * i], ey = X[3 * j + 1] - X[3 * i + 1],
                                     ez = X[3 * j + 2] - X[3 * i + 2];
                        const double dis = std::sqrt(ex * ex + ey * ey + ez * ez);
                        if (((dis < c1) && (j != i)) || ((dis > c1) && (dis < c2))) {
                            found++;
                            if (nc < MAXCAND) {
                                cand[nc] = j;
                                cd[nc] = dis;
                                nc++;
                            }
                        }
                    }
                }
        // ascending j (the reference scans j = 0..n-1)
        for (int a = 1; a < nc; a++) {
            const int v = cand[a];
            const double dv = cd[a];
            int b = a - 1;
            while (b >= 0 && cand[b] > v) {
                cand[b + 1] = cand[b];
                cd[b + 1] = cd[b];
                b--;
            }
            cand[b + 1] = v;
            cd[b + 1] = dv;
        }
        if (found > LPM_NN)
            over = std::min(over, i);
        const int m = std::min(nc, LPM_NN);
        for (int q = 0; q < m; q++) {
            const int j = cand[q];
            const double dis = cd[q];
            const size_t b = (size_t)i * LPM_NN + q;
            h.nbr[b] = j;
            h.shell[b] = ((dis < c1) && (j != i)) ? 0 : 1;
            h.cs0[3 * b] = (X[3 * i] - X[3 * j]) / dis;
            h.cs0[3 * b + 1] = (X[3 * i + 1] - X[3 * j + 1]) / dis;
            h.cs0[3 * b + 2] = (X[3 * i + 2] - X[3 * j + 2]) / dis;
            h.L0[b] = dis;
        }
        for (int q = m; q < LPM_NN; q++) {
            const size_t b = (size_t)i * LPM_NN + q;
            h.nbr[b] = -1;
            h.shell[b] = -1;
            h.cs0[3 * b] = h.cs0[3 * b + 1] = h.cs0[3 * b + 2] = 0.0;
            h.L0[b] = 0.0;
        }
        h.nb[i] = m;
    }
    if (over < n)
        return fail(LPM_ERR_ARG, "setup: particle " + std::to_string(over) + " has more than " +
                                     std::to_string(LPM_NN) + " bonds within the cut-offs (searchNormalNeighbor "
                                     "keeps at most nneighbors per particle)");
    return LPM_OK;
}

// searchAFEMNeighbor (src/neighbor.c:49-141): conn[i] = sorted unique union,
// over i's bonds, of the bond partner and that partner's neighbours of the
// same shell; K_pointer[i] = {#conn >= i, start of row in the upper CSR}.
void build_afem(HostSetup &h)
{
    const int n = h.n, w = 61;
    h.conn.resize((size_t)n * w);
    h.nconn.resize(n);
#pragma omp parallel for schedule(dynamic, 512)
    for (int i = 0; i < n; i++) {
        int col[LPM_NN * (LPM_NN + 1)];
        int nc = 0;
        for (int j = 0; j < h.nb[i]; j++) {
            const size_t b = (size_t)i * LPM_NN + j;
            const int p = h.nbr[b], s = h.shell[b];
            col[nc++] = p;
            for (int k = 0; k < h.nb[p]; k++)
                if (h.shell[(size_t)p * LPM_NN + k] == s)
                    col[nc++] = h.nbr[(size_t)p * LPM_NN + k];
        }
        std::sort(col, col + nc);
        const int m = (int)(std::unique(col, col + nc) - col);
        const int mm = std::min(m, w);
        for (int k = 0; k < w; k++)
            h.conn[(size_t)i * w + k] = k < mm ? col[k] : -1;
        h.nconn[i] = mm;
    }
    h.kp0.assign(n + 1, 0);
    h.kp1.assign(n + 1, 0);
    for (int i = 0; i < n; i++) {
        int c = 0;
        for (int k = 0; k < h.nconn[i]; k++)
            c += (h.conn[(size_t)i * w + k] >= i);
        h.kp0[i] = c;
        h.kp1[i + 1] = h.kp1[i] + 9 * c - 3;
    }
}

// Reverse bond slot (src/constitutive.c:654-658) and the stress weight
// opp_flag / particle_volume (src/constitutive.c:541-562, damage_broken = 1).
void build_bond_tables(HostSetup &h)
{
    const int n = h.n;
    const double eps = 1e-6;
    h.rev.resize((size_t)n * LPM_NN);
    h.oppv.resize((size_t)n * LPM_NN);
#pragma omp parallel for
    for (int i = 0; i < n; i++) {
        for (int j = h.nb[i]; j < LPM_NN; j++) {
            h.rev[(size_t)i * LPM_NN + j] = -1;
            h.oppv[(size_t)i * LPM_NN + j] = 0.0;
        }
        for (int j = 0; j < h.nb[i]; j++) {
            const size_t b = (size_t)i * LPM_NN + j;
            const int p = h.nbr[b];
            int rv = -1;
            for (int q = 0; q < LPM_NN; q++)
                if (h.nbr[(size_t)p * LPM_NN + q] == i)
                    rv = q;
            h.rev[b] = rv;
            double opp = 1.0;
            if (h.nb[i] == LPM_NN) {
                opp = 0.5;
            } else {
                for (int m = 0; m < h.nb[i]; m++) {
                    const size_t c = (size_t)i * LPM_NN + m;
                    if (std::fabs(h.cs0[3 * c] + h.cs0[3 * b]) < eps &&
                        std::fabs(h.cs0[3 * c + 1] + h.cs0[3 * b + 1]) < eps &&
                        std::fabs(h.cs0[3 * c + 2] + h.cs0[3 * b + 2]) < eps) {
                        opp = 0.5;
                        break;
                    }
                }
            }
            h.oppv[b] = opp / h.vol;
        }
    }
}

// Block-CSR: block row i holds the blocks of conn[i] (ascending particle
// index, i included), padded to a multiple of 4 with zero blocks on column i.
void build_block_pattern(HostSetup &h)
{
    const int n = h.n, w = 61;
    h.npad.assign(n, 0);
    h.rowoff.assign(n + 1, 0);
    for (int i = 0; i < n; i++) {
        h.npad[i] = (h.nconn[i] + 3) & ~3;
        h.rowoff[i + 1] = h.rowoff[i] + h.npad[i];
    }
    h.cols.resize((size_t)h.rowoff[n]);  // every entry written below
#pragma omp parallel for
    for (int i = 0; i < n; i++) {
        int *c = h.cols.data() + h.rowoff[i];
        for (int k = 0; k < h.npad[i]; k++)
            c[k] = k < h.nconn[i] ? h.conn[(size_t)i * w + k] : i;
    }
}

// Concatenate independently built specimens into one setup: particle,
// bond and block indices of specimen s are shifted by its particle offset,
// so no bond or stiffness block couples two specimens (a block-diagonal
// system) and each specimen's arrays equal those of a single-specimen setup.
void merge_setups(HostSetup &dst, const std::vector<HostSetup> &parts, std::vector<int> &offsets)
{
    dst = HostSetup();
    const HostSetup &f = parts.front();
    dst.lattice = f.lattice;
    dst.radius = f.radius;
    dst.vol = f.vol;
    dst.cut1 = f.cut1;
    dst.cut2 = f.cut2;
    dst.nn1 = f.nn1;
    dst.nn2 = f.nn2;
    const size_t ns = parts.size();
    offsets.assign(ns + 1, 0);
    std::vector<long long> kb(ns + 1, 0), rb(ns + 1, 0);
    for (size_t s = 0; s < ns; s++) {
        offsets[s + 1] = offsets[s] + parts[s].n;
        kb[s + 1] = kb[s] + parts[s].kp1[parts[s].n];
        rb[s + 1] = rb[s] + parts[s].rowoff[parts[s].n];
    }
    const int n = offsets.back();
    const long long kbase = kb[ns], rbase = rb[ns];
    const size_t w = 61;
    dst.n = n;
    // every array sized once, then each specimen's particles copied in
    // parallel (no reallocation; the result equals appending the parts)
    dst.xyz.resize(3 * (size_t)n);
    dst.nbr.resize((size_t)n * LPM_NN);
    dst.shell.resize((size_t)n * LPM_NN);
    dst.nb.resize(n);
    dst.rev.resize((size_t)n * LPM_NN);
    dst.L0.resize((size_t)n * LPM_NN);
    dst.cs0.resize((size_t)n * LPM_NN * 3);
    dst.oppv.resize((size_t)n * LPM_NN);
    dst.conn.resize((size_t)n * w);
    dst.nconn.resize(n);
    dst.npad.resize(n);
    dst.cols.resize((size_t)rbase);
    dst.kp0.assign(n + 1, 0);
    dst.kp1.assign(n + 1, 0);
    dst.rowoff.assign(n + 1, 0);
    for (size_t s = 0; s < ns; s++) {
        const HostSetup &p = parts[s];
        const int o = offsets[s];
        const long long kbs = kb[s], rbs = rb[s];
#pragma omp parallel for schedule(static)
        for (int i = 0; i < p.n; i++) {
            const size_t gi = (size_t)o + i;
            for (int d = 0; d < 3; d++)
                dst.xyz[3 * gi + d] = p.xyz[3 * (size_t)i + d];
            for (int j = 0; j < LPM_NN; j++) {
                const size_t a = (size_t)i * LPM_NN + j, g = gi * LPM_NN + j;
                const int v = p.nbr[a];
                dst.nbr[g] = v >= 0 ? v + o : v;
                dst.shell[g] = p.shell[a];
                dst.rev[g] = p.rev[a];
                dst.L0[g] = p.L0[a];
                dst.oppv[g] = p.oppv[a];
                for (int d = 0; d < 3; d++)
                    dst.cs0[3 * g + d] = p.cs0[3 * a + d];
            }
            dst.nb[gi] = p.nb[i];
            for (size_t k = 0; k < w; k++) {
                const int v = p.conn[(size_t)i * w + k];
                dst.conn[gi * w + k] = v >= 0 ? v + o : v;
            }
            dst.nconn[gi] = p.nconn[i];
            dst.npad[gi] = p.npad[i];
            const long long r0 = p.rowoff[i], r1 = p.rowoff[i + 1];
            for (long long k = r0; k < r1; k++)
                dst.cols[(size_t)(rbs + k)] = p.cols[(size_t)k] + o;
            dst.kp0[gi] = p.kp0[i];
            dst.kp1[gi] = (int)(p.kp1[i] + kbs);
            dst.rowoff[gi] = r0 + rbs;
        }
    }
    dst.kp1[n] = (int)kbase;
    dst.rowoff[n] = rbase;
    // K_pointer is the reference's int32 offset into one specimen's upper
    // CSR; a batch beyond 2^31 entries has no such layout
    if (kbase > 2147483647LL) {
        dst.kp0.clear();
        dst.kp1.clear();
    }
}

// Set up nspec specimens (one lattice box each) and concatenate them; the
// specimens are independent, so they are built in parallel.
int build_batch(HostSetup &dst, int lattice, double radius, int nspec, const double *boxes,
                std::vector<int> &offsets)
{
    std::vector<HostSetup> parts(nspec);
    std::vector<int> rcs(nspec, 0);
    std::vector<std::string> errs(nspec);
    auto one = [&](int s) {
        int rc = build_lattice(parts[s], lattice, radius, boxes + 6 * (size_t)s);
        if (rc < 0) {
            rcs[s] = rc;
            errs[s] = g_err;
            return;
        }
        if (parts[s].n <= 0) {
            rcs[s] = LPM_ERR_ARG;
            errs[s] = "specimen " + std::to_string(s) + " holds no particle";
            return;
        }
        if ((rc = build_neighbors(parts[s])) < 0) {
            rcs[s] = rc;
            errs[s] = g_err;
            return;
        }
        build_afem(parts[s]);
        build_bond_tables(parts[s]);
        build_block_pattern(parts[s]);
    };
    if (nspec >= omp_get_max_threads()) {
#pragma omp parallel for schedule(dynamic, 1)
        for (int s = 0; s < nspec; s++)
            one(s);
    } else {
        for (int s = 0; s < nspec; s++)
            one(s);
    }
    for (int s = 0; s < nspec; s++)
        if (rcs[s] < 0)
            return fail(rcs[s], "specimen " + std::to_string(s) + ": " + errs[s]);
    long long total = 0;
    for (int s = 0; s < nspec; s++)
        total += parts[s].n;
    if (total > 2147483647LL / 4)
        return fail(LPM_ERR_ARG, "batch too large: " + std::to_string(total) + " particles");
    merge_setups(dst, parts, offsets);
    return dst.n;
}

// The block-CSR values (component-major rows, see lpm_internal.h) written in
// the reference's 1-based upper-triangular scalar CSR, the layout of
// calcStiffness3DFiniteDifference (src/stiffness.c:431-515): per particle the
// upper part of its diagonal block, then for every connected particle jj > i
// the full 3x3 block, in three scalar rows.  Any output may be null.  Rows
// write disjoint ranges, so particles are converted in parallel.
template <typename T>
void export_upper_csr_host(const HostSetup &h, const T *val, double *Kg, int *IK, int *JK)
{
    const int n = h.n, w = 61;
#pragma omp parallel for schedule(dynamic, 1024)
    for (int i = 0; i < n; i++) {
        const int base = h.kp1[i], k0 = h.kp0[i], np = h.npad[i];
        const long long off = h.rowoff[i];
        int num1 = 0;
        for (int jid = 0; jid < h.nconn[i]; jid++) {
            const int jj = h.conn[(size_t)i * w + jid];
            auto V = [&](int r, int q) { return (double)val[9 * off + (size_t)(3 * r + q) * np + jid]; };
            if (jj == i) {
                const int pos[6] = {base, base + 1, base + 2, base + 3 * k0, base + 3 * k0 + 1, base + 6 * k0 - 1};
                const int rq[6][2] = {{0, 0}, {0, 1}, {0, 2}, {1, 1}, {1, 2}, {2, 2}};
                const int col[6] = {3 * (jj + 1) - 2, 3 * (jj + 1) - 1, 3 * (jj + 1), 3 * (jj + 1) - 1,
                                    3 * (jj + 1), 3 * (jj + 1)};
                for (int k = 0; k < 6; k++) {
                    if (Kg)
                        Kg[pos[k]] = V(rq[k][0], rq[k][1]);
                    if (JK)
                        JK[pos[k]] = col[k];
                }
            } else if (jj > i) {
                num1++;
                const int rowstart[3] = {base + 3 * num1, base + 3 * k0 + 3 * num1 - 1, base + 6 * k0 + 3 * num1 - 3};
                for (int r = 0; r < 3; r++)
                    for (int q = 0; q < 3; q++) {
                        if (Kg)
                            Kg[rowstart[r] + q] = V(r, q);
                        if (JK)
                            JK[rowstart[r] + q] = 3 * (jj + 1) - 2 + q;
                    }
            }
        }
        if (IK) {
            IK[3 * i] = base + 1;
            IK[3 * i + 1] = base + 3 * k0 + 1;
            IK[3 * i + 2] = base + 6 * k0;
        }
    }
    if (IK)
        IK[3 * n] = h.kp1[n] + 1;
}
template void export_upper_csr_host<double>(const HostSetup &, const double *, double *, int *, int *);
template void export_upper_csr_host<float>(const HostSetup &, const float *, double *, int *, int *);

// calcKnTv's KnTve = radius * mapping * [C11, C12, C44] per particle
// (src/stiffness.c:179-185 SC, :210-216 FCC), summed in the order of a
// plain row-major matrix-vector product.
void kntv_per_particle(int lattice, double radius, const double *c11, const double *c12,
                       const double *c44, int n, double *knt)
{
    const double r2 = std::sqrt(2.0);
    const double msc[9] = {1, -1, -1, 0, 0, 1, 0, 1.0 / 18.0, -1.0 / 18.0};
    const double mfcc[9] = {0, 0, r2, r2 / 4.0, -r2 / 4.0, -r2 / 4.0, 0, r2 / 24.0, -r2 / 24.0};
    const double *m = lattice == 2 ? msc : mfcc;
    for (int i = 0; i < n; i++) {
        const double ce[3] = {c11[i], c12[i], c44[i]};
        for (int r = 0; r < 3; r++) {
            double s = 0.0;
            for (int l = 0; l < 3; l++)
                s += m[3 * r + l] * ce[l];
            knt[3 * i + r] = radius * s;
        }
    }
}

}  // namespace lpm
