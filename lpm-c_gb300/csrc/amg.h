// Smoothed-aggregation multigrid hierarchy for the stiffness, built on the
// host (amg_setup.cpp).  Plain C++ (no CUDA types), so that it can be built
// and checked without a GPU.
#pragma once
#include <cstdint>
#include <memory>
#include <utility>
#include <vector>

namespace lpm {

// Allocator whose resize() leaves elements uninitialised, so that the large
// arrays of the build are first written by the parallel loops that fill
// them (no serial zero fill, pages touched by the threads that use them).
template <typename T>
struct AmgNoInit : std::allocator<T> {
    template <typename U>
    struct rebind {
        typedef AmgNoInit<U> other;
    };
    AmgNoInit() = default;
    template <typename U>
    AmgNoInit(const AmgNoInit<U> &) noexcept {}
    template <typename U>
    void construct(U *p) noexcept { ::new (static_cast<void *>(p)) U; }
    template <typename U, typename... A>
    void construct(U *p, A &&...a) { ::new (static_cast<void *>(p)) U(std::forward<A>(a)...); }
};
template <typename T>
using avec = std::vector<T, AmgNoInit<T>>;

// Block-CSR with R x C blocks, 0-based; block k is val[k*R*C ...], row-major.
struct Bsr {
    int nbr = 0, nbc = 0;  // block rows, block columns
    int R = 0, C = 0;
    avec<long long> ptr;
    avec<int> col;
    avec<double> val;
};

struct AmgLevel {
    int nblock = 0;            // block rows: particles on level 0, aggregates above
    int bs = 0;                // DOFs per block row: 3 on level 0, 6 above
    Bsr A;                     // operator of the level; empty on level 0 (the stiffness itself)
    std::vector<double> Dinv;  // inverse of each bs x bs diagonal block, row-major
    double omega = 1.0;        // smoother damping, 4/3 / rho(D^-1 A)
    Bsr P;                     // prolongation from the next level: bs x 6 blocks
    Bsr Pt;                    // its transpose (restriction): 6 x bs blocks
};

struct AmgHierarchy {
    std::vector<AmgLevel> levels;     // finest first; the coarsest operator is coarse_A
    Bsr coarse_A;                     // 6 x 6 blocks
    int coarse_n = 0;                 // scalar size of the coarsest operator
    std::vector<double> coarse_chol;  // dense lower Cholesky factor of coarse_A, row-major
    std::vector<double> coarse_inv;   // its dense inverse, row-major
};

// The stiffness in the device's block-CSR layout: block row i holds npad[i]
// blocks (nconn[i] real ones, then padding) at rowoff[i]; value (r, c) of
// block b is val[9 * rowoff[i] + (3 r + c) * npad[i] + b]; mask bit d of
// particle i set = DOF d free.  Constrained DOFs are removed (their rows and
// columns treated as zero).
struct AmgInput {
    int n = 0;
    const double *xyz = nullptr;      // initial positions, n x 3
    const uint8_t *mask = nullptr;
    const long long *rowoff = nullptr;
    const int *npad = nullptr;
    const int *nconn = nullptr;
    const int *cols = nullptr;
    const double *val = nullptr;
    const int *group = nullptr;       // specimen of each particle in a batch (null: one specimen);
                                      // aggregates never span two specimens
};

struct AmgOptions {
    double agg_spacing = 0.6;  // edge of a level-0 aggregate box (3 SC spacings at radius 0.1)
    int max_levels = 8;
    int coarse_blocks = 150;   // stop coarsening at this many block rows
    int power_iters = 15;      // power iterations for rho(D^-1 A)
    int max_coarse_dofs = 6000;  // largest coarsest operator factored densely
};

// Returns the number of levels above the coarsest; -1 when the coarsest
// operator is not positive definite, -2 when the coarsest operator would have
// more than max_coarse_dofs DOFs (the lattice did not coarsen).
int amg_build(const AmgInput &in, AmgHierarchy &H, const AmgOptions &opt = AmgOptions());

}  // namespace lpm
