"""The host-side smoothed-aggregation hierarchy (lpm-c_gb300/csrc/amg_setup.cpp)
on the CPU: built from the oracle's stiffness (the reference's FD matrix with
the boundary conditions of a load step) in the device block-CSR layout, then
used as the preconditioner of a CG in numpy (V-cycle as the device runs it:
two damped block-Jacobi sweeps before and after the coarse correction,
Galerkin coarse operators, the dense inverse on the coarsest level).  It must converge to 1e-10 in a small,
size-independent number of iterations where block-Jacobi PCG needs hundreds.
"""
import os
import subprocess

import numpy as np
import pytest
import scipy.sparse as sp

import cases

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "lpm-c_gb300", "csrc")


@pytest.fixture(scope="module")
def harness(tmp_path_factory):
    exe = str(tmp_path_factory.mktemp("amg") / "amg_harness")
    subprocess.check_call(["g++", "-O3", "-std=c++17", "-fopenmp", "-I", CSRC, "-o", exe,
                           os.path.join(ROOT, "tests", "amg_harness.cpp"), os.path.join(CSRC, "amg_setup.cpp")])
    return exe


def _system(O, lattice, size):
    o = O.Oracle()
    if lattice == 2:
        case = cases.SCCase(n=size)
        n = o.setup_lattice(case.lattice, case.radius, case.box)
        o.set_types(cases.sc_types(o.d("xyz", (n, 3)), o.i("nb", (n,)), case.radius))
        c11, c12, c44 = cases.iso_cubic(case.E, case.nu)
        o.set_material(c11, c12, c44, case.sigmay, case.H, 0.0, 0)
    else:
        case = cases.FCCCase(ncell=size)
        n = o.setup_lattice(case.lattice, case.radius, case.box)
        o.set_types(cases.sc_types(o.d("xyz", (n, 3)), o.i("nb", (n,)), case.radius))
        o.set_cp(*case.cp)
        o.set_material(case.C11, case.C12, case.C44, 0.0, 0.0, 0.0, 1)
    o.init_state()
    o.load_step(cases.sc_bcs(case.schedule[0]), [], 1e30, maxiter=0)  # BCs, predictor, stiffness
    nnz = o.nnz
    IK = o.i("IK", (3 * n + 1,)) - 1
    JK = o.i("JK", (nnz,)) - 1
    U = sp.csr_matrix((o.d("K_global", (nnz,)), JK, IK), shape=(3 * n, 3 * n))
    K = (U + sp.triu(U, 1).T).tocsr()
    dofmask = o.i("dispBC_index", (3 * n,)).reshape(n, 3)
    mask = (dofmask[:, 0] | (dofmask[:, 1] << 1) | (dofmask[:, 2] << 2)).astype(np.uint8)
    w = o.L.lo_nconn_max(o.h)
    conn, nconn = o.i("conn", (n, w)), o.i("nb_conn", (n,))
    return o, K, o.d("residual", (3 * n,)), o.d("xyz", (n, 3)), mask, conn, nconn


def _device_layout(K, conn, nconn):
    """Block-CSR as on the device: rows padded to 4 blocks with column i,
    values component-major per row."""
    n = len(nconn)
    npad = (nconn + 3) & ~3
    rowoff = np.zeros(n + 1, dtype=np.int64)
    rowoff[1:] = np.cumsum(npad)
    cols = np.repeat(np.arange(n, dtype=np.int32), npad)
    val = np.zeros(9 * rowoff[-1])
    I = np.repeat(np.arange(n), nconn)
    B = np.arange(len(I)) - np.repeat(np.cumsum(nconn) - nconn, nconn)
    J = conn[I, B]
    cols[rowoff[I] + B] = J
    for r in range(3):
        for c in range(3):
            val[9 * rowoff[I] + (3 * r + c) * npad[I] + B] = np.asarray(K[3 * I + r, 3 * J + c]).ravel()
    return rowoff, npad.astype(np.int32), cols, val


def _load_hierarchy(d):
    lines = open(os.path.join(d, "levels.txt")).read().split("\n")
    L, nc = map(int, lines[0].split())
    rd = lambda name, dt: np.fromfile(os.path.join(d, name), dtype=dt)  # noqa: E731

    def bsr(p, dims):
        nbr, nbc, R, C = dims
        if nbr == 0:
            return None
        ptr = rd(f"{p}_ptr.bin", np.int64)
        return sp.bsr_matrix((rd(f"{p}_val.bin", np.float64).reshape(-1, R, C), rd(f"{p}_col.bin", np.int32), ptr),
                             shape=(nbr * R, nbc * C)).tocsr()
    levels = []
    for lev in range(L):
        f = lines[1 + lev].split()
        nblock, bs, omega = int(f[0]), int(f[1]), float(f[2])
        dims = [tuple(map(int, f[3 + 4 * k:7 + 4 * k])) for k in range(3)]
        levels.append(dict(A=bsr(f"L{lev}_A", dims[0]), P=bsr(f"L{lev}_P", dims[1]),
                           Pt=bsr(f"L{lev}_Pt", dims[2]), bs=bs, omega=omega,
                           Dinv=rd(f"L{lev}_Dinv.bin", np.float64).reshape(nblock, bs, bs)))
    coarse = bsr("coarse_A", tuple(map(int, lines[1 + L].split())))
    return levels, coarse, rd("coarse_chol.bin", np.float64).reshape(nc, nc), rd("coarse_inv.bin", np.float64).reshape(nc, nc)


def _vcycle(levels, cinv, nu=1):
    """The V-cycle as the device runs it: on every level a damped block-Jacobi
    sweep from zero and nu - 1 more, the residual restricted, the coarse
    correction prolongated, nu sweeps; the coarsest level multiplies by the
    dense inverse."""
    def smooth(lv, x, b):
        r = (b - lv["A"] @ x).reshape(-1, lv["bs"])
        return x + lv["omega"] * np.einsum("nij,nj->ni", lv["Dinv"], r).ravel()

    def V(l, b):
        if l == len(levels):
            return cinv @ b
        lv = levels[l]
        x = lv["omega"] * np.einsum("nij,nj->ni", lv["Dinv"], b.reshape(-1, lv["bs"])).ravel()
        for _ in range(nu - 1):
            x = smooth(lv, x, b)
        x = x + lv["P"] @ V(l + 1, lv["Pt"] @ (b - lv["A"] @ x))
        for _ in range(nu):
            x = smooth(lv, x, b)
        return x
    return lambda r: V(0, r)


def _pcg(A, M, b, rtol=1e-10, maxit=5000):
    x = np.zeros_like(b)
    r = b.copy()
    z = M(r)
    p = z.copy()
    rz = r @ z
    bn = np.linalg.norm(b)
    for it in range(maxit):
        q = A @ p
        al = rz / (p @ q)
        x += al * p
        r -= al * q
        if np.linalg.norm(r) <= rtol * bn:
            return x, it + 1
        z = M(r)
        rz_old, rz = rz, r @ z
        p = z + (rz / rz_old) * p
    return x, maxit


@pytest.mark.parametrize("lattice,size,nu", [(2, 10, 1), (2, 16, 1), (2, 16, 2), (3, 6, 1), (3, 6, 3)])
def test_hierarchy_preconditions_cg(oracle_mod, harness, tmp_path, lattice, size, nu):
    o, K, res, xyz, mask, conn, nconn = _system(oracle_mod, lattice, size)
    n = len(nconn)
    rowoff, npad, cols, val = _device_layout(K, conn, nconn)
    d = str(tmp_path)
    open(os.path.join(d, "n.txt"), "w").write(str(n))
    for name, arr in (("xyz", xyz), ("mask", mask), ("rowoff", rowoff), ("npad", npad),
                      ("nconn", nconn.astype(np.int32)), ("cols", cols), ("val", val)):
        np.ascontiguousarray(arr).tofile(os.path.join(d, f"{name}.bin"))
    free = (np.repeat(mask[:, None], 3, axis=1) >> np.arange(3) & 1).ravel().astype(bool)
    b = res * free
    r4 = np.zeros((n, 4))
    r4[:, :3] = b.reshape(n, 3)
    r4.tofile(os.path.join(d, "r.bin"))  # the harness also applies the device's V-cycle to it
    subprocess.check_call([harness, d, "0.6", str(nu)])
    levels, coarse, chol, cinv = _load_hierarchy(d)
    assert len(levels) >= 1
    # level 0 operates with the stiffness, constrained rows and columns removed
    dfree = sp.diags(free.astype(float))
    A0 = (dfree @ K @ dfree).tocsr()
    levels[0]["A"] = A0
    for lv in levels[1:]:
        assert abs(lv["A"] - lv["A"].T).max() <= 1e-9 * abs(lv["A"]).max()
    # Galerkin products: each coarse operator is P^T A P of the level below
    ops = [lv["A"] for lv in levels] + [coarse]
    for l, lv in enumerate(levels):
        assert abs(lv["Pt"] - lv["P"].T).max() == 0.0
        G = (lv["Pt"] @ ops[l] @ lv["P"]).toarray()
        Ac = ops[l + 1].toarray()
        keep = np.abs(np.diag(G)) > 0  # coarse DOFs with a prolongation column
        assert np.allclose(Ac[np.ix_(keep, keep)], G[np.ix_(keep, keep)], rtol=1e-10, atol=1e-10 * abs(G).max())
        assert np.all(np.diag(Ac)[~keep] == 1.0)
    # constrained DOFs receive no prolongation
    assert abs(levels[0]["P"][~free]).max() == 0.0
    # the dense coarse factor and inverse
    assert np.allclose(chol @ chol.T, coarse.toarray() + np.diag((abs(coarse).sum(1).A1 == 0).astype(float)))
    assert np.allclose(cinv @ (chol @ chol.T), np.eye(len(cinv)), atol=1e-8)
    M = _vcycle(levels, cinv, nu)
    # the device's launch sequence and per-row arithmetic (emulated on the
    # host) give the numpy V-cycle's result; an index error would show as an
    # O(1) difference
    z = M(b)
    z64 = np.fromfile(os.path.join(d, "z.bin")).reshape(n, 4)
    z32 = np.fromfile(os.path.join(d, "z32.bin")).reshape(n, 4)
    assert np.all(z64[:, 3] == 0.0) and np.all(z64[:, :3].ravel()[~free] == 0.0)
    # (z32: the whole cycle in FP32 as the device runs it; agreement to FP32
    # rounding)
    assert np.abs(z64[:, :3].ravel() - z).max() <= 1e-5 * np.abs(z).max()
    assert np.abs(z32[:, :3].ravel() - z).max() <= 1e-4 * np.abs(z).max()
    x, it = _pcg(A0, M, b)
    # with P and P^T rounded to FP32 as the device keeps them, the cycle stays
    # symmetric and converges as fast
    lv32 = [dict(lv, P=lv["P"].astype(np.float32).astype(np.float64),
                 Pt=lv["Pt"].astype(np.float32).astype(np.float64)) for lv in levels]
    _, it32 = _pcg(A0, _vcycle(lv32, cinv, nu), b)
    assert it32 <= it + 1, (it, it32)
    Kf = K[free][:, free]
    assert np.linalg.norm(Kf @ x[free] - b[free]) <= 1e-10 * np.linalg.norm(b)
    # block-Jacobi PCG on the same system for reference
    dinv = levels[0]["Dinv"]
    _, it_bj = _pcg(A0, lambda r: np.einsum("nij,nj->ni", dinv, r.reshape(-1, 3)).ravel(), b)
    assert it <= 30 and it * 5 < it_bj, (it, it_bj)


def test_single_level_is_the_exact_inverse(oracle_mod, harness, tmp_path):
    """A lattice of at most 150 particles does not coarsen: the V-cycle is the
    dense inverse of the stiffness with the constrained DOFs removed."""
    o, K, res, xyz, mask, conn, nconn = _system(oracle_mod, 2, 4)
    n = len(nconn)
    assert n <= 150
    rowoff, npad, cols, val = _device_layout(K, conn, nconn)
    d = str(tmp_path)
    open(os.path.join(d, "n.txt"), "w").write(str(n))
    for name, arr in (("xyz", xyz), ("mask", mask), ("rowoff", rowoff), ("npad", npad),
                      ("nconn", nconn.astype(np.int32)), ("cols", cols), ("val", val)):
        np.ascontiguousarray(arr).tofile(os.path.join(d, f"{name}.bin"))
    free = (np.repeat(mask[:, None], 3, axis=1) >> np.arange(3) & 1).ravel().astype(bool)
    b = res * free
    r4 = np.zeros((n, 4))
    r4[:, :3] = b.reshape(n, 3)
    r4.tofile(os.path.join(d, "r.bin"))
    subprocess.check_call([harness, d, "0.6"])
    levels, coarse, chol, cinv = _load_hierarchy(d)
    assert levels == [] and cinv.shape == (3 * n, 3 * n)
    z = np.fromfile(os.path.join(d, "z.bin")).reshape(n, 4)[:, :3].ravel()
    x = np.zeros(3 * n)
    x[free] = np.linalg.solve(K[free][:, free].toarray(), b[free])
    assert np.abs(z - x).max() <= 1e-9 * np.abs(x).max()


def test_hierarchy_independent_of_thread_count(oracle_mod, harness, tmp_path):
    """Every output of the build is laid out by counting passes and summed in
    row order: 1 and 5 threads give the same bytes."""
    o, K, res, xyz, mask, conn, nconn = _system(oracle_mod, 2, 16)
    n = len(nconn)
    rowoff, npad, cols, val = _device_layout(K, conn, nconn)
    outs = []
    for threads in (1, 5):
        d = tmp_path / f"t{threads}"
        d.mkdir()
        open(d / "n.txt", "w").write(str(n))
        for name, arr in (("xyz", xyz), ("mask", mask), ("rowoff", rowoff), ("npad", npad),
                          ("nconn", nconn.astype(np.int32)), ("cols", cols), ("val", val)):
            np.ascontiguousarray(arr).tofile(d / f"{name}.bin")
        subprocess.check_call([harness, str(d), "0.6"], env=dict(os.environ, OMP_NUM_THREADS=str(threads)))
        outs.append({p.name: p.read_bytes() for p in sorted(d.iterdir()) if p.name.startswith(("L", "coarse"))})
    assert outs[0].keys() == outs[1].keys() and len(outs[0]) > 5
    assert all(outs[0][k] == outs[1][k] for k in outs[0])


def test_batch_groups_keep_specimens_apart(oracle_mod, harness, tmp_path):
    """Two specimens at the same place in space, as a batch puts them: with a
    specimen id per particle, no aggregate spans both, every level stays
    block-diagonal over the specimens (as per-specimen CG scalars need), and
    the V-cycle PCG converges as for one specimen."""
    o, K, res, xyz, mask, conn, nconn = _system(oracle_mod, 2, 12)
    n = len(nconn)
    rowoff, npad, cols, val = _device_layout(K, conn, nconn)
    rowoff2 = np.concatenate([rowoff, rowoff[1:] + rowoff[-1]])
    d = tmp_path
    open(d / "n.txt", "w").write(str(2 * n))
    group = np.repeat(np.arange(2, dtype=np.int32), n)
    for name, arr in (("xyz", np.vstack([xyz, xyz])), ("mask", np.concatenate([mask, mask])),
                      ("rowoff", rowoff2), ("npad", np.concatenate([npad, npad])),
                      ("nconn", np.concatenate([nconn, nconn]).astype(np.int32)),
                      ("cols", np.concatenate([cols, cols + n]).astype(np.int32)),
                      ("val", np.concatenate([val, val])), ("group", group)):
        np.ascontiguousarray(arr).tofile(d / f"{name}.bin")
    subprocess.check_call([harness, str(d), "0.6"])
    levels, coarse, chol, cinv = _load_hierarchy(str(d))
    assert len(levels) >= 1
    g = np.repeat(group, 3)  # specimen of each level-0 DOF
    for lv in levels:
        P = lv["P"].tocoo()
        owner = np.full(P.shape[1], -1)
        for r, c in zip(P.row, P.col):
            assert owner[c] in (-1, g[r]), "an aggregate spans two specimens"
            owner[c] = g[r]
        g = np.where(owner < 0, 0, owner)  # specimen of each coarse DOF (empty columns: either)
    # block-diagonal coarsest operator: no entry couples the two specimens
    C = coarse.tocoo()
    assert np.all(g[C.row] == g[C.col])
    free = (np.repeat(np.concatenate([mask, mask])[:, None], 3, axis=1) >> np.arange(3) & 1).ravel().astype(bool)
    K2 = sp.block_diag([K, K]).tocsr()
    dfree = sp.diags(free.astype(float))
    levels[0]["A"] = (dfree @ K2 @ dfree).tocsr()
    b = np.concatenate([res, 0.5 * res]) * free
    _, it = _pcg(levels[0]["A"], _vcycle(levels, cinv, 1), b)
    assert it <= 30, it


def test_notched_plate(oracle_mod, harness, tmp_path):
    """Irregular geometry: the notched plate of the gradient workload (24 x 3 x
    28 particles, notch 6 deep, seed-1 fields).  Aggregates are cut by the
    notch and by the three-layer thickness; the V-cycle PCG still converges
    in a few iterations where block-Jacobi needs hundreds (14 against 582)."""
    plate = cases.NotchedPlate(nx=24, ny=3, nz=28, notch=6, steps=4, strain=0.006, corr=3.0)
    o = oracle_mod.Oracle()
    n = o.setup_particles(plate.lattice, plate.radius, plate.xyz)
    o.set_types(cases.sc_types(o.d("xyz", (n, 3)), o.i("nb", (n,)), plate.radius))
    E, nu, sy, H = plate.fields(1)
    c11, c12, c44 = cases.iso_cubic(E, nu)
    o.set_material(c11, c12, c44, sy, H, 0.0, 0)
    o.init_state()
    o.load_step(plate.step_bcs()[0], [], 1e30, maxiter=0)
    nnz = o.nnz
    U = sp.csr_matrix((o.d("K_global", (nnz,)), o.i("JK", (nnz,)) - 1, o.i("IK", (3 * n + 1,)) - 1),
                      shape=(3 * n, 3 * n))
    K = (U + sp.triu(U, 1).T).tocsr()
    dm = o.i("dispBC_index", (3 * n,)).reshape(n, 3)
    mask = (dm[:, 0] | (dm[:, 1] << 1) | (dm[:, 2] << 2)).astype(np.uint8)
    conn, nconn = o.i("conn", (n, o.L.lo_nconn_max(o.h))), o.i("nb_conn", (n,))
    rowoff, npad, cols, val = _device_layout(K, conn, nconn)
    d = tmp_path
    open(d / "n.txt", "w").write(str(n))
    for name, arr in (("xyz", o.d("xyz", (n, 3))), ("mask", mask), ("rowoff", rowoff), ("npad", npad),
                      ("nconn", nconn.astype(np.int32)), ("cols", cols), ("val", val)):
        np.ascontiguousarray(arr).tofile(d / f"{name}.bin")
    subprocess.check_call([harness, str(d), "0.6"])
    levels, coarse, chol, cinv = _load_hierarchy(str(d))
    free = (np.repeat(mask[:, None], 3, axis=1) >> np.arange(3) & 1).ravel().astype(bool)
    dfree = sp.diags(free.astype(float))
    levels[0]["A"] = (dfree @ K @ dfree).tocsr()
    b = o.d("residual", (3 * n,)) * free
    x, it = _pcg(levels[0]["A"], _vcycle(levels, cinv, 1), b)
    Kf = K[free][:, free]
    assert np.linalg.norm(Kf @ x[free] - b[free]) <= 1e-10 * np.linalg.norm(b)
    assert it <= 25, it
