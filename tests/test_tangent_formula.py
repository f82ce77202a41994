"""The analytic elastic tangent assembled by lpm-c_gb300/csrc/k_stiff.cu
(k_tgeom + k_assemble), restated term by term in numpy, against the
reference's forward-difference stiffness (calcStiffness3DFiniteDifference,
src/stiffness.c:384-516, restated by the oracle) on SC and FCC lattices at a
deformed configuration.  This pins the derivation on the CPU for both
lattices; the GPU tests compare the kernels themselves with the same matrix.

Per bond j of particle i (partner p, shell s, unit vector c, length d):
  K_ii += (F_ij/d)(I - c c^T) + 2Kn c c^T + c (x) a_j
  K_ip += -(Fbar_ij/d)(I - c c^T) - 2Kn c c^T + c (x) b_j - a_j (x) c
  K_iq += -(Tv_pq + Tv_ij)/2 c (x) c_pq   for q a shell-s neighbour of p
with a_j = (W_i^s + Tv_ij U_i^s)/2, b_j = (W_p^s + Tv_ij U_p^s)/2, U and W the
plain and Tv-weighted sums of shell-s unit vectors.
"""
import numpy as np
import pytest

import cases


def _oracle_after_steps(O, case, steps, plmode):
    O.set_threads(1)
    o = O.Oracle()
    n = o.setup_lattice(case.lattice, case.radius, case.box)
    o.set_types(cases.sc_types(o.d("xyz", (n, 3)), o.i("nb", (n,)), case.radius))
    if plmode == 1:
        o.set_cp(*case.cp)
        o.set_material(case.C11, case.C12, case.C44, 0.0, 0.0, 0.0, 1)
    else:
        C11, C12, C44 = cases.iso_cubic(case.E, case.nu)
        o.set_material(C11, C12, C44, case.sigmay, case.H, 0.0, 0)
    o.init_state()
    for stp in case.schedule[:steps]:
        o.load_step(cases.sc_bcs(stp), [], 1e-10, 100, 1e-22, 0.0)
    return o


def analytic_tangent(o, damaged=False):
    """Full (both triangles) 3n x 3n tangent, restricted to each row's AFEM
    connectivity like the reference's pattern.  damaged: weigh bonds by
    damage_broken as k_stiff.cu does with the damage stage on (broken bonds
    leave the shell sums, their own terms and the two-hop terms through
    them; a pair counts only when both directions are intact)."""
    n, nn = o.n, o.nn
    xyz = o.d("xyz", (n, 3))
    nbr = o.i("neighbors", (n, nn))
    sh = o.i("nsign", (n, nn))
    nb = o.i("nb", (n,))
    L0 = o.d("distance_initial", (n, nn))
    Kn = o.d("Kn", (n, nn))
    Tv = o.d("Tv", (n, nn))
    dLp = o.d("dLp0", (n, nn))  # plastic bond stretch, state slot 0
    brk = o.d("damage_broken", (n, nn)) if damaged else np.ones((n, nn))
    conn = o.i("conn", (n, o.L.lo_nconn_max(o.h)))
    nconn = o.i("nb_conn", (n,))
    dL = np.zeros((n, nn))
    c = np.zeros((n, nn, 3))
    S = np.zeros((n, 2))
    T = np.zeros((n, 2))
    U = np.zeros((n, 2, 3))
    W = np.zeros((n, 2, 3))
    rev = -np.ones((n, nn), dtype=int)
    for i in range(n):
        for j in range(nb[i]):
            p = nbr[i, j]
            e = xyz[i] - xyz[p]
            dis = np.sqrt(e @ e)
            dL[i, j] = (dis - L0[i, j] - dLp[i, j]) * brk[i, j]
            c[i, j] = e / dis
            s = sh[i, j]
            S[i, s] += dL[i, j]
            T[i, s] += Tv[i, j] * dL[i, j]
            U[i, s] += brk[i, j] * c[i, j]
            W[i, s] += brk[i, j] * Tv[i, j] * c[i, j]
            hits = np.nonzero(nbr[p, :nb[p]] == i)[0]
            if hits.size:
                rev[i, j] = hits[-1]
    K = np.zeros((3 * n, 3 * n))
    for i in range(n):
        cs = set(conn[i, :nconn[i]].tolist())
        kii = np.zeros((3, 3))
        for j in range(nb[i]):
            p, s, cc = nbr[i, j], sh[i, j], c[i, j]
            if brk[i, j] * (brk[p, rev[i, j]] if rev[i, j] >= 0 else 1.0) == 0.0:
                continue
            d = np.linalg.norm(xyz[i] - xyz[p])
            kn, tv = Kn[i, j], Tv[i, j]
            tsum, ssum = T[i, s] + T[p, s], S[i, s] + S[p, s]
            dlji = dL[p, rev[i, j]] if rev[i, j] >= 0 else dL[i, j]
            fel = 2 * kn * dL[i, j] + 0.5 * tsum + 0.5 * tv * ssum
            fbar = kn * (dL[i, j] + dlji) + 0.5 * tsum + 0.5 * tv * ssum
            a = 0.5 * (W[i, s] + tv * U[i, s])
            b = 0.5 * (W[p, s] + tv * U[p, s])
            proj = np.eye(3) - np.outer(cc, cc)
            kii += fel / d * proj + 2 * kn * np.outer(cc, cc) + np.outer(cc, a)
            if p in cs:
                K[3 * i:3 * i + 3, 3 * p:3 * p + 3] += (-fbar / d * proj - 2 * kn * np.outer(cc, cc)
                                                        + np.outer(cc, b) - np.outer(a, cc))
            for m in range(nb[p]):
                if sh[p, m] != s or brk[p, m] == 0.0:
                    continue
                q = nbr[p, m]
                blk = -0.5 * (Tv[p, m] + tv) * np.outer(cc, c[p, m])
                if q == i:
                    kii += blk
                elif q in cs:
                    K[3 * i:3 * i + 3, 3 * q:3 * q + 3] += blk
        K[3 * i:3 * i + 3, 3 * i:3 * i + 3] += kii
    return K


@pytest.mark.parametrize("lattice", ["sc", "fcc"])
def test_analytic_tangent_matches_reference_fd(oracle_mod, lattice):
    if lattice == "sc":
        case, plmode, steps = cases.SCCase(n=4, sigmay=150.0), 0, 3
    else:
        case, plmode, steps = cases.FCCCase(ncell=2), 1, 3
    o = _oracle_after_steps(oracle_mod, case, steps, plmode)
    K = analytic_tangent(o)
    n = o.n
    # symmetric: the averaged force in the off-diagonal geometric term is
    # the reference's 0.5 (K_ik + K_ki^T)
    assert np.linalg.norm(K - K.T) <= 1e-12 * np.linalg.norm(K)
    o.fd_stiffness()
    nnz = o.nnz
    IK = o.i("IK", (3 * n + 1,)) - 1
    JK = o.i("JK", (nnz,)) - 1
    Kfd = o.d("K_global", (nnz,))
    rows = np.repeat(np.arange(3 * n), np.diff(IK))
    Ku = K[rows, JK]
    # the deformed state carries bond forces (geometric terms are active)
    assert np.abs(o.d("F", (n, o.nn))).max() > 0.0
    rel = np.linalg.norm(Ku - Kfd) / np.linalg.norm(Kfd)
    # forward differences with h = 1e-6 r: truncation ~1e-7 relative here
    assert rel < 1e-5, rel
    # and the tangent is not trivially the FD matrix of the rest state
    o2 = _oracle_after_steps(oracle_mod, case, 0, plmode)
    o2.fd_stiffness()
    assert np.linalg.norm(o2.d("K_global", (nnz,)) - Kfd) > 100 * rel * np.linalg.norm(Kfd)


@pytest.mark.parametrize("which,steps", [("ductile", 6), ("brittle", 6)])
def test_damaged_tangent_matches_reference_fd(oracle_mod, which, steps):
    """With broken bonds (the damage stage of the reference's main, restated by
    the oracle): the tangent with the broken-bond weights against the FD
    stiffness of the damaged state, and the undamaged formula far from it."""
    from test_oracle_damage import _brittle, _ductile
    o, _, step_bcs, tol = (_ductile if which == "ductile" else _brittle)(oracle_mod)
    for bcs in step_bcs[:steps]:
        o.load_step_damage(bcs, [], tol, 200, 1e-20, 0.0, 50)
    n = o.n
    assert (o.d("damage_broken", (n, o.nn)) == 0.0).sum() > 0
    o.fd_stiffness()
    nnz = o.nnz
    IK = o.i("IK", (3 * n + 1,)) - 1
    JK = o.i("JK", (nnz,)) - 1
    Kfd = o.d("K_global", (nnz,))
    rows = np.repeat(np.arange(3 * n), np.diff(IK))
    rel = np.linalg.norm(analytic_tangent(o, damaged=True)[rows, JK] - Kfd) / np.linalg.norm(Kfd)
    rel0 = np.linalg.norm(analytic_tangent(o)[rows, JK] - Kfd) / np.linalg.norm(Kfd)
    assert rel < 1e-5, rel
    assert rel0 > 1e-2, rel0
