"""The oracle (CPU restatement) against golden vectors produced by the LPM-C
reference itself (tests/golden/make_golden.py, reference built from its own
sources).  Everything here is bit-exact: same inputs, same operation order,
same BLAS/CG shim.
"""
import os

import numpy as np
import pytest

import cases
from conftest import golden
from setup_helpers import sc_oracle


@pytest.fixture(scope="module")
def sc10(oracle_mod):
    case = cases.SCCase(n=10)
    o, types = sc_oracle(oracle_mod, case, threads=1)
    return case, o, types


def test_setup_bit_exact(sc10):
    case, o, types = sc10
    g = golden("sc10_setup.npz")
    n, nn = o.n, o.nn
    assert n == 1000
    assert np.array_equal(g["xyz"], o.d("xyz_initial", (n, 3)))
    assert np.array_equal(g["types"], types)
    assert np.array_equal(g["neighbors"], o.i("neighbors", (n, nn)))
    assert np.array_equal(g["nsign"], o.i("nsign", (n, nn)))
    assert np.array_equal(g["nb"], o.i("nb", (n,)))
    for k in ("distance_initial", "csx_initial", "csy_initial", "csz_initial", "Kn", "Tv"):
        assert np.array_equal(g[k], o.d(k, (n, nn))), k
    assert np.array_equal(g["conn"], o.i("conn", (n, 61)))
    assert np.array_equal(g["nb_conn"], o.i("nb_conn", (n,)))
    kp = g["K_pointer"]
    assert np.array_equal(kp[:n, 0], o.i("kp0", (n + 1,))[:n])
    assert np.array_equal(kp[:, 1], o.i("kp1", (n + 1,)))


def test_fd_stiffness_rest_bit_exact(oracle_mod):
    case = cases.SCCase(n=10)
    o, _ = sc_oracle(oracle_mod, case, threads=1)
    g = golden("sc10_K_step1.npz")
    o.fd_stiffness()
    nnz = o.nnz
    assert np.array_equal(g["IK"], o.i("IK", (3 * o.n + 1,)))
    assert np.array_equal(g["JK"], o.i("JK", (nnz,)))
    assert np.array_equal(g["K_global"], o.d("K_global", (nnz,)))


def test_fd_stiffness_plastic_state_bit_exact(oracle_mod):
    """K at the converged state entering step 14 (plastic stretches present)."""
    case = cases.SCCase(n=10)
    o, _ = sc_oracle(oracle_mod, case, threads=1)
    g = golden("sc10_K_step14.npz")
    o.set_d("xyz", g["in_xyz"])
    o.set_d("dLp0", g["in_dLp"])
    o.fd_stiffness()
    assert np.array_equal(g["K_global"], o.d("K_global", (o.nnz,)))


def restore(o, g, s):
    """Restore the converged end-of-step state of snapshot s into the oracle."""
    for slot in ("0", "1", "2"):
        o.set_d("dLp" + slot, g[f"s{s}_dLp"])
        o.set_d("alpha" + slot, g[f"s{s}_alpha"])
        o.set_d("beta" + slot, g[f"s{s}_beta"])
    o.set_d("xyz", g[f"s{s}_xyz"])
    o.set_d("F", g[f"s{s}_F"])
    for c in ("csx", "csy", "csz"):
        o.set_d(c, g[f"s{s}_{c}"])
    o.set_d("Pex", g[f"s{s}_Pex"])


def test_cyclic_start_bit_exact(oracle_mod):
    """First 14 load steps (elastic ramp into yield) of the C1 cyclic case."""
    case = cases.SCCase(n=10)
    o, types = sc_oracle(oracle_mod, case, threads=1)
    g = golden("sc10_cyclic.npz")
    n = o.n
    x0 = o.d("xyz_initial", (n, 3))
    top = types == cases.T_TOP
    for k, stp in enumerate(case.schedule[:14]):
        st = o.load_step(cases.sc_bcs(stp), [], case.newton_tol, 100, 1e-20, 0.0)
        assert st[0] == g["iters"][k]
        xyz = o.d("xyz", (n, 3))
        assert (xyz[top, 2].sum() - x0[top, 2].sum()) / top.sum() == g["disp_top"][k]
        F = o.d("F", (n, 18))
        csz = o.d("csz", (n, 18))
        assert np.sum(-csz[top] * F[top]) == g["react_top"][k]
    for key in ("xyz", "alpha", "dLp", "stress"):
        name = {"alpha": "alpha1", "dLp": "dLp1", "stress": "stress_tensor"}.get(key, key)
        shape = g[f"s14_{key}"].shape
        assert np.array_equal(g[f"s14_{key}"], o.d(name, shape)), key


def test_resume_from_checkpoint_bit_exact(oracle_mod):
    """Restart from the converged state after step 20 and replay steps 21-22."""
    case = cases.SCCase(n=10)
    o, types = sc_oracle(oracle_mod, case, threads=1)
    g = golden("sc10_cyclic.npz")
    restore(o, g, 20)
    n = o.n
    x0 = o.d("xyz_initial", (n, 3))
    top = types == cases.T_TOP
    for k in (20, 21):
        st = o.load_step(cases.sc_bcs(case.schedule[k]), [], case.newton_tol, 100, 1e-20, 0.0)
        assert st[0] == g["iters"][k]
        xyz = o.d("xyz", (n, 3))
        assert (xyz[top, 2].sum() - x0[top, 2].sum()) / top.sum() == g["disp_top"][k]


def test_radial_return_closed_form(oracle_mod):
    """J2 radial return under a homogeneous strain: with the trial stress
    recomputed independently in numpy from the bond forces
    (src/constitutive.c:526-567), the multiplier is the closed form
    dlambda = (sigma_eq - sigma_y) / (3 G + H) (:591-596) and the plastic
    bond stretch is L0 * (dlambda 1.5 s/sigma_eq) : n n (:601-621)."""
    case = cases.SCCase(n=8)
    o, types = sc_oracle(oracle_mod, case, threads=1)
    n, nn = o.n, o.nn
    X = o.d("xyz_initial", (n, 3))
    eps = np.array([[1.5e-3, 2e-4, 0.0], [2e-4, -4e-4, 1e-4], [0.0, 1e-4, -4e-4]])
    x = X + X @ eps.T
    o.set_d("xyz", x)
    o.force(0)
    nbr, shell, nb = o.i("neighbors", (n, nn)), o.i("nsign", (n, nn)), o.i("nb", (n,))
    L0, Kn, Tv, opp = (o.d(k, (n, nn)) for k in ("distance_initial", "Kn", "Tv", "opp"))
    vol = (2 * case.radius) ** 3
    c44 = cases.iso_cubic(case.E, case.nu)[2]
    dl = o.d("J2_dlambda", (n,))
    dlp = o.d("dLp2", (n, nn))
    checked = 0
    for i in np.nonzero(nb == 18)[0][:20]:
        d = x[i] - x[nbr[i]]
        dis = np.linalg.norm(d, axis=1)
        c = d / dis[:, None]
        dL = dis - L0[i]
        S = np.array([dL[shell[i] == s].sum() for s in (0, 1)])
        T = np.array([(Tv[i] * dL)[shell[i] == s].sum() for s in (0, 1)])
        F = 2 * Kn[i] * dL + T[shell[i]] + Tv[i] * S[shell[i]]
        w = opp[i] / vol * L0[i] * F
        st = np.array([np.sum(w * c[:, 0] ** 2), np.sum(w * c[:, 1] ** 2), np.sum(w * c[:, 2] ** 2),
                       np.sum(w * c[:, 1] * c[:, 2]), np.sum(w * c[:, 0] * c[:, 2]), np.sum(w * c[:, 0] * c[:, 1])])
        s = st.copy()
        s[:3] -= st[:3].mean()
        seq = np.sqrt(1.5 * (np.sum(s[:3] ** 2) + 2 * np.sum(s[3:] ** 2)))
        assert seq > case.sigmay
        want = (seq - case.sigmay) / (3 * c44 + case.H)
        assert abs(dl[i] - want) <= 1e-10 * want
        e = want * 1.5 * s / seq
        ddlp = L0[i] * (e[0] * c[:, 0] ** 2 + e[1] * c[:, 1] ** 2 + e[2] * c[:, 2] ** 2 +
                        2 * e[3] * c[:, 1] * c[:, 2] + 2 * e[4] * c[:, 0] * c[:, 2] + 2 * e[5] * c[:, 0] * c[:, 1])
        assert np.allclose(dlp[i], ddlp, rtol=1e-9, atol=1e-18)
        checked += 1
    assert checked == 20


def fcc_oracle(O, case, threads=1):
    O.set_threads(threads)
    o = O.Oracle()
    n = o.setup_lattice(case.lattice, case.radius, case.box)
    types = cases.sc_types(o.d("xyz", (n, 3)), o.i("nb", (n,)), case.radius)
    o.set_types(types)
    o.set_cp(*case.cp)
    o.set_material(case.C11, case.C12, case.C44, 0.0, 0.0, 0.0, 1)
    o.init_state()
    return o, types


def test_fcc_cp_bit_exact(oracle_mod):
    """FCC crystal plasticity (computeBondForceCPMiehe) on 4^3 cells, [001]
    tension, 12 steps (8 elastic, 4 plastic): the oracle reproduces the
    reference's iterations, displacements, reactions and slip state."""
    g = golden("fcc4_cp.npz")
    case = cases.FCCCase(ncell=4)
    o, types = fcc_oracle(oracle_mod, case)
    n, nn = o.n, o.nn
    assert np.array_equal(g["types"], types)
    assert np.array_equal(g["neighbors"], o.i("neighbors", (n, nn)))
    assert np.array_equal(g["Kn"], o.d("Kn", (n, nn)))
    ns = 24
    assert np.array_equal(g["schmid"], o.d("schmid", (ns, 6)))
    assert np.array_equal(g["cp_Cab"], o.d("cp_Cab", (n, ns * ns)))
    x0 = o.d("xyz_initial", (n, 3))
    top = types == cases.T_TOP
    for k, stp in enumerate(g["schedule"]):
        st = o.load_step(cases.sc_bcs(stp), [], case.newton_tol, 100, 1e-20, 0.0)
        assert st[0] == g["iters"][k], k
        xyz = o.d("xyz", (n, 3))
        assert (xyz[top, 2].sum() - x0[top, 2].sum()) / top.sum() == g["disp_top"][k]
    last = len(g["schedule"])
    assert np.array_equal(g[f"s{last}_cp_gy"], o.d("cp_gy1", (n, ns)))
    assert np.array_equal(g[f"s{last}_cp_A"], o.d("cp_A1", (n,)))
    assert np.array_equal(g[f"s{last}_dLp"], o.d("dLp1", (n, nn)))
    assert o.d("cp_A1", (n,)).max() > 0.0


def test_fcc_cp_latent_saturating_bit_exact(oracle_mod):
    """Crystal plasticity with latent hardening (q = 1.2) and a finite
    saturation stress (taus = 150 MPa), 4^3 cells, 9 steps (the 9th plastic):
    the oracle reproduces the reference's iterations, residuals,
    displacements and slip state (tests/golden/fcc4_sat_cp.npz).  Latent
    hardening changes the plastic step (residual 3.61e-7 against 3.71e-7
    with q = 1); the reference's modified Newton stops converging from the
    next step on, so the case ends there."""
    g = golden("fcc4_sat_cp.npz")
    case = cases.FCCCase(ncell=4, **cases.FCC_SAT)
    assert np.array_equal(g["cp"], np.array(case.cp))
    o, types = fcc_oracle(oracle_mod, case)
    n, nn = o.n, o.nn
    ns = 24
    assert np.array_equal(g["cp_Cab"], o.d("cp_Cab", (n, ns * ns)))
    x0 = o.d("xyz_initial", (n, 3))
    top = types == cases.T_TOP
    for k, stp in enumerate(g["schedule"]):
        st = o.load_step(cases.sc_bcs(stp), [], case.newton_tol, 100, 1e-20, 0.0)
        assert st[0] == g["iters"][k] and st[3] == g["nres"][k], k
        xyz = o.d("xyz", (n, 3))
        assert (xyz[top, 2].sum() - x0[top, 2].sum()) / top.sum() == g["disp_top"][k]
    last = len(g["schedule"])
    assert np.array_equal(g[f"s{last}_xyz"], o.d("xyz", (n, 3)))
    assert np.array_equal(g[f"s{last}_cp_gy"], o.d("cp_gy1", (n, ns)))
    assert np.array_equal(g[f"s{last}_cp_A_single"], o.d("cp_As1", (n, ns)))
    assert np.array_equal(g[f"s{last}_cp_A"], o.d("cp_A1", (n,)))
    assert np.array_equal(g[f"s{last}_dLp"], o.d("dLp1", (n, nn)))
    assert o.d("cp_A1", (n,)).max() > 0.0


def test_fcc_schmid_factors_001():
    """[001] tension: 8 of the 24 signed {111}<110> systems carry the Schmid
    factor 1/sqrt(6) (both signs of the 4 loaded slip directions... here: the
    positive ones), the others are 0 or negative."""
    g = golden("fcc4_cp.npz")
    m = g["schmid"][:, 2]  # resolved shear factor of sigma_zz
    assert np.isclose(m.max(), 1 / np.sqrt(6))
    assert np.sum(np.isclose(m, 1 / np.sqrt(6))) == 8
    assert np.sum(np.isclose(m, -1 / np.sqrt(6))) == 8
    assert np.sum(np.isclose(m, 0.0)) == 8


def test_force_bc_bit_exact(oracle_mod):
    """Force-controlled SC J2 case (setForceBC, src/boundary.c:50-70): a
    top-face force ramp with x and z components into the plastic range."""
    case = cases.ForceCase()
    o, types = sc_oracle(oracle_mod, case, threads=1)
    g = golden("sc_force.npz")
    n = o.n
    assert np.array_equal(types, g["types"])
    x0 = o.d("xyz_initial", (n, 3))
    top = types == cases.T_TOP
    disp, force = case.bcs()
    for k in range(case.steps):
        st = o.load_step(disp, force, case.newton_tol, 100, 1e-20, 0.0)
        assert st[0] == g["iters"][k], k
        assert st[1] == g["nres0"][k] and st[2] == g["nreac0"][k], k
        xyz = o.d("xyz", (n, 3))
        assert (xyz[top, 0].sum() - x0[top, 0].sum()) / top.sum() == g["disp_top_x"][k], k
        assert (xyz[top, 2].sum() - x0[top, 2].sum()) / top.sum() == g["disp_top_z"][k], k
    assert np.array_equal(o.d("xyz", (n, 3)), g["s_xyz"])
    assert np.array_equal(o.d("alpha1", (n,)), g["s_alpha"])
    assert g["s_alpha"].max() > 0.0
    assert np.array_equal(o.d("Pex", (3 * n,)), g["s_Pex"])
    assert np.array_equal(o.d("F", (n, 18)), g["s_F"])


@pytest.mark.parametrize("name", sorted(cases.SETUP_SHAPES))
def test_setup_shapes_bit_exact(oracle_mod, name):
    """Bond lists, AFEM connectivity and K_pointer of the 20^3 SC cube and of
    ragged SC and FCC boxes (searchNormalNeighbor, searchAFEMNeighbor)."""
    lattice, radius, box = cases.SETUP_SHAPES[name]
    g = golden(f"setup_{name}.npz")
    o = oracle_mod.Oracle()
    n = o.setup_lattice(lattice, radius, box)
    nn = o.nn
    assert n == g["xyz"].shape[0]
    assert np.array_equal(o.d("xyz", (n, 3)), g["xyz"])
    assert np.array_equal(o.i("neighbors", (n, nn)), g["neighbors"])
    assert np.array_equal(o.i("nsign", (n, nn)), g["nsign"])
    assert np.array_equal(o.i("nb", (n,)), g["nb"])
    assert np.array_equal(o.d("distance_initial", (n, nn)), g["distance_initial"])
    for k in ("x", "y", "z"):
        assert np.array_equal(o.d(f"cs{k}_initial", (n, nn)), g[f"cs{k}_initial"])
    w = g["conn"].shape[1]
    assert np.array_equal(o.i("conn", (n, w)), g["conn"])
    assert np.array_equal(o.i("nb_conn", (n,)), g["nb_conn"])
    kp = g["K_pointer"]
    assert np.array_equal(o.i("kp0", (n + 1,))[:n], kp[:n, 0])
    assert np.array_equal(o.i("kp1", (n + 1,)), kp[:, 1])


def test_per_particle_moduli_bit_exact(oracle_mod):
    """Per-particle E (the C2 material model at 8^3): bond Kn/Tv as the
    averages of the two end particles (src/stiffness.c:186-200), then 14 cyclic
    steps into the plastic range.  The reference ran with one type per particle
    and the usual types as BC groups; the oracle takes per-particle moduli."""
    case = cases.SCCase(n=8, sigmay=150.0, e_noise=0.05, seed=1)
    g = golden("sc8_enoise.npz")
    o, types = sc_oracle(oracle_mod, case, threads=1)
    n, nn = o.n, o.nn
    assert np.array_equal(types, g["groups"])
    assert np.array_equal(o.d("Kn", (n, nn)), g["Kn"])
    assert np.array_equal(o.d("Tv", (n, nn)), g["Tv"])
    x0 = o.d("xyz_initial", (n, 3))
    top = types == cases.T_TOP
    for k, stp in enumerate(case.schedule[:14]):
        st = o.load_step(cases.sc_bcs(stp), [], case.newton_tol, 100, 1e-20, 0.0)
        assert st[0] == g["iters"][k] and st[3] == g["nres"][k], k
        xyz = o.d("xyz", (n, 3))
        assert (xyz[top, 2].sum() - x0[top, 2].sum()) / top.sum() == g["disp_top"][k], k
    assert np.array_equal(o.d("xyz", (n, 3)), g["s_xyz"])
    assert np.array_equal(o.d("alpha1", (n,)), g["s_alpha"])
    assert np.array_equal(o.d("F", (n, nn)), g["s_F"])
    assert g["s_alpha"].max() > 0.0


def test_kinematic_hardening_bit_exact(oracle_mod):
    """Mixed linear hardening (J2_xi = 0.5) over three quarters of a load
    cycle of SC 6^3 with reverse yielding: per-step Newton iterations,
    residuals and top displacement, and the final positions, plastic strain,
    back stress and bond forces equal the reference's
    (tests/golden/sc6_kinematic.npz)."""
    case = cases.SCCase(n=6, sigmay=150.0, xi=0.5, steps_per_quarter=8, cycles=1)
    g = golden("sc6_kinematic.npz")
    o, types = sc_oracle(oracle_mod, case, threads=1)
    n, nn = o.n, o.nn
    assert np.array_equal(types, g["types"])
    x0 = o.d("xyz_initial", (n, 3))
    top = types == cases.T_TOP
    assert len(g["iters"]) == 24
    for k, stp in enumerate(case.schedule[:24]):
        st = o.load_step(cases.sc_bcs(stp), [], case.newton_tol, 100, 1e-20, 0.0)
        assert st[0] == g["iters"][k] and st[3] == g["nres"][k], k
        xyz = o.d("xyz", (n, 3))
        assert (xyz[top, 2].sum() - x0[top, 2].sum()) / top.sum() == g["disp_top"][k], k
    assert np.array_equal(o.d("xyz", (n, 3)), g["s_xyz"])
    assert np.array_equal(o.d("alpha1", (n,)), g["s_alpha"])
    assert np.array_equal(o.d("beta1", (n, 6)), g["s_beta"])
    assert np.array_equal(o.d("F", (n, nn)), g["s_F"])
    assert np.abs(g["s_beta"]).max() > 0.0


def test_per_particle_yield_stress_bit_exact(oracle_mod):
    """Per-particle yield stress (sigmay[i], src/constitutive.c:591; U[200,
    400] MPa as the batch workload draws it), 20 cyclic steps of SC 8^3 with
    progressive yielding: the oracle equals the reference
    (tests/golden/sc8_sigmay.npz)."""
    case = cases.SCCase(n=8)
    g = golden("sc8_sigmay.npz")
    oracle_mod.set_threads(1)
    o = oracle_mod.Oracle()
    n = o.setup_lattice(case.lattice, case.radius, case.box)
    nn = o.nn
    types = cases.sc_types(o.d("xyz", (n, 3)), o.i("nb", (n,)), case.radius)
    assert np.array_equal(types, g["types"])
    o.set_types(types)
    sy = cases.sigmay_field(n)
    assert np.array_equal(sy, g["sigmay"])
    c11, c12, c44 = cases.iso_cubic(case.E, case.nu)
    o.set_material(np.full(n, c11), np.full(n, c12), np.full(n, c44), sy, case.H, 0.0, 0)
    o.init_state()
    x0 = o.d("xyz_initial", (n, 3))
    top = types == cases.T_TOP
    for k, stp in enumerate(case.schedule[:20]):
        st = o.load_step(cases.sc_bcs(stp), [], case.newton_tol, 100, 1e-20, 0.0)
        assert st[0] == g["iters"][k] and st[3] == g["nres"][k], k
        xyz = o.d("xyz", (n, 3))
        assert (xyz[top, 2].sum() - x0[top, 2].sum()) / top.sum() == g["disp_top"][k], k
    assert np.array_equal(o.d("xyz", (n, 3)), g["s_xyz"])
    assert np.array_equal(o.d("alpha1", (n,)), g["s_alpha"])
    assert np.array_equal(o.d("F", (n, nn)), g["s_F"])


def test_fcc_j2_bit_exact(oracle_mod):
    """J2 plasticity on the FCC lattice (plmode 0 on lattice 3), 4^3 cells,
    [001] tension, 12 steps with yield from step 8: the oracle equals the
    reference (tests/golden/fcc4_j2.npz)."""
    case = cases.FCCCase(ncell=4)
    g = golden("fcc4_j2.npz")
    oracle_mod.set_threads(1)
    o = oracle_mod.Oracle()
    n = o.setup_lattice(case.lattice, case.radius, case.box)
    nn = o.nn
    types = cases.sc_types(o.d("xyz", (n, 3)), o.i("nb", (n,)), case.radius)
    assert np.array_equal(types, g["types"])
    o.set_types(types)
    o.set_material(case.C11, case.C12, case.C44, cases.FCC_J2["sigmay"], cases.FCC_J2["H"], 0.0, 0)
    o.init_state()
    x0 = o.d("xyz_initial", (n, 3))
    top = types == cases.T_TOP
    for k, stp in enumerate(case.schedule[:12]):
        st = o.load_step(cases.sc_bcs(stp), [], case.newton_tol, 100, 1e-20, 0.0)
        assert st[0] == g["iters"][k] and st[3] == g["nres"][k], k
        xyz = o.d("xyz", (n, 3))
        assert (xyz[top, 2].sum() - x0[top, 2].sum()) / top.sum() == g["disp_top"][k], k
    assert np.array_equal(o.d("xyz", (n, 3)), g["s_xyz"])
    assert np.array_equal(o.d("alpha1", (n,)), g["s_alpha"])
    assert np.array_equal(o.d("dLp1", (n, nn)), g["s_dLp"])
    assert np.array_equal(o.d("F", (n, nn)), g["s_F"])
    assert g["s_alpha"].max() > 0.0


def _cyclic_segment(first):
    """Steps first+1 .. first+20 of the C1 cyclic case in the oracle, started
    from the reference's converged state after step `first` (fresh for 0);
    returns the mismatches against the reference's fixture."""
    import oracle as O
    case = cases.SCCase(n=10)
    o, types = sc_oracle(O, case, threads=1)
    g = golden("sc10_cyclic.npz")
    if first:
        restore(o, g, first)
    n = o.n
    x0 = o.d("xyz_initial", (n, 3))
    top = types == cases.T_TOP
    bad = []
    for k in range(first, first + 20):
        st = o.load_step(cases.sc_bcs(case.schedule[k]), [], case.newton_tol, 100, 1e-20, 0.0)
        xyz = o.d("xyz", (n, 3))
        F, csz = o.d("F", (n, 18)), o.d("csz", (n, 18))
        if not (st[0] == g["iters"][k] and st[3] == g["nres"][k] and
                (xyz[top, 2].sum() - x0[top, 2].sum()) / top.sum() == g["disp_top"][k] and
                np.sum(-csz[top] * F[top]) == g["react_top"][k]):
            bad.append(("step", k + 1))
    last = first + 20
    for key in ("xyz", "alpha", "dLp", "stress"):
        name = {"alpha": "alpha1", "dLp": "dLp1", "stress": "stress_tensor"}.get(key, key)
        shape = g[f"s{last}_{key}"].shape
        if not np.array_equal(g[f"s{last}_{key}"], o.d(name, shape)):
            bad.append((key, last))
    return bad


def test_full_cyclic_run_bit_exact(oracle_mod):
    """All 160 load steps of the C1 case (two cycles, eight plastic stretches
    that stop at the reference's MAXITER) against the reference's own run:
    per-step Newton iterations, final residual, top displacement and reaction,
    and the converged state every 20 steps, bit for bit.  The run is replayed
    as eight segments of 20 steps, each started from the reference's state at
    its first step (the resume itself is pinned above), in parallel."""
    import multiprocessing as mp
    g = golden("sc10_cyclic.npz")
    starts = list(range(0, 160, 20))
    assert all(s + 20 in set(int(k) for k in g["snap_steps"]) for s in starts)
    with mp.get_context("spawn").Pool(min(len(starts), max(1, os.cpu_count() or 1))) as pool:
        results = pool.map(_cyclic_segment, starts)
    assert all(not r for r in results), results
