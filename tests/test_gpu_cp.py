"""Crystal plasticity (computeBondForceCPMiehe, plmode 1) on the GPU against the
oracle (which matches the reference bit for bit, tests/test_oracle_golden.py)."""
import numpy as np
import pytest

import cases

pytestmark = pytest.mark.gpu


def fcc_gpu(G, case, precision=0, **solver):
    s = G.Specimen(0)
    n = s.setup_lattice(case.lattice, case.radius, case.box)
    types = cases.sc_types(s.get("xyz"), s.get("nb"), case.radius)
    s.set_types(types)
    s.set_cp(*case.cp)
    s.set_material(case.C11, case.C12, case.C44, 0.0, 0.0, 0.0, G.PL_CP)
    s.init_state()
    s.set_solver(precision=precision, newton_tol=case.newton_tol, **solver)
    return s, types


def fcc_oracle(O, case, threads=4):
    O.set_threads(threads)
    o = O.Oracle()
    n = o.setup_lattice(case.lattice, case.radius, case.box)
    types = cases.sc_types(o.d("xyz", (n, 3)), o.i("nb", (n,)), case.radius)
    o.set_types(types)
    o.set_cp(*case.cp)
    o.set_material(case.C11, case.C12, case.C44, 0.0, 0.0, 0.0, 1)
    o.init_state()
    return o, types


def test_fcc_setup_and_cab(oracle_mod, gpu_lib):
    case = cases.FCCCase(ncell=4)
    s, types = fcc_gpu(gpu_lib, case)
    o, types_o = fcc_oracle(oracle_mod, case)
    n, nn = o.n, o.nn
    assert np.array_equal(types, types_o)
    assert np.array_equal(s.get("neighbors"), o.i("neighbors", (n, nn)))
    assert np.array_equal(s.get("Kn"), o.d("Kn", (n, nn)))
    cab_g = s.get("cp_Cab")
    cab_o = o.d("cp_Cab", (n, 24 * 24))
    assert np.allclose(cab_g, cab_o, rtol=1e-12, atol=1e-9 * np.abs(cab_o).max())


@pytest.mark.parametrize("precision", [0, 1])
def test_fcc_cp_steps_match_oracle(oracle_mod, gpu_lib, precision):
    """[001] tension of a 4^3-cell FCC crystal into the plastic range (steps 1-11):
    displacements, slip resistances and accumulated slip agree with the oracle."""
    case = cases.FCCCase(ncell=4, newton_tol=1e-10)
    s, types = fcc_gpu(gpu_lib, case, precision=precision, newton_maxiter=300, cg_rtol=1e-11)
    o, _ = fcc_oracle(oracle_mod, case)
    n = o.n
    x0 = o.d("xyz_initial", (n, 3))
    for k, stp in enumerate(case.schedule[:11]):
        st = s.load_step(cases.sc_bcs(stp))
        o.load_step(cases.sc_bcs(stp), [], 1e-10, 300, 1e-22, 0.0)
        assert st["status"] == 0, (k + 1, st)
        du_g = s.get("xyz") - x0
        du_o = o.d("xyz", (n, 3)) - x0
        err = np.abs(du_g - du_o).max() / np.abs(du_o).max()
        assert err < 1e-8, (k + 1, err, st)
    A_o = o.d("cp_A1", (n,))
    assert A_o.max() > 0.0
    assert np.abs(s.get("cp_A") - A_o).max() <= 1e-8 * A_o.max()
    gy_o = o.d("cp_gy1", (n, 24))
    assert np.abs(s.get("cp_gy") - gy_o).max() <= 1e-8 * np.abs(gy_o).max()


@pytest.mark.gpu_last
def test_fcc_cp_latent_saturating_match_oracle(oracle_mod, gpu_lib):
    """Latent hardening (q = 1.2) and a finite saturation stress, steps 1-9
    (the case the oracle matches bit for bit against the reference,
    tests/golden/fcc4_sat_cp.npz): displacements and slip state agree with the
    oracle."""
    case = cases.FCCCase(ncell=4, newton_tol=1e-10, **cases.FCC_SAT)
    s, _ = fcc_gpu(gpu_lib, case, precision=0, newton_maxiter=300, cg_rtol=1e-11)
    o, _ = fcc_oracle(oracle_mod, case)
    n = o.n
    x0 = o.d("xyz_initial", (n, 3))
    for k, stp in enumerate(case.schedule[:9]):
        st = s.load_step(cases.sc_bcs(stp))
        o.load_step(cases.sc_bcs(stp), [], 1e-10, 300, 1e-22, 0.0)
        assert st["status"] == 0, (k + 1, st)
        du_g = s.get("xyz") - x0
        du_o = o.d("xyz", (n, 3)) - x0
        assert np.abs(du_g - du_o).max() < 1e-8 * np.abs(du_o).max(), k + 1
    A_o = o.d("cp_A1", (n,))
    assert A_o.max() > 0.0
    assert np.abs(s.get("cp_A") - A_o).max() <= 1e-8 * A_o.max()
    gy_o = o.d("cp_gy1", (n, 24))
    assert np.abs(s.get("cp_gy") - gy_o).max() <= 1e-8 * np.abs(gy_o).max()


@pytest.mark.gpu_last
@pytest.mark.parametrize("steps", [0, 3])
def test_fcc_stiffness_vs_fd(oracle_mod, gpu_lib, steps):
    """Analytic tangent vs the reference's forward-difference K on the FCC
    lattice (calcStiffness3DFiniteDifference differentiates the elastic bond
    force for every material model), at rest and after three [001] tension
    steps, where the force-dependent (geometric) terms are non-zero."""
    case = cases.FCCCase(ncell=4, newton_tol=1e-10)
    s, _ = fcc_gpu(gpu_lib, case, newton_maxiter=300, cg_rtol=1e-11)
    o, _ = fcc_oracle(oracle_mod, case)
    for stp in case.schedule[:steps]:
        assert s.load_step(cases.sc_bcs(stp))["status"] == 0
        o.load_step(cases.sc_bcs(stp), [], 1e-10, 300, 1e-22, 0.0)
    o.fd_stiffness()
    s.assemble_stiffness()
    K, IK, JK = s.export_upper_csr()
    nnz = o.nnz
    assert np.array_equal(IK, o.i("IK", (3 * o.n + 1,)))
    assert np.array_equal(JK, o.i("JK", (nnz,)))
    Kf = o.d("K_global", (nnz,))
    rel = np.linalg.norm(K - Kf) / np.linalg.norm(Kf)
    # forward differences with h = 1e-6 r: truncation ~1e-6 relative
    assert rel < 1e-5, rel


@pytest.mark.gpu_last
@pytest.mark.parametrize("precision", [0, 1])
def test_fcc_j2_match_oracle(oracle_mod, gpu_lib, precision):
    """J2 plasticity on the FCC lattice (the case the oracle matches bit for
    bit against the reference, tests/golden/fcc4_j2.npz): 12 steps of [001]
    tension, displacements and plastic strain against the oracle."""
    G = gpu_lib
    case = cases.FCCCase(ncell=4, newton_tol=1e-10)
    sy, H = cases.FCC_J2["sigmay"], cases.FCC_J2["H"]
    oracle_mod.set_threads(4)
    o = oracle_mod.Oracle()
    n = o.setup_lattice(case.lattice, case.radius, case.box)
    types = cases.sc_types(o.d("xyz", (n, 3)), o.i("nb", (n,)), case.radius)
    o.set_types(types)
    o.set_material(case.C11, case.C12, case.C44, sy, H, 0.0, 0)
    o.init_state()
    s = G.Specimen(0)
    assert s.setup_lattice(case.lattice, case.radius, case.box) == n
    s.set_types(types)
    s.set_material(case.C11, case.C12, case.C44, sy, H, 0.0, G.PL_J2)
    s.init_state()
    s.set_solver(precision=precision, newton_tol=1e-10, newton_maxiter=300, cg_rtol=1e-11)
    x0 = o.d("xyz_initial", (n, 3))
    for k, stp in enumerate(case.schedule[:12]):
        st = s.load_step(cases.sc_bcs(stp))
        o.load_step(cases.sc_bcs(stp), [], 1e-10, 300, 1e-22, 0.0)
        assert st["status"] == 0, (k + 1, st)
        du_g = s.get("xyz") - x0
        du_o = o.d("xyz", (n, 3)) - x0
        assert np.abs(du_g - du_o).max() < 1e-8 * np.abs(du_o).max(), k + 1
    a_o = o.d("alpha1", (n,))
    assert a_o.max() > 0.0
    assert np.abs(s.get("J2_alpha") - a_o).max() <= 1e-8 * a_o.max()
