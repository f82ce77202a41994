"""The reference main's damage stage on the GPU (lpm_set_damage) against the
oracle, whose damage stage reproduces the reference bit for bit
(tests/test_oracle_damage.py).

Per load step: the number of Newton passes (1 + re-solves after breaking), the
sum of updateDamageGeneral's return values, the set of bonds broken in the
step, intact-bond counts and damage_broken exactly; displacements within 1e-8
and the nonlocal damage and bond weights within 1e-6 relative (the nonlocal
sum runs in a different order and with CUDA's exp).  The order of bonds
within one brittle pass is not compared: equal-strain bonds swap places there
under round-off-level differences of the solution, in the reference too.
"""
import numpy as np
import pytest

import cases
from test_oracle_damage import _brittle, _ductile

pytestmark = [pytest.mark.gpu, pytest.mark.gpu_last]

# Both sides converge to 1e-9: the converged displacements are then within
# 2e-9 of the 1e-10 solution (measured on the oracle), while 1e-10 sits at the
# force residual's round-off floor in these damaged specimens (the brittle one
# reaches it at step 9, where the reference's CG then divides 0 by 0).
TOL = 1e-9


def _gpu(G, which, precision):
    s = G.Specimen(0)
    if which == "ductile":
        case = cases.DuctileDamageCase()
        n = s.setup_lattice(case.lattice, case.radius, case.box)
        xyz0 = s.get("xyz")
        s.set_types(cases.sc_types(xyz0, s.get("nb"), case.radius))
        c11, c12, c44 = cases.iso_cubic(case.E, case.nu)
        s.set_material(np.full(n, c11), np.full(n, c12), np.full(n, c44), case.sigmay(xyz0), np.full(n, case.H),
                       0.0, G.PL_J2)
        s.init_state()
        s.set_damage(length=case.L, threshold=case.threshold, triax_coeff=0.0)
        step_bcs = [cases.sc_bcs(v) for v in case.schedule]
    else:
        case = cases.BrittleCase()
        n = s.setup_lattice(case.lattice, case.radius, case.box)
        xyz0 = s.get("xyz")
        s.set_types(case.types(xyz0, s.get("nb")))
        c11, c12, c44 = cases.iso_cubic(case.E, case.nu)
        s.set_material(np.full(n, c11), np.full(n, c12), np.full(n, c44), np.full(n, 1e30), np.zeros(n), 0.0,
                       G.PL_ELASTIC)
        s.init_state()
        s.set_damage(critical_bstrain=case.crit, nbreak=case.nbreak)
        step_bcs = [case.bcs(v) for v in case.schedule[:8]]
    s.set_solver(precision=precision, newton_tol=TOL, newton_maxiter=400, cg_rtol=1e-11)
    return s, step_bcs


@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("which", ["ductile", "brittle"])
def test_damage_stage_matches_oracle(oracle_mod, gpu_lib, which, precision):
    s, step_bcs = _gpu(gpu_lib, which, precision)
    o, _, _, _ = (_ductile if which == "ductile" else _brittle)(oracle_mod)
    o.L.lo_set_threads(4)
    n, nn = o.n, o.nn
    assert s.n == n
    x0 = o.d("xyz_initial", (n, 3))
    done_g = done_o = 0
    for k, bcs in enumerate(step_bcs, start=1):
        st = s.load_step(bcs)
        so = o.load_step_damage(bcs, [], TOL, 400, 1e-22, 0.0, 50)
        assert st["status"] == 0, (k, st)
        assert st["damage_passes"] == int(so[5]) and st["bonds_broken"] == int(so[6]), (k, st, so)
        lg, lo = s.damage_log(), o.broken_log()
        assert set(map(tuple, lg[done_g:].tolist())) == set(map(tuple, lo[done_o:].tolist())), k
        done_g, done_o = lg.shape[0], lo.shape[0]
        assert np.array_equal(s.get("damage_broken"), o.d("damage_broken", (n, nn))), k
        assert np.array_equal(s.get("nb_current"), o.i("nb_current", (n,))), k
        du_g = s.get("xyz") - x0
        du_o = o.d("xyz", (n, 3)) - x0
        err = np.abs(du_g - du_o).max() / np.abs(du_o).max()
        assert err < 1e-8, (k, err)
        dn_o = o.d("damage_nonlocal1", (n,))
        assert np.abs(s.get("damage_nonlocal") - dn_o).max() <= 1e-6 * max(dn_o.max(), 1e-300), k
        assert np.abs(s.get("damage_w") - o.d("damage_w", (n, nn))).max() <= 1e-6, k
    assert done_o > 0  # the case broke bonds
    if which == "ductile":
        assert np.array_equal(s.damage_log(), o.broken_log())  # no ties in the ductile breaking order


def test_damage_stage_is_inert_for_crystal_plasticity(gpu_lib):
    """updateDamageGeneral does nothing for crystal plasticity and updateCrack
    then multiplies by w = 1: switching the stage on changes no bit."""
    case = cases.FCCCase(ncell=4)
    out = []
    for on in (False, True):
        s = gpu_lib.Specimen(0)
        n = s.setup_lattice(case.lattice, case.radius, case.box)
        s.set_types(cases.sc_types(s.get("xyz"), s.get("nb"), case.radius))
        s.set_cp(*case.cp)
        s.set_material(case.C11, case.C12, case.C44, 0.0, 0.0, 0.0, gpu_lib.PL_CP)
        s.init_state()
        s.set_solver(precision=0, newton_tol=1e-8, newton_maxiter=300)
        if on:
            s.set_damage()
        for stp in case.schedule[:4]:
            st = s.load_step(cases.sc_bcs(stp))
            assert st["status"] == 0
            assert st["damage_passes"] == (1 if on else 0) and st["bonds_broken"] == 0
        out.append((s.get("xyz"), s.get("F"), s.get("stress_tensor")))
    for a, b in zip(*out):
        assert np.array_equal(a, b)


def test_damage_off_restores_the_undamaged_path(gpu_lib):
    """Switching the stage on and off again, or re-initialising the state,
    leaves the solve path bit-identical to a specimen that never had it."""
    case = cases.SCCase(n=6, sigmay=150.0)
    runs = []
    for mode in ("never", "on_off", "on_reinit"):
        s = gpu_lib.Specimen(0)
        n = s.setup_lattice(case.lattice, case.radius, case.box)
        s.set_types(cases.sc_types(s.get("xyz"), s.get("nb"), case.radius))
        c11, c12, c44 = cases.iso_cubic(case.E, case.nu)
        s.set_material(np.full(n, c11), np.full(n, c12), np.full(n, c44), case.sigmay, case.H, 0.0, gpu_lib.PL_J2)
        s.init_state()
        s.set_solver(precision=0, newton_tol=1e-8, newton_maxiter=300)
        if mode != "never":
            s.set_damage(length=0.15, threshold=1e-4)
            for stp in case.schedule[:10]:  # break bonds and change the stress weights
                s.load_step(cases.sc_bcs(stp))
            if mode == "on_off":
                s.set_damage(enabled=False)
            s.init_state()
        for stp in case.schedule[:12]:
            assert s.load_step(cases.sc_bcs(stp))["status"] == 0
        runs.append(s.get("xyz"))
    assert np.array_equal(runs[0], runs[1]) and np.array_equal(runs[0], runs[2])
