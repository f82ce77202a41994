"""The reference-named drop-in (liblpmgpu_legacy.so) driven by the C host loop
(liblpmhost.so, the src/lpmc_project.c:382-471 sequence over include/lpm.h
globals) reproduces the oracle's load steps."""
import numpy as np
import pytest

import cases
from setup_helpers import material_arrays, sc_oracle

pytestmark = pytest.mark.gpu


def test_legacy_host_loop_matches_oracle(oracle_mod, gpu_lib):
    import lpm_host
    case = cases.SCCase(n=8, newton_tol=1e-10)
    h = lpm_host.HostDriver()
    n = h.setup(case.lattice, case.radius, case.box)
    s = gpu_lib.Specimen(0)
    s.setup_lattice(case.lattice, case.radius, case.box)
    types = cases.sc_types(h.get("xyz"), s.get("nb"), case.radius)
    s.close()
    h.set_types(types, cases.NTYPE)
    h.set_material(case.ce_per_type(), 0, case.sigmay, 0.0, case.H)
    h.set_solver(precision=gpu_lib.PREC_FP64, cg_rtol=1e-10)
    h.init()
    o, types_o = sc_oracle(oracle_mod, case, threads=2)
    assert np.array_equal(types, types_o)
    x0 = o.d("xyz_initial", (n, 3))
    assert np.array_equal(h.get("xyz_initial"), x0)
    for k, stp in enumerate(case.schedule[:14]):
        st = h.load_step(cases.sc_bcs(stp), newton_tol=1e-10, maxiter=300)
        o.load_step(cases.sc_bcs(stp), [], 1e-10, 300, 1e-20, 0.0)
        du_h = h.get("xyz") - x0
        du_o = o.d("xyz", (n, 3)) - x0
        err = np.abs(du_h - du_o).max() / np.abs(du_o).max()
        assert err < 1e-8, (k + 1, err, st)
    assert np.abs(h.get("J2_alpha") - o.d("alpha1", (n,))).max() < 1e-10
    h2d, d2h = h.traffic()
    assert h2d > 0 and d2h > 0
    # computeStrain through the drop-in equals the context entry point on the same bond stretches
    e_host = h.compute_strain()
    s = gpu_lib.Specimen(0)
    s.setup_lattice(case.lattice, case.radius, case.box)
    s.set_types(types)
    c11, c12, c44 = cases.iso_cubic(case.E, case.nu)
    s.set_material(np.full(n, c11), np.full(n, c12), np.full(n, c44), case.sigmay, case.H, 0.0, gpu_lib.PL_J2)
    s.init_state()
    s.set("dL", h.get("dL"))
    assert np.array_equal(e_host, s.compute_strain())
    assert np.abs(e_host).max() > 0.0
    s.close()


@pytest.mark.gpu_last
def test_legacy_per_particle_moduli_match_oracle(oracle_mod, gpu_lib):
    """The C2 material model (E +-5 % per particle) through the drop-in as the
    reference expresses it: one type per particle with its own Ce row
    (src/stiffness.c:186-200), the boundary conditions given as BC groups.
    Bond Kn/Tv in the host globals are bit-exact with the reference's
    (tests/golden/sc8_enoise.npz); the 9 cyclic steps on which the
    reference's modified Newton converges (two of them plastic) match the
    oracle within 1e-8."""
    import lpm_host
    from conftest import golden
    case = cases.SCCase(n=8, sigmay=150.0, e_noise=0.05, seed=1, newton_tol=1e-10)
    g = golden("sc8_enoise.npz")
    h = lpm_host.HostDriver()
    n = h.setup(case.lattice, case.radius, case.box)
    o, types = sc_oracle(oracle_mod, case, threads=4)
    h.set_types(np.arange(n, dtype=np.int32), n)
    h.set_bc_groups(types, cases.NTYPE)
    c11, c12, c44 = material_arrays(case, n)
    h.set_material(np.stack([c11, c12, c44], axis=1), 0, case.sigmay, 0.0, case.H)
    h.set_solver(precision=gpu_lib.PREC_MIXED, cg_rtol=1e-10)
    h.init()
    assert np.array_equal(h.get("Kn"), g["Kn"]) and np.array_equal(h.get("Tv"), g["Tv"])
    x0 = o.d("xyz_initial", (n, 3))
    for k, stp in enumerate(case.schedule[:9]):
        h.load_step(cases.sc_bcs(stp), newton_tol=1e-10, maxiter=300)
        o.load_step(cases.sc_bcs(stp), [], 1e-10, 300, 1e-20, 0.0)
        du_h = h.get("xyz") - x0
        du_o = o.d("xyz", (n, 3)) - x0
        err = np.abs(du_h - du_o).max() / np.abs(du_o).max()
        assert err < 1e-8, (k + 1, err)
    a_o = o.d("alpha1", (n,))
    assert a_o.max() > 0.0
    assert np.abs(h.get("J2_alpha") - a_o).max() <= 1e-8 * a_o.max()


def _bond_file(path):
    """The reference's bond file: per TIMESTEP, its broken (i, j) pairs."""
    steps = {}
    cur = None
    with open(path) as f:
        for line in f:
            p = line.split()
            if not p:
                continue
            if p[0] == "TIMESTEP":
                cur = int(p[1])
                steps.setdefault(cur, [])
            else:
                steps[cur].append((int(p[0]), int(p[1])))
    return steps


@pytest.mark.gpu_last
@pytest.mark.parametrize("which", ["ductile", "brittle"])
def test_legacy_damage_stage_matches_oracle(oracle_mod, gpu_lib, tmp_path, which):
    """main's damage stage through the drop-in: the C host loop calls
    updateDamageGeneral and updateCrack of liblpmgpu_legacy.so after each
    converged pass and re-enters the Newton loop after broken bonds
    (src/lpmc_project.c:466-470, :528-546).  Against the oracle's damage stage
    per load step: Newton passes and the sum of updateDamageGeneral's return
    values, the bonds the step wrote to the bond file (as a set: equal-strain
    bonds of a brittle pass swap places under round-off), damage_broken and
    the intact-bond counts nb exactly, displacements within 1e-8."""
    import lpm_host
    from test_oracle_damage import _brittle, _ductile
    tol = 1e-9  # as tests/test_gpu_damage.py: above the round-off floor of the damaged specimens
    o, types, step_bcs, _ = (_ductile if which == "ductile" else _brittle)(oracle_mod)
    o.L.lo_set_threads(4)
    n, nn = o.n, o.nn
    case = cases.DuctileDamageCase() if which == "ductile" else cases.BrittleCase()
    h = lpm_host.HostDriver()
    assert h.setup(case.lattice, case.radius, case.box) == n
    xyz0 = h.get("xyz_initial")
    assert np.array_equal(xyz0, o.d("xyz_initial", (n, 3)))
    ntype = int(types.max()) + 1
    h.set_types(types, ntype)
    ce = np.tile(cases.iso_cubic(case.E, case.nu), (ntype, 1))
    bond_file = str(tmp_path / "result_brokenbonds.txt")
    if which == "ductile":
        h.set_material(ce, 0, case.sigmay(xyz0), 0.0, case.H)
        h.set_damage(bond_file, length=case.L, threshold=case.threshold, triax_coeff=0.0, max_passes=50)
    else:
        h.set_material(ce, 6, 1e30, 0.0, 0.0)
        h.set_damage(bond_file, critical_bstrain=case.crit, nbreak=case.nbreak, max_passes=50)
        step_bcs = step_bcs[:8]
    h.set_solver(precision=gpu_lib.PREC_FP64, cg_rtol=1e-11)
    h.init()
    done_o = 0
    for k, bcs in enumerate(step_bcs, start=1):
        st = h.load_step(bcs, newton_tol=tol, maxiter=400)
        so = o.load_step_damage(bcs, [], tol, 400, 1e-22, 0.0, 50)
        assert int(st[5]) == int(so[5]) and int(st[6]) == int(so[6]), (k, st, so)
        lo = o.broken_log()
        logged = _bond_file(bond_file)
        assert set(logged.get(k, [])) == set(map(tuple, lo[done_o:].tolist())), k
        assert len(logged.get(k, [])) == lo.shape[0] - done_o, k
        done_o = lo.shape[0]
        assert np.array_equal(h.get("damage_broken"), o.d("damage_broken", (n, nn))), k
        assert np.array_equal(h.get("nb").astype(np.int32), o.i("nb_current", (n,))), k
        du_h = h.get("xyz") - xyz0
        du_o = o.d("xyz", (n, 3)) - xyz0
        err = np.abs(du_h - du_o).max() / np.abs(du_o).max()
        assert err < 1e-8, (k, err)
    assert done_o > 0  # the case broke bonds
    assert sorted(_bond_file(bond_file)) == list(range(1, len(step_bcs) + 1))  # a TIMESTEP line per step
