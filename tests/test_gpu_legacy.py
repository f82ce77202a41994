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
