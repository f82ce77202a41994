"""The reference-named drop-in (liblpmgpu_legacy.so) driven by the C host loop
(liblpmhost.so, the src/lpmc_project.c:382-471 sequence over include/lpm.h
globals) reproduces the oracle's load steps."""
import numpy as np
import pytest

import cases
from setup_helpers import sc_oracle

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
