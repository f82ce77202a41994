"""Mixed precision on an ill-conditioned specimen (six decades of stiffness
contrast between particles): the FP32-vector PCG may stagnate there and the
solve then continues with FP64 vectors; either way the step must converge to
the FP64 path's displacements."""
import numpy as np
import pytest

import cases

pytestmark = pytest.mark.gpu


def contrast_specimen(G, precision):
    case = cases.SCCase(n=10, sigmay=1e12, newton_tol=1e-10)
    s = G.Specimen(0)
    n = s.setup_lattice(case.lattice, case.radius, case.box)
    s.set_types(cases.sc_types(s.get("xyz"), s.get("nb"), case.radius))
    E = case.E * 10.0 ** (-6.0 * cases.splitmix64_uniform(5, n))
    c11, c12, c44 = cases.iso_cubic(E, case.nu)
    s.set_material(c11, c12, c44, case.sigmay, case.H, 0.0, G.PL_J2)
    s.init_state()
    s.set_solver(precision=precision, newton_tol=case.newton_tol, newton_maxiter=200, cg_rtol=1e-10,
                 cg_maxiter=50000)
    return s, case


def test_mixed_converges_on_high_contrast(gpu_lib):
    G = gpu_lib
    ref, case = contrast_specimen(G, 0)
    mix, _ = contrast_specimen(G, 1)
    x0 = ref.get("xyz_initial")
    for stp in case.schedule[:3]:
        a = ref.load_step(cases.sc_bcs(stp))
        b = mix.load_step(cases.sc_bcs(stp))
        assert a["status"] == 0 and b["status"] == 0, (a, b)
        da, db = ref.get("xyz") - x0, mix.get("xyz") - x0
        assert np.abs(da - db).max() <= 1e-8 * np.abs(da).max()
    ref.close()
    mix.close()
