"""A context set up a second time (another specimen size) gives the same
results as a fresh context: nothing captured or sized for the first specimen
(PCG graphs, Anderson history, adjoint state) survives the new setup."""
import numpy as np
import pytest

import cases
from setup_helpers import material_arrays

pytestmark = pytest.mark.gpu


def prepare(s, G, case):
    n = s.setup_lattice(case.lattice, case.radius, case.box)
    s.set_types(cases.sc_types(s.get("xyz"), s.get("nb"), case.radius))
    c11, c12, c44 = material_arrays(case, n)
    s.set_material(c11, c12, c44, case.sigmay, case.H, 0.0, G.PL_J2)
    s.init_state()
    s.set_solver(precision=1, newton_tol=case.newton_tol, newton_accel=4)


def test_resetup_matches_fresh_context(gpu_lib):
    G = gpu_lib
    small, big = cases.SCCase(n=6), cases.SCCase(n=8, e_noise=0.05)
    reused = G.Specimen(0)
    prepare(reused, G, small)
    for stp in small.schedule[:2]:
        reused.load_step(cases.sc_bcs(stp))
    prepare(reused, G, big)
    fresh = G.Specimen(0)
    prepare(fresh, G, big)
    for stp in big.schedule[:3]:
        a = reused.load_step(cases.sc_bcs(stp))
        b = fresh.load_step(cases.sc_bcs(stp))
        assert a["status"] == 0 and b["status"] == 0
        assert np.array_equal(reused.get("xyz"), fresh.get("xyz"))
    reused.close()
    fresh.close()
