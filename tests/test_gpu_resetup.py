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


def test_overfull_neighbourhood_is_an_error(gpu_lib):
    """A particle with more bonds than the 18 slots fails the setup with
    LPM_ERR_ARG naming it (the reference writes past its row then), instead of
    silently dropping bonds; the context stays usable."""
    G = gpu_lib
    case = cases.SCCase(n=5)
    s = G.Specimen(0)
    n = s.setup_lattice(case.lattice, case.radius, case.box)
    xyz = s.get("xyz")
    # a particle at the centre of an interior cell: within the first cut-off
    # of its 8 corners, which then hold 19 bonds
    lo = xyz.min(axis=0)
    centre = lo + 2.0 * case.radius * np.array([1.5, 1.5, 1.5])
    with pytest.raises(G.LPMError, match="more than 18 bonds"):
        s.setup_particles(case.lattice, case.radius, np.vstack([xyz, centre]))
    assert s.setup_particles(case.lattice, case.radius, xyz) == n
    s.close()
