"""Mixed linear hardening (J2_xi = 0.5) on the GPU against the oracle, which
matches the reference bit for bit on the same case
(tests/test_oracle_golden.py::test_kinematic_hardening_bit_exact): 24 steps
of SC 6^3 with reverse yielding, FP64 and mixed precision, both sides
converged to 1e-10."""
import numpy as np
import pytest

import cases
from setup_helpers import sc_gpu, sc_oracle

pytestmark = [pytest.mark.gpu, pytest.mark.gpu_last]


@pytest.mark.parametrize("precision", [0, 1])
def test_kinematic_hardening_matches_oracle(oracle_mod, gpu_lib, precision):
    case = cases.SCCase(n=6, sigmay=150.0, xi=0.5, steps_per_quarter=8, cycles=1, newton_tol=1e-10)
    o, _ = sc_oracle(oracle_mod, case, threads=4)
    s, _ = sc_gpu(gpu_lib, case, precision=precision, newton_maxiter=300, cg_rtol=1e-10)
    n = o.n
    x0 = o.d("xyz_initial", (n, 3))
    for k, stp in enumerate(case.schedule[:24]):
        st = s.load_step(cases.sc_bcs(stp))
        o.load_step(cases.sc_bcs(stp), [], 1e-10, 300, 1e-20, 0.0)
        assert st["status"] == 0, (k + 1, st)
        du_g = s.get("xyz") - x0
        du_o = o.d("xyz", (n, 3)) - x0
        err = np.abs(du_g - du_o).max() / np.abs(du_o).max()
        assert err < 1e-8, (k + 1, err)
    a_o, b_o = o.d("alpha1", (n,)), o.d("beta1", (n, 6))
    assert a_o.max() > 0.0 and np.abs(b_o).max() > 0.0
    assert np.abs(s.get("J2_alpha") - a_o).max() <= 1e-8 * a_o.max()
    assert np.abs(s.get("J2_beta") - b_o).max() <= 1e-7 * np.abs(b_o).max()
