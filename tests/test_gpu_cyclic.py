"""The whole C1 case on the GPU against the reference's own run.

SC 10^3, two load cycles of +-0.2 % strain in 160 steps, Newton tolerance
1e-8 with the reference's MAXITER of 100 (include/lpm.h:39; the plastic steps
of this case stop there), linear solves to 1e-10 relative.  The fixture
tests/golden/sc10_cyclic.npz was written by the reference itself
(tests/golden/make_golden.py) with the same settings; the oracle reproduces it
bit for bit (tests/test_oracle_golden.py).  Compared, and printed for each
observable:
- the reaction of the top face at every step (writeReaction's sum of
  -cs_z F over the particles of the type, src/data_handler.c:309-335);
- the displacements of every particle at the converged end of steps 20, 40,
  ..., 160 (every quarter cycle), against the largest displacement of the
  run;
- the plastic strain J2_alpha and the plastic bond stretches dLp at the end.
Bars: 1e-8 relative to the largest magnitude of each observable."""
import numpy as np
import pytest

import cases
from conftest import golden
from setup_helpers import sc_gpu

pytestmark = [pytest.mark.gpu, pytest.mark.gpu_last]

TOL = 1e-8


@pytest.mark.parametrize("precision", [0, 1])
def test_full_cyclic_run_matches_reference(gpu_lib, precision):
    g = golden("sc10_cyclic.npz")
    case = cases.SCCase(n=10)
    s, types = sc_gpu(gpu_lib, case, precision=precision, newton_maxiter=100, cg_rtol=1e-10)
    n = s.n
    x0 = s.get("xyz_initial")
    top = types == cases.T_TOP
    snaps = set(int(k) for k in g["snap_steps"])
    # the largest displacement of the run (at the load peaks): the scale of the
    # displacement errors (at the zero crossings only the small residual
    # plastic deformation remains)
    du_scale = max(float(np.abs(g[f"s{k}_xyz"] - x0).max()) for k in snaps)
    react = np.zeros(len(case.schedule))
    du_err = {}
    iters = []
    for k, stp in enumerate(case.schedule):
        st = s.load_step(cases.sc_bcs(stp))
        assert st["status"] & ~gpu_lib.STATUS_NEWTON_MAXIT == 0, (k + 1, st)
        iters.append(st["newton_iters"])
        F, csz = s.get("F"), s.get("csz")
        react[k] = np.sum(-csz[top] * F[top])
        if (k + 1) in snaps and (k + 1) >= 20:
            du = s.get("xyz") - x0
            ref = g[f"s{k + 1}_xyz"] - x0
            du_err[k + 1] = float(np.abs(du - ref).max()) / du_scale
    r_err = np.abs(react - g["react_top"]) / np.abs(g["react_top"]).max()
    last = len(case.schedule)
    a, a_ref = s.get("J2_alpha"), g[f"s{last}_alpha"]
    dlp, dlp_ref = s.get("dLp"), g[f"s{last}_dLp"]
    a_err = float(np.abs(a - a_ref).max() / np.abs(a_ref).max())
    dlp_err = float(np.abs(dlp - dlp_ref).max() / np.abs(dlp_ref).max())
    it_diff = int(np.abs(np.array(iters) - g["iters"].astype(int)).max())
    print(f"\nC1 full run, precision {precision}: reaction max rel err {r_err.max():.3e} (step "
          f"{int(r_err.argmax()) + 1}); displacement rel err by step {du_err}; J2_alpha {a_err:.3e}; "
          f"dLp {dlp_err:.3e}; Newton iterations differ by at most {it_diff}")
    assert a_ref.max() > 0.0
    assert r_err.max() < TOL, r_err.max()
    assert max(du_err.values()) < TOL, du_err
    assert a_err < TOL and dlp_err < TOL, (a_err, dlp_err)
    s.close()
