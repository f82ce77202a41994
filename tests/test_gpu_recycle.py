"""Initial guesses from the load step's earlier Newton solutions
(opts.recycle): every linear solve still ends at its tolerance, so the load
steps reach the same displacements and plastic strain, with fewer PCG
iterations in the plastic range, where modified Newton contracts slowly and
successive right-hand sides lie close to the span of the earlier ones."""
import numpy as np
import pytest

import cases
from setup_helpers import sc_gpu

pytestmark = [pytest.mark.gpu, pytest.mark.gpu_option]


def _run(G, precision, recycle, precond):
    case = cases.SCCase(n=10)
    s, _ = sc_gpu(G, case, precision=precision, newton_maxiter=100, cg_rtol=1e-10, cg_maxiter=20000,
                  preconditioner=precond, recycle=recycle)
    x0 = s.get("xyz_initial")
    cg, newton, du = [], [], []
    for stp in case.schedule[:16]:
        st = s.load_step(cases.sc_bcs(stp))
        assert st["status"] & ~G.STATUS_NEWTON_MAXIT == 0, st
        cg.append(st["cg_iters"])
        newton.append(st["newton_iters"])
        du.append(s.get("xyz") - x0)
    alpha = s.get("J2_alpha")
    s.close()
    return np.array(cg), np.array(newton), du, alpha


@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("precond", [0, 1])
def test_recycled_guesses_same_steps_fewer_iterations(gpu_lib, precision, precond):
    G = gpu_lib
    cg0, nt0, du0, a0 = _run(G, precision, 0, precond)
    cg1, nt1, du1, a1 = _run(G, precision, 8, precond)
    # the same Newton iteration (a step whose residual ends next to the
    # tolerance may take one iteration more or less)
    assert np.abs(nt0 - nt1).max() <= 1, (nt0, nt1)
    scale = max(np.abs(d).max() for d in du0)
    err = max(np.abs(a - b).max() for a, b in zip(du0, du1)) / scale
    assert err < 1e-8, err
    assert np.abs(a1 - a0).max() <= 1e-8 * a0.max()
    plastic = nt0 > 10
    assert plastic.any()
    print(f"\nrecycle, precision {precision}, preconditioner {precond}: PCG iterations in the plastic steps "
          f"{cg0[plastic].sum()} -> {cg1[plastic].sum()}, displacement difference {err:.2e}")
    assert cg1[plastic].sum() < 0.8 * cg0[plastic].sum()
