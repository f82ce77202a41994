"""Autotuner and SpMV launch shapes: every shape computes the same product
(up to the order of the row sums), the tuner returns a valid shape, and a
solve with a tuned shape follows the default solve."""
import numpy as np
import pytest

import cases
from setup_helpers import batch_gpu, sc_gpu

pytestmark = pytest.mark.gpu

SHAPES = [(v, g) for v in range(4) for g in (2, 16)]


@pytest.mark.parametrize("precision,rtol", [(0, 1e-13), (1, 2e-6)])
def test_spmv_shapes_agree(gpu_lib, precision, rtol):
    case = cases.SCCase(n=12, e_noise=0.05)
    s, _ = sc_gpu(gpu_lib, case, precision=precision)
    s.assemble_stiffness()
    rng = np.random.default_rng(5)
    x = rng.standard_normal((s.n, 3))
    y0 = s.spmv(x)
    scale = np.abs(y0).max()
    for v, g in SHAPES:
        s.set_tuning(spmv_variant=v, spmv_per_sm=g, cg_per_sm=g)
        t = s.get_tuning()
        assert (t["spmv_lanes"], t["spmv_blocks"]) == [(16, 4), (8, 4), (32, 2), (4, 4)][v]
        y = s.spmv(x)
        assert np.abs(y - y0).max() <= rtol * scale, (v, g)
    s.close()


def test_autotune_then_solve(gpu_lib):
    case = cases.SCCase(n=10, newton_tol=1e-10)
    ref, _ = sc_gpu(gpu_lib, case, precision=1, newton_maxiter=300, cg_rtol=1e-11)
    tun, _ = sc_gpu(gpu_lib, case, precision=1, newton_maxiter=300, cg_rtol=1e-11)
    tun.assemble_stiffness()
    t = tun.autotune()
    assert 0 <= t["spmv_variant"] <= 3 and 1 <= t["spmv_per_sm"] <= 16 and 1 <= t["cg_per_sm"] <= 16
    assert 0.0 < t["spmv_ms"] <= t["spmv_ms_default"] * 1.0001
    x0 = ref.get("xyz_initial")
    for stp in case.schedule[:14]:
        a = ref.load_step(cases.sc_bcs(stp))
        b = tun.load_step(cases.sc_bcs(stp))
        assert a["status"] == 0 and b["status"] == 0
        da, db = ref.get("xyz") - x0, tun.get("xyz") - x0
        assert np.abs(da - db).max() <= 1e-9 * np.abs(da).max()
    ref.close()
    tun.close()


def test_batch_with_other_shape(gpu_lib):
    case = cases.BatchCase(nspec=5, edge_lo=4, edge_hi=8, strain=0.004, steps=8, seed=11)
    a, off = batch_gpu(gpu_lib, case, precision=0, newton_maxiter=300, cg_rtol=1e-11)
    b, _ = batch_gpu(gpu_lib, case, precision=0, newton_maxiter=300, cg_rtol=1e-11)
    b.set_tuning(spmv_variant=2, spmv_per_sm=4, cg_per_sm=16)
    x0 = a.get("xyz_initial")
    for _ in range(3):
        a.batch_load_step(case.step_bcs())
        b.batch_load_step(case.step_bcs())
    da, db = a.get("xyz") - x0, b.get("xyz") - x0
    assert np.abs(da - db).max() <= 1e-9 * np.abs(da).max()
    a.close()
    b.close()
