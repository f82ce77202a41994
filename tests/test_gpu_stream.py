"""The multigrid PCG's launch shapes: the streamed difference-form product
and the streamed level-0 smoother (tiles of 16 rows copied into
shared-memory stages by the bulk-copy engine) compute every row as the
register-fed kernels do, and the autotuner's choice among the product and
smoother shapes leaves later load steps where the untuned run puts them."""
import numpy as np
import pytest

import cases
from setup_helpers import sc_gpu

pytestmark = [pytest.mark.gpu, pytest.mark.gpu_option]


def _opts(G, precision):
    return dict(precision=precision, newton_maxiter=300, cg_rtol=1e-11, preconditioner=G.PRECOND_AMG,
                cg_maxiter=2000)


@pytest.mark.parametrize("edge,precision,diff_stream,smooth_stream",
                         [(12, 1, 1, 0), (30, 1, 1, 0), (30, 1, 2, 0), (30, 1, 3, 0), (12, 0, 0, 1), (30, 0, 0, 1),
                          (30, 0, 0, 2), (30, 0, 0, 3), (30, 1, 1, 1), (12, 1, 3, 3)])
def test_streamed_kernels_follow_register_fed(gpu_lib, edge, precision, diff_stream, smooth_stream):
    """The streamed product (mixed) and the streamed level-0 smoother (both
    precisions), alone and together; variants 1 and 2 walk tiles of 16 rows
    with 1 or 2 thread blocks per SM, variant 3 tiles of 8 rows with 5
    (product) or 6 (smoother).  SC 12^3: 108 tiles of 16 rows, fewer than
    thread blocks (most blocks get none).  SC 30^3: 1,688 tiles, the last one
    partial, and more tiles per thread block than the ring has stages (the
    stage barriers change phase); the FP16 values of half of the tiles start
    8 bytes off a 16-byte boundary."""
    G = gpu_lib
    case = cases.SCCase(n=edge, e_noise=0.05, newton_tol=1e-10)
    ref, _ = sc_gpu(G, case, **_opts(G, precision))
    st, _ = sc_gpu(G, case, **_opts(G, precision))
    st.set_tuning(diff_stream=diff_stream, smooth_stream=smooth_stream)
    t = st.get_tuning()
    assert t["diff_stream"] == diff_stream and t["smooth_stream"] == smooth_stream
    x0 = ref.get("xyz_initial")
    worst = 0.0
    for stp in case.schedule[:8]:
        a = ref.load_step(cases.sc_bcs(stp))
        b = st.load_step(cases.sc_bcs(stp))
        assert a["status"] == 0 and b["status"] == 0, (a["status"], b["status"])
        assert abs(a["cg_iters"] - b["cg_iters"]) <= 2 + a["cg_iters"] // 20
        da, db = ref.get("xyz") - x0, st.get("xyz") - x0
        err = float(np.abs(da - db).max() / np.abs(da).max())
        worst = max(worst, err)
        assert err <= 1e-9
    print(f"\nSC {edge}^3, precision {precision}, streamed product {diff_stream} / smoother {smooth_stream} "
          f"block(s) per SM: displacements within {worst:.2e} of the register-fed kernels")
    ref.close()
    st.close()


@pytest.mark.parametrize("precision", [0, 1])
def test_autotune_multigrid_then_solve(gpu_lib, precision):
    """With the multigrid preconditioner the tuner also picks the lanes per
    block row of the difference-form product or its streamed form (mixed)
    and of the level-0 smoother; later load steps follow the untuned run."""
    G = gpu_lib
    case = cases.SCCase(n=12, e_noise=0.05, newton_tol=1e-10)
    ref, _ = sc_gpu(G, case, **_opts(G, precision))
    tun, _ = sc_gpu(G, case, **_opts(G, precision))
    x0 = ref.get("xyz_initial")
    for k, stp in enumerate(case.schedule[:14]):
        a = ref.load_step(cases.sc_bcs(stp))
        b = tun.load_step(cases.sc_bcs(stp))
        if k == 0:
            t = tun.autotune()
            assert t["smooth_lanes"] in (4, 8, 16) and t["smooth_ms"] > 0.0
            assert t["diff_stream"] in ((0, 1, 2, 3) if precision == G.PREC_MIXED else (0,))
            assert t["smooth_stream"] in (0, 1, 2, 3)
        assert a["status"] == 0 and b["status"] == 0
        da, db = ref.get("xyz") - x0, tun.get("xyz") - x0
        assert np.abs(da - db).max() <= 1e-9 * np.abs(da).max()
    ref.close()
    tun.close()
