"""GPU parity against the oracle (the CPU restatement pinned to the reference).

Bit-exact: bond lists, AFEM connectivity and the upper-CSR pattern; the FP64
bond-force kernels (elastic predictor, J2 return map, averaged force) on the
same input state.  Tolerance-based: the analytic tangent against the
reference's forward-difference stiffness; PCG solutions; load steps.
"""
import numpy as np
import pytest

import cases
from setup_helpers import sc_gpu, sc_oracle

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def sc10(oracle_mod, gpu_lib):
    case = cases.SCCase(n=10)
    o, types = sc_oracle(oracle_mod, case)
    s, types2 = sc_gpu(gpu_lib, case)
    assert np.array_equal(types, types2)
    return case, o, s


def test_setup_bit_exact(sc10):
    case, o, s = sc10
    n, nn = o.n, o.nn
    assert s.n == n
    assert np.array_equal(s.get("xyz"), o.d("xyz", (n, 3)))
    assert np.array_equal(s.get("neighbors"), o.i("neighbors", (n, nn)))
    assert np.array_equal(s.get("nsign"), o.i("nsign", (n, nn)))
    assert np.array_equal(s.get("nb"), o.i("nb", (n,)))
    assert np.array_equal(s.get("distance_initial"), o.d("distance_initial", (n, nn)))
    cs0 = s.get("cs_initial")
    assert np.array_equal(cs0[:, :, 0], o.d("csx_initial", (n, nn)))
    assert np.array_equal(cs0[:, :, 2], o.d("csz_initial", (n, nn)))
    assert np.array_equal(s.get("conn"), o.i("conn", (n, 61)))
    kp = s.get("K_pointer")
    assert np.array_equal(kp[:n, 0], o.i("kp0", (n + 1,))[:n])
    assert np.array_equal(kp[:, 1], o.i("kp1", (n + 1,)))
    assert np.array_equal(s.get("Kn"), o.d("Kn", (n, nn)))
    assert np.array_equal(s.get("Tv"), o.d("Tv", (n, nn)))


def test_stiffness_vs_fd(sc10):
    """Analytic tangent vs the reference's finite-difference K (same layout)."""
    case, o, s = sc10
    o.fd_stiffness()
    s.assemble_stiffness()
    K, IK, JK = s.export_upper_csr()
    nnz = o.nnz
    assert np.array_equal(IK, o.i("IK", (3 * o.n + 1,)))
    assert np.array_equal(JK, o.i("JK", (nnz,)))
    Kf = o.d("K_global", (nnz,))
    rel = np.linalg.norm(K - Kf) / np.linalg.norm(Kf)
    # forward differences with h = 1e-6 r: truncation ~1e-6, rounding ~1e-9 / 1e-7
    assert rel < 1e-5, rel
