"""lpm_update_rr_noalloc (the allocation-free residual update) against the
context entry point lpm_compute_force, through the C ABI.

The residual is elementwise arithmetic and must match exactly; the two norms
are deterministic sums taken in a different order, compared at rtol 1e-12."""
import ctypes as C

import numpy as np
import pytest

import cases
from setup_helpers import sc_gpu

NORM_RTOL = 1e-12


def _dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def _noalloc(G, Pin, Pex, bc, norms=True):
    """One call of the entry point on device copies of the host arrays;
    returns (residual, norms) on the host."""
    import torch
    L = G.load()
    n = Pin.shape[0]
    d_pin, d_pex, d_bc = _dev(Pin), _dev(Pex), _dev(bc.astype(np.int32))
    d_res = torch.full((n, 3), np.nan, dtype=torch.float64, device="cuda")
    out = np.full(2, np.nan)
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    rc = L.lpm_update_rr_noalloc(n, C.c_void_p(d_pin.data_ptr()), C.c_void_p(d_pex.data_ptr()),
                                 C.c_void_p(d_bc.data_ptr()), C.c_void_p(d_res.data_ptr()),
                                 out.ctypes.data_as(C.POINTER(C.c_double)) if norms else None, stream)
    assert rc == 0, L.lpm_last_error().decode()
    torch.cuda.synchronize()
    return d_res.cpu().numpy(), out


def _context_state(s):
    return s.get("Pin"), s.get("Pex"), s.get("dispBC_index"), s.get("residual")


def _check(G, s, norms_ref):
    Pin, Pex, bc, res_ref = _context_state(s)
    res, norms = _noalloc(G, Pin, Pex, bc)
    assert np.array_equal(res, res_ref)
    assert np.allclose(norms, norms_ref, rtol=NORM_RTOL, atol=0.0), (norms, norms_ref)
    return norms


@pytest.mark.gpu
def test_noalloc_matches_compute_force_two_calls(gpu_lib):
    """Two calls in a row on one specimen (different states), then a call on a
    smaller specimen: each equals what lpm_compute_force computed."""
    G = gpu_lib
    case = cases.SCCase(n=20, e_noise=0.1)  # 8000 particles: 32 blocks of 256
    s, _ = sc_gpu(G, case)
    n = s.n
    rng = np.random.default_rng(7)
    s.set("Pex", rng.uniform(-1.0, 1.0, (n, 3)))
    s.begin_step()
    s.apply_bc(cases.sc_bcs(case.schedule[0]))
    norms1 = _check(G, s, s.compute_force(G.PL_J2))
    assert norms1[0] > 0.0 and norms1[1] > 0.0
    # second call: state after one Newton correction
    s.assemble_stiffness()
    s.solve()
    norms2 = _check(G, s, s.compute_force(G.PL_J2))
    assert not np.allclose(norms1, norms2)
    # a smaller specimen (one block): nothing of the larger call leaks into it
    small = cases.SCCase(n=6)
    t, _ = sc_gpu(G, small)
    t.begin_step()
    t.apply_bc(cases.sc_bcs(small.schedule[0]))
    _check(G, t, t.compute_force(G.PL_J2))
    s.close()
    t.close()


@pytest.mark.gpu
def test_noalloc_without_norms(gpu_lib):
    """norms == NULL: only the residual is written (stream-ordered, no wait)."""
    G = gpu_lib
    case = cases.SCCase(n=8)
    s, _ = sc_gpu(G, case)
    s.begin_step()
    s.apply_bc(cases.sc_bcs(case.schedule[0]))
    s.compute_force(G.PL_J2)
    Pin, Pex, bc, res_ref = _context_state(s)
    res, _ = _noalloc(G, Pin, Pex, bc, norms=False)
    assert np.array_equal(res, res_ref)
    s.close()


def test_noalloc_rejects_oversize(gpu_lib):
    """Sizes beyond the fixed scratch limit fail with LPM_ERR_ARG before any
    device work (runs without a GPU)."""
    L = gpu_lib.load()
    limit = 4194304  # LPM_NOALLOC_MAX_PARTICLES
    out = np.zeros(2)
    rc = L.lpm_update_rr_noalloc(limit + 1, None, None, None, None,
                                 out.ctypes.data_as(C.POINTER(C.c_double)), None)
    assert rc == -1
    msg = L.lpm_last_error().decode()
    assert "4194304" in msg and "limit" in msg
    assert L.lpm_update_rr_noalloc(-1, None, None, None, None, None, None) == -1
