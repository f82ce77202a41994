"""The multigrid preconditioner (opts.preconditioner = PRECOND_AMG) on the GPU:
the same load steps as the block-Jacobi PCG, to the same tolerances, with far
fewer PCG iterations.  Parity is against the oracle, as for the block-Jacobi
path (tests/test_gpu_parity.py): both solve every system to the same relative
tolerance, so the displacements agree to the Newton tolerance's level.  The
hierarchy itself is checked on the CPU (tests/test_amg_setup.py)."""
import numpy as np
import pytest

import cases
from setup_helpers import sc_gpu, sc_oracle

pytestmark = [pytest.mark.gpu, pytest.mark.gpu_option]


@pytest.mark.parametrize("precision", [0, 1])
def test_amg_load_steps_match_oracle(oracle_mod, gpu_lib, precision):
    """C1 cyclic case, SC 10^3, steps 1-15: displacements within 1e-8 of the
    oracle's, plastic state within 1e-10."""
    G = gpu_lib
    case = cases.SCCase(n=10, newton_tol=1e-10)
    o, _ = sc_oracle(oracle_mod, case, threads=4)
    s, _ = sc_gpu(G, case, precision=precision, newton_maxiter=300, cg_rtol=1e-10,
                  preconditioner=G.PRECOND_AMG)
    n = o.n
    x0 = o.d("xyz_initial", (n, 3))
    builds = 0
    for k, stp in enumerate(case.schedule[:15]):
        st = s.load_step(cases.sc_bcs(stp))
        o.load_step(cases.sc_bcs(stp), [], 1e-10, 300, 1e-20, 0.0)
        assert st["status"] == 0, st
        builds += st["amg_builds"]
        du_g = s.get("xyz") - x0
        du_o = o.d("xyz", (n, 3)) - x0
        err = np.abs(du_g - du_o).max() / np.abs(du_o).max()
        assert err < 1e-8, (k + 1, err, st)
    assert np.abs(s.get("J2_alpha") - o.d("alpha1", (n,))).max() < 1e-10
    assert 1 <= builds <= 3, builds


@pytest.mark.parametrize("precision", [0, 1])
def test_amg_fewer_iterations_same_answer(gpu_lib, precision):
    """SC 20^3, five cyclic steps: the same displacements as block-Jacobi
    (both to cg_rtol 1e-10, Newton 1e-10), at least 5x fewer PCG iterations."""
    G = gpu_lib
    case = cases.SCCase(n=20, newton_tol=1e-10)
    runs = []
    for pc in (G.PRECOND_BJ, G.PRECOND_AMG):
        s, _ = sc_gpu(G, case, precision=precision, newton_maxiter=300, cg_rtol=1e-10, preconditioner=pc)
        x0 = s.get("xyz")
        cg = 0
        for stp in case.schedule[:5]:
            st = s.load_step(cases.sc_bcs(stp))
            assert st["status"] == 0, st
            cg += st["cg_iters"]
        runs.append((s.get("xyz") - x0, cg))
    (du_bj, cg_bj), (du_amg, cg_amg) = runs
    err = np.abs(du_amg - du_bj).max() / np.abs(du_bj).max()
    assert err < 1e-8, err
    assert cg_amg * 5 < cg_bj, (cg_amg, cg_bj)


@pytest.mark.parametrize("precision", [0, 1])
def test_amg_fcc_cp(gpu_lib, precision):
    """FCC 4^3 cells, crystal plasticity: multigrid and block-Jacobi PCG
    give the same converged steps, in FP64 and in mixed precision."""
    G = gpu_lib
    case = cases.FCCCase(ncell=4)
    out = []
    for pc in (G.PRECOND_BJ, G.PRECOND_AMG):
        s = G.Specimen(0)
        n = s.setup_lattice(case.lattice, case.radius, case.box)
        s.set_types(cases.sc_types(s.get("xyz"), s.get("nb"), case.radius))
        s.set_cp(*case.cp)
        s.set_material(np.full(n, case.C11), np.full(n, case.C12), np.full(n, case.C44), 0.0, 0.0, 0.0, G.PL_CP)
        s.init_state()
        s.set_solver(precision=precision, newton_tol=1e-10, newton_maxiter=300, cg_rtol=1e-10, preconditioner=pc)
        x0 = s.get("xyz")
        for stp in case.schedule[:4]:
            st = s.load_step(cases.sc_bcs(stp))
            assert st["status"] == 0, st
        out.append(s.get("xyz") - x0)
    err = np.abs(out[1] - out[0]).max() / np.abs(out[0]).max()
    assert err < 1e-8, err


def test_amg_rebuild_on_new_constraints(gpu_lib):
    """A load step that constrains other DOFs rebuilds the hierarchy; the
    step after it with the same constraints does not."""
    G = gpu_lib
    case = cases.SCCase(n=10, newton_tol=1e-9)
    s, _ = sc_gpu(G, case, precision=0, newton_maxiter=300, cg_rtol=1e-10, preconditioner=G.PRECOND_AMG)
    st1 = s.load_step(cases.sc_bcs(case.schedule[0]))
    st2 = s.load_step(cases.sc_bcs(case.schedule[1]))
    assert st1["amg_builds"] == 1 and st2["amg_builds"] == 0, (st1, st2)
    # also hold the top face in x: a different DOF mask
    st3 = s.load_step(cases.sc_bcs(case.schedule[2]) + [(cases.T_TOP, "x", 0.0)])
    assert st3["amg_builds"] == 1 and st3["status"] == 0, st3
    st4 = s.load_step(cases.sc_bcs(case.schedule[3]) + [(cases.T_TOP, "x", 0.0)])
    assert st4["amg_builds"] == 0 and st4["status"] == 0, st4
