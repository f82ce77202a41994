"""Anderson-accelerated Newton loop (opts.newton_accel) against the
reference's plain modified Newton: same converged displacements, fewer
iterations in the plastic range."""
import numpy as np
import pytest

import cases
from setup_helpers import sc_gpu

pytestmark = [pytest.mark.gpu, pytest.mark.gpu_option]


def test_anderson_matches_modified_newton_sc(gpu_lib):
    case = cases.SCCase(n=10, newton_tol=1e-10)
    plain, _ = sc_gpu(gpu_lib, case, precision=0, newton_maxiter=2000, cg_rtol=1e-12)
    accel, _ = sc_gpu(gpu_lib, case, precision=0, newton_maxiter=2000, cg_rtol=1e-12, newton_accel=8)
    x0 = plain.get("xyz_initial")
    it_plain = it_accel = 0
    for stp in case.schedule[:24]:
        a = plain.load_step(cases.sc_bcs(stp))
        b = accel.load_step(cases.sc_bcs(stp))
        assert a["status"] == 0 and b["status"] == 0, (a, b)
        it_plain += a["newton_iters"]
        it_accel += b["newton_iters"]
        da, db = plain.get("xyz") - x0, accel.get("xyz") - x0
        assert np.abs(da - db).max() <= 1e-8 * np.abs(da).max()
    # two solutions each converged to a 1e-10 residual: plastic strains agree to ~1e-8
    assert np.abs(plain.get("J2_alpha") - accel.get("J2_alpha")).max() <= 1e-7 * plain.get("J2_alpha").max()
    assert plain.get("J2_alpha").max() > 0.0
    assert it_accel < it_plain, (it_accel, it_plain)
    plain.close()
    accel.close()


def test_anderson_on_notched_plate(gpu_lib):
    G = gpu_lib
    plate = cases.NotchedPlate(nx=10, ny=2, nz=12, notch=4, steps=6, strain=0.006, corr=3.0)
    E, nu, sy, H = plate.fields(1)
    c11, c12, c44 = cases.iso_cubic(E, nu)
    runs = []
    for accel in (0, 8):
        s = G.Specimen(0)
        s.setup_particles(plate.lattice, plate.radius, plate.xyz)
        s.set_types(cases.sc_types(s.get("xyz"), s.get("nb"), plate.radius))
        s.set_material(c11, c12, c44, sy, H, 0.0, G.PL_J2)
        s.init_state()
        s.set_solver(precision=0, newton_tol=1e-11, newton_maxiter=3000, cg_rtol=1e-13, newton_accel=accel)
        its = 0
        for b in plate.step_bcs():
            st = s.load_step(b)
            assert st["status"] == 0, (accel, st)
            its += st["newton_iters"]
        runs.append((s.get("xyz") - s.get("xyz_initial"), its))
        s.close()
    (da, ia), (db, ib) = runs
    assert np.abs(da - db).max() <= 1e-8 * np.abs(da).max()
    assert ib * 3 < ia, (ib, ia)
