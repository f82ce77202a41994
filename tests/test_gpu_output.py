"""Output writers on the GPU path: the same cases as the reference's golden
output files (tests/golden/make_output_golden.py) run on the GPU, written by
the context writers (writeDump asynchronously, while the next load step
runs), compared field by field with the reference's text; integer fields
exactly, printed reals to the 5 significant digits they carry."""
import numpy as np
import pytest

import cases
from conftest import golden

pytestmark = pytest.mark.gpu


def fields(txt):
    return [ln.split() for ln in txt.splitlines()]


def same_text(ours, ref):
    a, b = fields(ours), fields(ref)
    assert len(a) == len(b)
    for la, lb in zip(a, b):
        assert len(la) == len(lb), (la, lb)
        for x, y in zip(la, lb):
            if x == y:
                continue
            fx, fy = float(x), float(y)  # a printed real one digit apart
            assert abs(fx - fy) <= 2e-4 * max(abs(fy), 1e-6), (x, y, la[:2])


def run_sc(G):
    case = cases.SCCase(n=6, sigmay=150.0)
    s = G.Specimen(0)
    n = s.setup_lattice(case.lattice, case.radius, case.box)
    s.set_types(cases.sc_types(s.get("xyz"), s.get("nb"), case.radius))
    c11, c12, c44 = cases.iso_cubic(case.E, case.nu)
    s.set_material(np.full(n, c11), np.full(n, c12), np.full(n, c44), case.sigmay, case.H, 0.0, G.PL_J2)
    s.init_state()
    s.set_solver(precision=0, newton_tol=case.newton_tol, cg_rtol=1e-10, newton_maxiter=300)
    return s, case


def test_writers_match_reference_sc(gpu_lib, tmp_path):
    G = gpu_lib
    d = golden("output_sc6_j2.npz")
    s, case = run_sc(G)
    for stp in case.schedule[:14]:
        st = s.load_step(cases.sc_bcs(stp))
        assert st["status"] == 0
    assert np.array_equal(s.get("pl_flag"), d["pl_flag"])
    p = {k: str(tmp_path / f"{k}.txt") for k in ("dump", "disp", "reaction", "stress")}
    s.write_disp(p["disp"], "z", cases.T_TOP, 14)
    s.write_reaction(p["reaction"], "z", cases.T_TOP, 14)
    s.write_stress(p["stress"], cases.T_INTERIOR, 14)
    s.write_dump(p["dump"], 14, "s", case.box)
    s.load_step(cases.sc_bcs(case.schedule[14]))  # runs while the dump is written
    s.write_wait()
    for k in p:
        same_text(open(p[k]).read(), bytes(d["text_" + k]).decode())
    s.close()


def test_strain_bit_exact(gpu_lib, tmp_path):
    """computeStrain on the GPU from the reference's bond stretches equals the
    reference's strain tensor bit for bit; writeStrain text too."""
    G = gpu_lib
    d = golden("output_sc6_j2.npz")
    s, case = run_sc(G)
    s.set("dL", d["dL"])
    e = s.compute_strain()
    assert np.array_equal(e, d["strain"])
    path = str(tmp_path / "strain.txt")
    s.write_strain(path, cases.T_INTERIOR, int(d["step"]))
    assert open(path).read() == bytes(d["text_strain"]).decode()
    s.close()


def test_dump_cp_matches_host_formatter(gpu_lib, tmp_path):
    """Crystal plasticity (FCC 4^3 cells into the plastic range, the case of
    tests/test_gpu_cp.py): the asynchronous device dump equals the host
    formatter fed with the same context's arrays, and pl_flag marks exactly
    the particles with slip."""
    import ctypes as C
    G = gpu_lib
    case = cases.FCCCase(ncell=4, newton_tol=1e-10)
    s = G.Specimen(0)
    n = s.setup_lattice(case.lattice, case.radius, case.box)
    types = cases.sc_types(s.get("xyz"), s.get("nb"), case.radius)
    s.set_types(types)
    s.set_cp(*case.cp)
    s.set_material(case.C11, case.C12, case.C44, 0.0, 0.0, 0.0, G.PL_CP)
    s.init_state()
    s.set_solver(precision=0, newton_tol=case.newton_tol, newton_maxiter=300, cg_rtol=1e-11)
    for stp in case.schedule[:11]:
        assert s.load_step(cases.sc_bcs(stp))["status"] == 0
    path = str(tmp_path / "dump.txt")
    s.write_dump(path, 11, "s", case.box)
    s.write_wait()
    A = s.get("cp_A")
    pl = s.get("pl_flag")
    assert A.max() > 0.0 and np.array_equal(pl > 0, A > 0)
    keep = dict(box=np.ascontiguousarray(case.box, dtype=np.float64), type=s.get("type"), xyz=s.get("xyz"),
                xyz0=s.get("xyz_initial"), stress=s.get("stress_tensor"), pl=pl, As=s.get("cp_A_single"), A=A)
    dp = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))  # noqa: E731
    ip = lambda a: a.ctypes.data_as(C.POINTER(C.c_int))  # noqa: E731
    ref = str(tmp_path / "host.txt")
    L = G.load()
    assert L.lpm_format_dump(ref.encode(), 11, b"s", n, dp(keep["box"]), 1, ip(keep["type"]), dp(keep["xyz"]),
                             dp(keep["xyz0"]), dp(keep["stress"]), None, ip(keep["pl"]), dp(keep["As"]),
                             keep["As"].shape[1], dp(keep["A"])) == 0
    assert open(path).read() == open(ref).read()
    s.close()
