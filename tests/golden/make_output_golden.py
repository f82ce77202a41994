"""Golden files of the reference's output writers (src/data_handler.c).

Runs the LPM-C reference built from its own sources (oracle/_ref) into the
plastic range and writes, with the reference's own writeDump, writeDisp,
writeReaction, writeStress and writeStrain (after computeStress and
computeStrain), the files its main loop writes (src/lpmc_project.c:466-515).
Stores those files' text together with the arrays the writers read, so the
repository's writers can be checked byte for byte without the reference:

    python tests/golden/make_output_golden.py

-> tests/golden/output_sc6_j2.npz (J2, SC 6^3, 14 steps of the cyclic case with
   a lowered yield stress) and tests/golden/output_fcc2_cp.npz (crystal
   plasticity, FCC 2^3 cells, 12 steps).  The reference runs single-threaded.
"""
import ctypes as C
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, HERE)

import refdrv as R  # noqa: E402
import cases  # noqa: E402


def write_all(tmp, t_disp, comp, step):
    L = R.lib()
    L.computeStress()
    L.computeStrain()
    names = {k: os.path.join(tmp, k + ".txt") for k in ("dump", "disp", "reaction", "stress", "strain")}
    L.writeDump.argtypes = [C.c_char_p, C.c_int, C.c_char]
    L.writeDisp.argtypes = [C.c_char_p, C.c_char, C.c_int, C.c_int]
    L.writeReaction.argtypes = [C.c_char_p, C.c_char, C.c_int, C.c_int]
    L.writeStress.argtypes = [C.c_char_p, C.c_int, C.c_int]
    L.writeStrain.argtypes = [C.c_char_p, C.c_int, C.c_int]
    L.writeDump(names["dump"].encode(), step, b"s")
    L.writeDisp(names["disp"].encode(), comp, t_disp, step)
    L.writeReaction(names["reaction"].encode(), comp, t_disp, step)
    L.writeStress(names["stress"].encode(), cases.T_INTERIOR, step)
    L.writeStrain(names["strain"].encode(), cases.T_INTERIOR, step)
    return {k: open(v).read() for k, v in names.items()}


def arrays(n, nn, xyz0, types, box):
    return dict(
        box=np.array(box), type=types, xyz=R.get_d2("xyz", n, 3), xyz0=xyz0,
        stress=R.get_d2("stress_tensor", n, 6), pl_flag=R.get_i1("pl_flag", n), nb=R.get_i1("nb", n),
        csx=R.get_d2("csx", n, nn), csy=R.get_d2("csy", n, nn), csz=R.get_d2("csz", n, nn), F=R.get_d2("F", n, nn),
        dL=R.get_d2("dL", n, nn), distance_initial=R.get_d2("distance_initial", n, nn))


def sc_j2(tmp):
    case = cases.SCCase(n=6, sigmay=150.0)
    n = R.setup(case.lattice, case.radius, case.box)
    nn = R.gint("nneighbors")
    xyz0 = R.get_d2("xyz", n, 3)
    types = cases.sc_types(xyz0, R.get_i1("nb", n), case.radius)
    R.set_types(types, cases.NTYPE)
    R.material(case.ce_per_type(), 0, np.full(n, case.sigmay), 0.0, case.H)
    R.init_state()
    R.set_cg_tol(1e-20, 0.0)
    nsteps = 14
    for stp in case.schedule[:nsteps]:
        with R.quiet():
            R.load_step(cases.sc_bcs(stp), [], case.newton_tol)
    out = arrays(n, nn, xyz0, types, case.box)
    out["alpha"] = R.get_d2("J2_alpha", n, 3)[:, 0]
    texts = write_all(tmp, cases.T_TOP, b"z", nsteps)
    out["strain"] = R.get_d2("strain_tensor", n, 6)
    out.update({"text_" + k: np.frombuffer(v.encode(), dtype=np.uint8) for k, v in texts.items()})
    out["step"] = nsteps
    return out


def fcc_cp(tmp):
    case = cases.FCCCase(ncell=2, strain=0.05, steps=60)
    n = R.setup(case.lattice, case.radius, case.box)
    nn = R.gint("nneighbors")
    xyz0 = R.get_d2("xyz", n, 3)
    types = cases.sc_types(xyz0, R.get_i1("nb", n), case.radius)
    R.set_types(types, cases.NTYPE)
    R.material(case.ce_per_type(), 1, np.zeros(n), 0.0, 0.0, np.array(case.cp))
    R.init_state()
    R.set_cg_tol(1e-20, 0.0)
    ns = R.gint("nslipSys")
    nsteps = 12
    for stp in case.schedule[:nsteps]:
        with R.quiet():
            R.load_step(cases.sc_bcs(stp), [], case.newton_tol)
    out = arrays(n, nn, xyz0, types, case.box)
    out["cp_A_single"] = R.get_d3("cp_A_single", n, ns, 0)
    out["cp_A"] = R.get_d2("cp_A", n, 3)[:, 0]
    texts = write_all(tmp, cases.T_TOP, b"z", nsteps)
    out.update({"text_" + k: np.frombuffer(v.encode(), dtype=np.uint8) for k, v in texts.items()})
    out["step"] = nsteps
    return out


def main():
    which = sys.argv[1] if len(sys.argv) > 1 else None
    if which is None:  # one process per case: the reference keeps global state
        import subprocess
        for w in ("sc", "fcc"):
            subprocess.check_call([sys.executable, __file__, w])
        return
    R.lib()
    with tempfile.TemporaryDirectory() as tmp:
        if which == "sc":
            np.savez_compressed(os.path.join(HERE, "output_sc6_j2.npz"), **sc_j2(tmp))
        else:
            np.savez_compressed(os.path.join(HERE, "output_fcc2_cp.npz"), **fcc_cp(tmp))


if __name__ == "__main__":
    main()
