"""Output writers against the reference's own writeDump / writeDisp /
writeReaction / writeStress (golden files from tests/golden/make_output_golden.py):
byte-identical text for the same arrays.  Runs without a GPU (host-array
formatters of the CUDA library)."""
import ctypes as C
import os

import numpy as np
import pytest

import cases
from conftest import golden

FIXTURES = ["output_sc6_j2.npz", "output_fcc2_cp.npz"]


def _dp(a):
    return np.ascontiguousarray(a, dtype=np.float64).ctypes.data_as(C.POINTER(C.c_double))


def _ip(a):
    return np.ascontiguousarray(a, dtype=np.int32).ctypes.data_as(C.POINTER(C.c_int))


def text(d, key):
    return bytes(d["text_" + key]).decode()


@pytest.mark.parametrize("fixture", FIXTURES)
def test_formats_match_reference_writers(gpu_lib, tmp_path, fixture):
    d = golden(fixture)
    L = gpu_lib.load()
    n = d["type"].shape[0]
    nn = d["F"].shape[1]
    step = int(d["step"])
    cp = "cp_A" in d
    keep = []  # keep converted arrays alive across the calls

    def arr(a, f):
        b = np.ascontiguousarray(a)
        keep.append(b)
        return f(b)

    p = str(tmp_path / "dump.txt").encode()
    if cp:
        ns = d["cp_A_single"].shape[1]
        rc = L.lpm_format_dump(p, step, b"s", n, arr(d["box"], _dp), 1, arr(d["type"], _ip), arr(d["xyz"], _dp),
                               arr(d["xyz0"], _dp), arr(d["stress"], _dp), None, arr(d["pl_flag"], _ip),
                               arr(d["cp_A_single"], _dp), ns, arr(d["cp_A"], _dp))
    else:
        rc = L.lpm_format_dump(p, step, b"s", n, arr(d["box"], _dp), 0, arr(d["type"], _ip), arr(d["xyz"], _dp),
                               arr(d["xyz0"], _dp), arr(d["stress"], _dp), arr(d["alpha"], _dp),
                               arr(d["pl_flag"], _ip), None, 0, None)
    assert rc == 0
    assert open(p.decode()).read() == text(d, "dump")
    p = str(tmp_path / "disp.txt").encode()
    assert L.lpm_format_disp(p, b"z", cases.T_TOP, step, n, arr(d["type"], _ip), arr(d["xyz"], _dp),
                             arr(d["xyz0"], _dp)) == 0
    assert open(p.decode()).read() == text(d, "disp")
    p = str(tmp_path / "reaction.txt").encode()
    assert L.lpm_format_reaction(p, b"z", cases.T_TOP, step, n, nn, arr(d["type"], _ip), arr(d["nb"], _ip),
                                 arr(d["csx"], _dp), arr(d["csy"], _dp), arr(d["csz"], _dp), arr(d["F"], _dp)) == 0
    assert open(p.decode()).read() == text(d, "reaction")
    p = str(tmp_path / "stress.txt").encode()
    assert L.lpm_format_stress(p, cases.T_INTERIOR, step, n, arr(d["type"], _ip), arr(d["stress"], _dp)) == 0
    assert open(p.decode()).read() == text(d, "stress")
    if "strain" in d:
        p = str(tmp_path / "strain.txt").encode()
        assert L.lpm_format_strain(p, cases.T_INTERIOR, step, n, arr(d["type"], _ip), arr(d["strain"], _dp)) == 0
        assert open(p.decode()).read() == text(d, "strain")


def test_dump_appends(gpu_lib, tmp_path):
    """flag 's' starts the file, any other flag appends a frame."""
    z = golden("output_sc6_j2.npz")
    d = {k: np.ascontiguousarray(z[k]) for k in ("box", "type", "xyz", "xyz0", "stress", "alpha", "pl_flag")}
    d["type"] = d["type"].astype(np.int32)
    d["pl_flag"] = d["pl_flag"].astype(np.int32)
    L = gpu_lib.load()
    n = d["type"].shape[0]
    p = str(tmp_path / "dump.txt").encode()
    args = [n, _dp(d["box"]), 0, _ip(d["type"]), _dp(d["xyz"]), _dp(d["xyz0"]), _dp(d["stress"]), _dp(d["alpha"]),
            _ip(d["pl_flag"]), None, 0, None]
    assert L.lpm_format_dump(p, 1, b"s", *args) == 0
    assert L.lpm_format_dump(p, 2, b"a", *args) == 0
    s = open(p.decode()).read()
    assert s.count("ITEM: TIMESTEP") == 2 and s.startswith("ITEM: TIMESTEP\n1\n")
