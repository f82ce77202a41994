"""The C-ABI libraries load on a machine without a GPU and export every symbol
their headers declare; calls fail loudly (no CPU fallback) when no GPU exists."""
import ctypes as C
import os
import re

import pytest

from conftest import ROOT

INCLUDE = os.path.join(ROOT, "include")


def declared_functions(header):
    text = open(os.path.join(INCLUDE, header)).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    text = re.sub(r"//[^\n]*", "", text)
    names = re.findall(r"\b([A-Za-z_][A-Za-z0-9_]*)\s*\([^;{]*\)\s*;", text)
    return sorted(set(n for n in names if n not in ("if", "while", "for", "return", "sizeof")))


def test_gpu_library_exports_header(gpu_lib):
    names = declared_functions("lpm_gpu.h")
    assert len(names) >= 25
    lib = gpu_lib.load()
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    assert set(names) == set(gpu_lib.EXPORTED)


def test_no_silent_cpu_fallback(gpu_lib):
    """lpm_create must fail with a CUDA error when there is no device."""
    import subprocess
    import sys
    code = ("import sys; sys.path.insert(0, %r); import ctypes as C, lpm_gb300 as G; L = G.load(); "
            "h = C.c_void_p(); rc = L.lpm_create(C.byref(h), 0); print(rc)" % os.path.join(ROOT, "lpm-c_gb300"))
    env = dict(os.environ, CUDA_VISIBLE_DEVICES="")
    out = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, env=env)
    assert out.returncode == 0, out.stderr
    assert int(out.stdout.strip().splitlines()[-1]) == -2  # LPM_ERR_CUDA


def test_legacy_library_exports_header():
    path = os.path.join(ROOT, "lpm-c_gb300", "_build", "liblpmgpu_legacy.so")
    hdr = os.path.join(INCLUDE, "lpm_legacy.h")
    if not os.path.exists(hdr):
        pytest.skip("legacy header not present")
    assert os.path.exists(path), "legacy drop-in library not built"
    # the legacy library resolves the include/lpm.h globals from its host
    # program; the C host driver library defines them
    host = os.path.join(ROOT, "lpm-c_gb300", "_build", "liblpmhost.so")
    assert os.path.exists(host), "C host driver library not built"
    hlib = C.CDLL(host, mode=C.RTLD_GLOBAL)
    lib = C.CDLL(path)
    names = declared_functions("lpm_legacy.h")
    assert len(names) >= 30
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    for g in ("xyz", "K_global", "dLp", "J2_alpha", "residual", "nparticle"):
        assert hasattr(hlib, g), g


def test_struct_layouts_match_header(gpu_lib, tmp_path):
    """The ctypes mirrors of the option and statistics structs have the C
    header's size and field offsets (a field appended on one side only would
    shift every later one)."""
    import subprocess
    structs = {"lpm_solver_opts": gpu_lib.SolverOpts, "lpm_step_stats": gpu_lib.StepStats,
               "lpm_damage_opts": gpu_lib.DamageOpts, "lpm_adjoint_opts": gpu_lib.AdjointOpts,
               "lpm_adjoint_stats": gpu_lib.AdjointStats, "lpm_tuning": gpu_lib.Tuning}
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "lpm_gpu.h"', "int main(void) {"]
    for cname, py in structs.items():
        lines.append('printf("%s %%zu\\n", sizeof(%s));' % (cname, cname))
        for f, _ in py._fields_:
            lines.append('printf("%s.%s %%zu\\n", offsetof(%s, %s));' % (cname, f, cname, f))
    lines.append("return 0; }")
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.check_call(["gcc", "-std=c11", "-I", INCLUDE, "-o", str(exe), str(src)])
    got = dict(l.split() for l in subprocess.check_output([str(exe)], text=True).splitlines())
    for cname, py in structs.items():
        if cname not in ("lpm_solver_opts", "lpm_adjoint_opts"):  # returned to callers as dicts
            d = py().as_dict()
            assert list(d) == [f for f, _ in py._fields_], cname
        assert int(got[cname]) == C.sizeof(py), cname
        for f, _ in py._fields_:
            assert int(got[f"{cname}.{f}"]) == getattr(py, f).offset, (cname, f)
