"""Build recipe of the GB300 LPM library (in-tree, no cmake).

    python lpm-c_gb300/build.py          # -> lpm-c_gb300/_build/liblpmgpu.so

CUDA sources are compiled for sm_103a only; the FP64 force kernels are built
with -fmad=false so that their arithmetic follows the reference's operation
order exactly.  Host setup code is compiled with -ffp-contract=off for the
same reason.  Translation units compile in parallel.
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "liblpmgpu.so")
LEGACY_LIB = os.path.join(OUT, "liblpmgpu_legacy.so")
HOST_LIB = os.path.join(OUT, "liblpmhost.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-I", INCLUDE,
               "--expt-relaxed-constexpr"]
# (file, extra flags)
CU_UNITS = [
    ("k_force.cu", ["-fmad=false"]),
    ("k_cp.cu", ["-fmad=false"]),
    ("k_stiff.cu", []),
    ("k_solve.cu", []),
    ("lpm_api.cu", ["-Xcompiler", "-fopenmp"]),
    ("k_batch.cu", []),
    ("k_adjoint.cu", ["-fmad=false"]),
    ("k_strain.cu", ["-fmad=false"]),
    ("adjoint.cu", []),
    ("k_noalloc.cu", []),
    ("k_damage.cu", ["-fmad=false"]),
    ("k_amg.cu", ["-Xcompiler", "-fopenmp"]),
]
CPP_UNITS = [("setup.cpp", ["-ffp-contract=off", "-fopenmp"]), ("output.cpp", ["-ffp-contract=off"]),
             ("amg_setup.cpp", ["-O3", "-fopenmp"])]
LEGACY_UNITS = [("legacy.cpp", ["-fopenmp"])]


def _nvcc():
    for p in ("/usr/local/cuda/bin/nvcc", "nvcc"):
        if os.path.sep not in p or os.path.exists(p):
            return p
    return "nvcc"


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _headers():
    hs = [os.path.join(SRC, f) for f in os.listdir(SRC) if f.endswith(".h")]
    hs += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")]
    return hs


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: " + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stdout + r.stderr


def build(verbose=False, ptxas_info=False):
    os.makedirs(OUT, exist_ok=True)
    nvcc = _nvcc()
    hdr = _headers()
    jobs = []
    objs = []
    for f, extra in CU_UNITS:
        src = os.path.join(SRC, f)
        obj = os.path.join(OUT, f + ".o")
        objs.append(obj)
        if _stale(obj, [src] + hdr) or ptxas_info:
            cmd = [nvcc] + ARCH + NVCC_COMMON + extra + ["-c", src, "-o", obj]
            if ptxas_info:
                cmd.insert(1, "-Xptxas=-v")
            jobs.append(cmd)
    for f, extra in CPP_UNITS:
        src = os.path.join(SRC, f)
        obj = os.path.join(OUT, f + ".o")
        objs.append(obj)
        if _stale(obj, [src] + hdr):
            cuda_inc = "/usr/local/cuda/include"
            jobs.append(["g++", "-O2", "-std=c++17", "-fPIC", "-I", INCLUDE, "-I", cuda_inc] + extra +
                        ["-c", src, "-o", obj])
    with ThreadPoolExecutor(max_workers=max(2, min(8, os.cpu_count() or 2))) as ex:
        logs = list(ex.map(_run, jobs))
    if verbose or ptxas_info:
        for l in logs:
            if l.strip():
                print(l)
    if _stale(LIB, objs):
        _run([nvcc] + ARCH + ["-shared", "-o", LIB] + objs + ["-Xcompiler", "-fopenmp", "-lcudart"])
    # reference-named drop-in layer (operates on the include/lpm.h globals)
    lobjs = []
    for f, extra in LEGACY_UNITS:
        src = os.path.join(SRC, f)
        if not os.path.exists(src):
            continue
        obj = os.path.join(OUT, f + ".o")
        lobjs.append(obj)
        if _stale(obj, [src] + hdr):
            _run(["g++", "-O2", "-std=c++17", "-fPIC", "-I", INCLUDE] + extra + ["-c", src, "-o", obj])
    if lobjs and _stale(LEGACY_LIB, lobjs + [LIB]):
        _run(["g++", "-shared", "-fopenmp", "-o", LEGACY_LIB] + lobjs + ["-L", OUT, "-llpmgpu",
                                                                         "-Wl,-rpath,$ORIGIN"])
    # C host driver: defines the include/lpm.h globals, runs the reference loop
    host_src = os.path.join(HERE, "host", "lpm_host.c")
    if os.path.exists(host_src) and _stale(HOST_LIB, [host_src, LEGACY_LIB] + hdr):
        _run(["gcc", "-std=gnu11", "-O2", "-fPIC", "-shared", "-ffp-contract=off", "-I", INCLUDE,
              "-o", HOST_LIB, host_src, "-L", OUT, "-llpmgpu_legacy", "-llpmgpu",
              "-Wl,-rpath,$ORIGIN", "-lm"])
    return LIB


if __name__ == "__main__":
    build(verbose=True, ptxas_info="--ptxas" in sys.argv)
    print("built", LIB)
