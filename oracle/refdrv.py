"""ctypes access to the LPM-C reference built from its own sources (oracle/_ref).

TEST INFRASTRUCTURE ONLY: used by tests/ (CPU, in the container that holds the
reference) and by tests/golden/make_golden.py to produce the golden vectors.
The library exists only where oracle/build_ref.sh could read the reference
sources; on machines without them :func:`available` is False.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_ref", "libref_lpm.so")

_lib = None


class DispBC(C.Structure):
    """struct dispBCPara (include/lpm.h:83-88)."""
    _fields_ = [("type", C.c_int), ("flag", C.c_char), ("step", C.c_double)]


class ForceBC(C.Structure):
    """struct forceBCPara (include/lpm.h:90-99)."""
    _fields_ = [("type", C.c_int), ("flag1", C.c_char), ("step1", C.c_double),
                ("flag2", C.c_char), ("step2", C.c_double),
                ("flag3", C.c_char), ("step3", C.c_double)]


def available():
    return os.path.exists(LIB_PATH)


def lib():
    global _lib
    if _lib is None:
        _lib = C.CDLL(LIB_PATH, mode=C.RTLD_GLOBAL)
        _lib.refd_setup.argtypes = [C.c_int, C.c_double, C.POINTER(C.c_double)]
        _lib.refd_load_step.argtypes = [C.c_int, C.POINTER(DispBC), C.c_int, C.POINTER(ForceBC),
                                        C.c_int, C.c_double, C.c_int, C.POINTER(C.c_double)]
        _lib.refd_set_cg_tol.argtypes = [C.c_double, C.c_double]
        _lib.refd_material.argtypes = [C.POINTER(C.c_double), C.c_int, C.POINTER(C.c_double),
                                       C.c_double, C.c_double, C.POINTER(C.c_double)]
        _lib.refd_set_threads(1)
    return _lib


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _ip(a):
    return a.ctypes.data_as(C.POINTER(C.c_int))


def gint(name):
    return C.c_int.in_dll(lib(), name).value


def gdouble(name):
    return C.c_double.in_dll(lib(), name).value


def get_d1(name, n):
    p = C.POINTER(C.c_double).in_dll(lib(), name)
    return np.ctypeslib.as_array(p, shape=(n,)).copy()


def get_i1(name, n):
    p = C.POINTER(C.c_int).in_dll(lib(), name)
    return np.ctypeslib.as_array(p, shape=(n,)).copy()


def get_d2(name, rows, cols):
    out = np.zeros((rows, cols))
    p = C.POINTER(C.POINTER(C.c_double)).in_dll(lib(), name)
    lib().refd_get_d2(p, rows, cols, _dp(out))
    return out


def get_i2(name, rows, cols):
    out = np.zeros((rows, cols), dtype=np.int32)
    p = C.POINTER(C.POINTER(C.c_int)).in_dll(lib(), name)
    lib().refd_get_i2(p, rows, cols, _ip(out))
    return out


def get_d3(name, rows, cols, slot):
    out = np.zeros((rows, cols))
    p = C.POINTER(C.POINTER(C.POINTER(C.c_double))).in_dll(lib(), name)
    lib().refd_get_d3(p, rows, cols, slot, _dp(out))
    return out


def set_d2(name, arr):
    arr = np.ascontiguousarray(arr, dtype=np.float64)
    p = C.POINTER(C.POINTER(C.c_double)).in_dll(lib(), name)
    lib().refd_set_d2(p, arr.shape[0], arr.shape[1], _dp(arr))


def setup(lattice, radius, box):
    box = np.asarray(box, dtype=np.float64)
    n = lib().refd_setup(lattice, radius, _dp(box))
    if n <= 0:
        raise RuntimeError("reference setup failed")
    return n


def set_types(types, ntype):
    t = np.ascontiguousarray(types, dtype=np.int32)
    lib().refd_set_types(_ip(t), int(ntype))


def set_bc_groups(groups):
    if groups is None:
        lib().refd_set_bc_groups(None)
    else:
        g = np.ascontiguousarray(groups, dtype=np.int32)
        lib().refd_set_bc_groups(_ip(g))


def material(ce, plmode, sigmay, xi, H, cp=None):
    ce = np.ascontiguousarray(ce, dtype=np.float64).reshape(-1)
    sy = np.ascontiguousarray(sigmay, dtype=np.float64)
    cpa = None if cp is None else np.ascontiguousarray(cp, dtype=np.float64)
    lib().refd_material(_dp(ce), plmode, _dp(sy), float(xi), float(H),
                        None if cpa is None else _dp(cpa))


def init_state():
    lib().refd_init_state()


def load_step(disp_bcs, force_bcs, newton_tol, maxiter=100, load_ind=1):
    """disp_bcs: list of (type, 'x'|'y'|'z', step); force_bcs: list of (type, fx, fy, fz)."""
    nd = len(disp_bcs)
    nf = len(force_bcs)
    darr = (DispBC * max(nd, 1))()
    for k, (t, f, s) in enumerate(disp_bcs):
        darr[k] = DispBC(t, f.encode(), s)
    farr = (ForceBC * max(nf, 1))()
    for k, (t, fx, fy, fz) in enumerate(force_bcs):
        farr[k] = ForceBC(t, b"x", fx, b"y", fy, b"z", fz)
    stats = np.zeros(5)
    lib().refd_load_step(nd, darr, nf, farr, load_ind, newton_tol, maxiter, _dp(stats))
    return stats


def set_damage(L=0.5, threshold=0.9, cA=0.0, crit_bstrain=1e-2, nbreak=20):
    """damage_L, damage_threshold, damagec_A, critical_bstrain, nbreak."""
    L_ = lib()
    L_.refd_set_damage.argtypes = [C.c_double, C.c_double, C.c_double, C.c_double, C.c_int]
    L_.refd_set_damage(L, threshold, cA, crit_bstrain, nbreak)


def load_step_damage(disp_bcs, force_bcs, newton_tol, bondfile, step, maxiter=100, max_passes=1000,
                     load_ind=1):
    """One load step of main with the damage stage; broken bonds are appended
    to `bondfile` by the reference.  Returns the 7 stats of refd_load_step_damage."""
    nd, nf = len(disp_bcs), len(force_bcs)
    darr = (DispBC * max(nd, 1))()
    for k, (t, f, s) in enumerate(disp_bcs):
        darr[k] = DispBC(t, f.encode(), s)
    farr = (ForceBC * max(nf, 1))()
    for k, (t, fx, fy, fz) in enumerate(force_bcs):
        farr[k] = ForceBC(t, b"x", fx, b"y", fy, b"z", fz)
    stats = np.zeros(7)
    L_ = lib()
    L_.refd_load_step_damage.argtypes = [C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_double,
                                         C.c_int, C.c_int, C.c_char_p, C.c_int, C.c_void_p]
    L_.refd_load_step_damage(nd, darr, nf, farr, load_ind, newton_tol, maxiter, max_passes,
                             bondfile.encode(), step, _dp(stats))
    return stats


def set_cg_tol(rtol_sq, atol_sq):
    """Override the reference's hard-coded dcg tolerances (squared norms)."""
    lib().refd_set_cg_tol(float(rtol_sq), float(atol_sq))


class quiet:
    """Silence the reference's printf output (C-level stdout) in a block."""

    def __enter__(self):
        import sys
        sys.stdout.flush()
        self.saved = os.dup(1)
        self.null = os.open(os.devnull, os.O_WRONLY)
        os.dup2(self.null, 1)
        return self

    def __exit__(self, *exc):
        C.CDLL(None).fflush(None)
        os.dup2(self.saved, 1)
        os.close(self.saved)
        os.close(self.null)
        return False


def nparticle():
    return gint("nparticle")
