"""ctypes wrapper of the CPU restatement (lpm_oracle.c).

TEST INFRASTRUCTURE ONLY: the checker used by tests/, __graft_entry__.smoke()
and bench.py's CPU-baseline leg.  It never backs the product path.
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liblpm_oracle.so")

_lib = None


class DispBC(C.Structure):
    _fields_ = [("type", C.c_int), ("flag", C.c_char), ("step", C.c_double)]


class ForceBC(C.Structure):
    _fields_ = [("type", C.c_int), ("flag1", C.c_char), ("step1", C.c_double),
                ("flag2", C.c_char), ("step2", C.c_double),
                ("flag3", C.c_char), ("step3", C.c_double)]


def build(force=False):
    """Compile lpm_oracle.c + the MKL-API shim with gcc (OpenMP, no FP contraction)."""
    if os.path.exists(LIB_PATH) and not force:
        src = [os.path.join(HERE, f) for f in ("lpm_oracle.c", "lpm_oracle.h", "cg_rci.h",
                                               "mkl_shim/mkl_shim.c", "mkl_shim/mkl.h")]
        if all(os.path.getmtime(s) <= os.path.getmtime(LIB_PATH) for s in src):
            return LIB_PATH
    os.makedirs(os.path.dirname(LIB_PATH), exist_ok=True)
    cmd = ["gcc", "-std=gnu11", "-O2", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared",
           "-o", LIB_PATH, os.path.join(HERE, "lpm_oracle.c"),
           os.path.join(HERE, "mkl_shim", "mkl_shim.c"), "-lm"]
    subprocess.check_call(cmd)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB_PATH)
        vp = C.c_void_p
        L.lo_create.restype = vp
        L.lo_free.argtypes = [vp]
        L.lo_setup_lattice.argtypes = [vp, C.c_int, C.c_double, C.POINTER(C.c_double)]
        L.lo_setup_particles.argtypes = [vp, C.c_int, C.c_double, C.c_int, C.POINTER(C.c_double)]
        L.lo_set_types.argtypes = [vp, C.POINTER(C.c_int)]
        dp = C.POINTER(C.c_double)
        L.lo_set_material.argtypes = [vp, dp, dp, dp, dp, dp, C.c_double, C.c_int]
        L.lo_set_cp.argtypes = [vp, dp]
        for f in ("lo_init_state", "lo_computedL", "lo_fd_stiffness", "lo_bc_stiffness_update",
                  "lo_update_rr", "lo_csr_pattern"):
            getattr(L, f).argtypes = [vp]
        L.lo_fd_stiffness_range.argtypes = [vp, C.c_int, C.c_int]
        L.lo_cg_iterations.argtypes = [vp, C.c_int]
        L.lo_fd_stiffness_timing.argtypes = [vp, C.c_int, C.c_int]
        L.lo_fd_stiffness_timing.restype = C.c_double
        L.lo_set_disp_bc.argtypes = [vp, C.c_int, C.POINTER(DispBC)]
        L.lo_set_force_bc.argtypes = [vp, C.c_int, C.POINTER(ForceBC)]
        L.lo_solver_cg.argtypes = [vp, C.c_double, C.c_double]
        L.lo_force.argtypes = [vp, C.c_int]
        L.lo_switch_state.argtypes = [vp, C.c_int]
        L.lo_load_step.argtypes = [vp, C.c_int, C.POINTER(DispBC), C.c_int, C.POINTER(ForceBC),
                                   C.c_double, C.c_int, C.c_double, C.c_double, dp]
        for f in ("lo_n", "lo_nn", "lo_nnz", "lo_nslip", "lo_nconn_max"):
            getattr(L, f).argtypes = [vp]
        L.lo_d.argtypes = [vp, C.c_char_p]
        L.lo_d.restype = dp
        L.lo_i.argtypes = [vp, C.c_char_p]
        L.lo_i.restype = C.POINTER(C.c_int)
        L.lo_set_threads.argtypes = [C.c_int]
        L.lo_set_damage.argtypes = [vp, C.c_double, C.c_double, C.c_double, C.c_double, C.c_int]
        L.lo_damage_update.argtypes = [vp, C.c_int]
        L.lo_update_crack.argtypes = [vp]
        L.lo_broken_log.argtypes = [vp, C.POINTER(C.c_int)]
        L.lo_brittle_select.argtypes = [C.POINTER(C.c_int), C.POINTER(C.c_int), dp, C.c_int, C.c_int]
        L.lo_load_step_damage.argtypes = [vp, C.c_int, C.POINTER(DispBC), C.c_int, C.POINTER(ForceBC),
                                          C.c_double, C.c_int, C.c_double, C.c_double, C.c_int, dp]
        _lib = L
    return _lib


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def set_threads(n):
    lib().lo_set_threads(int(n))


def bc_arrays(disp_bcs, force_bcs):
    nd, nf = len(disp_bcs), len(force_bcs)
    darr = (DispBC * max(nd, 1))()
    for k, (t, f, s) in enumerate(disp_bcs):
        darr[k] = DispBC(t, f.encode(), s)
    farr = (ForceBC * max(nf, 1))()
    for k, (t, fx, fy, fz) in enumerate(force_bcs):
        farr[k] = ForceBC(t, b"x", fx, b"y", fy, b"z", fz)
    return nd, darr, nf, farr


def brittle_select(bi, bj, strain, nbreak):
    """updateBrittleDamage's choice among candidates given in scan order:
    the chosen (i, j) slots in the order they break."""
    bi = np.ascontiguousarray(bi, dtype=np.int32).copy()
    bj = np.ascontiguousarray(bj, dtype=np.int32).copy()
    bs = np.ascontiguousarray(strain, dtype=np.float64).copy()
    first = lib().lo_brittle_select(bi.ctypes.data_as(C.POINTER(C.c_int)), bj.ctypes.data_as(C.POINTER(C.c_int)),
                                    _dp(bs), len(bs), int(nbreak))
    return np.stack([bi[first:], bj[first:]], axis=1)


class Oracle:
    """One oracle instance (owns a lpm_oracle*)."""

    def __init__(self):
        self.L = lib()
        self.h = self.L.lo_create()

    def __del__(self):
        if getattr(self, "h", None):
            self.L.lo_free(self.h)
            self.h = None

    # ---- setup
    def setup_lattice(self, lattice, radius, box):
        box = np.ascontiguousarray(box, dtype=np.float64)
        n = self.L.lo_setup_lattice(self.h, lattice, radius, _dp(box))
        if n <= 0:
            raise RuntimeError("oracle lattice setup failed")
        return n

    def setup_particles(self, lattice, radius, xyz):
        xyz = np.ascontiguousarray(xyz, dtype=np.float64)
        return self.L.lo_setup_particles(self.h, lattice, radius, xyz.shape[0], _dp(xyz))

    def set_types(self, types):
        t = np.ascontiguousarray(types, dtype=np.int32)
        self.L.lo_set_types(self.h, t.ctypes.data_as(C.POINTER(C.c_int)))

    def set_material(self, c11, c12, c44, sy, H, xi=0.0, plmode=0):
        n = self.n
        arr = [np.ascontiguousarray(np.broadcast_to(np.asarray(v, dtype=np.float64), (n,)))
               for v in (c11, c12, c44, sy, H)]
        self._keep = arr
        self.L.lo_set_material(self.h, *[_dp(a) for a in arr], float(xi), int(plmode))

    def set_cp(self, tau0, taus, h0, p, q, eta, maxloop, dtime):
        cp = np.array([tau0, taus, h0, p, q, eta, maxloop, dtime], dtype=np.float64)
        self.L.lo_set_cp(self.h, _dp(cp))

    def init_state(self):
        self.L.lo_init_state(self.h)

    # ---- sizes / views
    @property
    def n(self):
        return self.L.lo_n(self.h)

    @property
    def nn(self):
        return self.L.lo_nn(self.h)

    @property
    def nnz(self):
        return self.L.lo_nnz(self.h)

    def d(self, name, shape):
        p = self.L.lo_d(self.h, name.encode())
        if not p:
            raise KeyError(name)
        return np.ctypeslib.as_array(p, shape=shape).copy()

    def i(self, name, shape):
        p = self.L.lo_i(self.h, name.encode())
        if not p:
            raise KeyError(name)
        return np.ctypeslib.as_array(p, shape=shape).copy()

    def set_d(self, name, arr):
        p = self.L.lo_d(self.h, name.encode())
        a = np.ascontiguousarray(arr, dtype=np.float64).reshape(-1)
        C.memmove(p, a.ctypes.data, a.nbytes)

    # ---- hot-path pieces
    def fd_stiffness(self):
        self.L.lo_fd_stiffness(self.h)

    def force(self, plmode):
        self.L.lo_force(self.h, plmode)

    def switch_state(self, flag):
        self.L.lo_switch_state(self.h, flag)

    def update_rr(self):
        self.L.lo_update_rr(self.h)

    # ---- damage (updateDamageGeneral, updateCrack, main's re-solve)
    def set_damage(self, L=0.5, threshold=0.9, cA=0.0, crit_bstrain=1e-2, nbreak=20):
        self.L.lo_set_damage(self.h, L, threshold, cA, crit_bstrain, nbreak)

    def damage_update(self, plmode):
        return self.L.lo_damage_update(self.h, plmode)

    def update_crack(self):
        self.L.lo_update_crack(self.h)

    def broken_log(self):
        k = self.L.lo_broken_log(self.h, None)
        out = np.zeros((k, 2), dtype=np.int32)
        if k:
            self.L.lo_broken_log(self.h, out.ctypes.data_as(C.POINTER(C.c_int)))
        return out

    def load_step_damage(self, disp_bcs, force_bcs, newton_tol, maxiter=100, cg_rtol_sq=1e-20,
                         cg_atol_sq=0.0, max_passes=1000):
        """stats: Newton iterations (all passes), |r0|, |reaction0|, final |r|, CG
        iterations, passes, bonds broken."""
        nd, darr, nf, farr = bc_arrays(disp_bcs, force_bcs)
        stats = np.zeros(7)
        self.L.lo_load_step_damage(self.h, nd, darr, nf, farr, newton_tol, maxiter, cg_rtol_sq,
                                   cg_atol_sq, max_passes, _dp(stats))
        return stats

    def load_step(self, disp_bcs, force_bcs, newton_tol, maxiter=100, cg_rtol_sq=1e-20,
                  cg_atol_sq=0.0):
        nd, darr, nf, farr = bc_arrays(disp_bcs, force_bcs)
        stats = np.zeros(5)
        self.L.lo_load_step(self.h, nd, darr, nf, farr, newton_tol, maxiter, cg_rtol_sq,
                            cg_atol_sq, _dp(stats))
        return stats
