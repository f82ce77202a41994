"""ctypes binding of the C host driver (liblpmhost.so): the reference's
load-step loop (src/lpmc_project.c:382-471) run in C through the
reference-named drop-in symbols of liblpmgpu_legacy.so, with all state in the
include/lpm.h globals on the host.  Used for the end-to-end (host buffers)
measurement and the drop-in parity tests."""
import ctypes as C
import os

import numpy as np

import lpm_gb300 as G

HERE = os.path.dirname(os.path.abspath(__file__))
HOST_LIB = os.path.join(HERE, "_build", "liblpmhost.so")


class HostDriver:
    def __init__(self):
        if not os.path.exists(HOST_LIB):
            raise G.LPMError(f"{HOST_LIB} not found: build first")
        self.L = C.CDLL(HOST_LIB, mode=C.RTLD_GLOBAL)
        dp = C.POINTER(C.c_double)
        self.L.lpmh_setup.argtypes = [C.c_int, C.c_double, dp, C.c_int]
        self.L.lpmh_set_types.argtypes = [C.POINTER(C.c_int), C.c_int]
        self.L.lpmh_set_bc_groups.argtypes = [C.POINTER(C.c_int), C.c_int]
        self.L.lpmh_set_material.argtypes = [dp, C.c_int, dp, C.c_double, C.c_double, dp]
        self.L.lpmh_load_step.argtypes = [C.c_int, C.POINTER(G.DispBC), C.c_int, C.POINTER(G.ForceBC),
                                          C.c_double, C.c_int, dp]
        self.L.lpmh_get.argtypes = [C.c_char_p, dp]
        self.L.lpmh_set_damage.argtypes = [C.c_double, C.c_double, C.c_double, C.c_double, C.c_int, C.c_char_p,
                                           C.c_int]
        self.L.lpm_legacy_set_solver.argtypes = [C.c_void_p]
        self.L.lpm_legacy_traffic.argtypes = [C.POINTER(C.c_longlong), C.POINTER(C.c_longlong), C.c_int]
        self.n = 0

    def setup(self, lattice, radius, box, nslip=0):
        box = np.ascontiguousarray(box, dtype=np.float64)
        self.n = self.L.lpmh_setup(lattice, radius, box.ctypes.data_as(C.POINTER(C.c_double)), nslip)
        if self.n <= 0:
            raise G.LPMError("host setup failed")
        return self.n

    def set_types(self, types, ntype):
        t = np.ascontiguousarray(types, dtype=np.int32)
        self.L.lpmh_set_types(t.ctypes.data_as(C.POINTER(C.c_int)), int(ntype))

    def set_bc_groups(self, groups, ngroup):
        """Boundary conditions select particles by these labels instead of
        their type (per-particle moduli: one type per particle)."""
        if groups is None:
            self.L.lpmh_set_bc_groups(None, 0)
            return
        g = np.ascontiguousarray(groups, dtype=np.int32)
        self.L.lpmh_set_bc_groups(g.ctypes.data_as(C.POINTER(C.c_int)), int(ngroup))

    def set_material(self, ce, plmode, sigmay, xi, H, cp=None):
        ce = np.ascontiguousarray(ce, dtype=np.float64).reshape(-1)
        sy = np.ascontiguousarray(np.broadcast_to(np.asarray(sigmay, dtype=np.float64), (self.n,)))
        cpa = None if cp is None else np.ascontiguousarray(cp, dtype=np.float64)
        dp = C.POINTER(C.c_double)
        self.L.lpmh_set_material(ce.ctypes.data_as(dp), int(plmode), sy.ctypes.data_as(dp), float(xi),
                                 float(H), None if cpa is None else cpa.ctypes.data_as(dp))

    def set_solver(self, **kw):
        o = G.default_opts()
        for k, v in kw.items():
            setattr(o, k, v)
        self._opts = o
        rc = self.L.lpm_legacy_set_solver(C.cast(C.byref(o), C.c_void_p))
        if rc < 0:
            raise G.LPMError("legacy solver options rejected")

    def set_damage(self, bondfile, length=0.5, threshold=0.9, triax_coeff=0.0, critical_bstrain=1e-2, nbreak=20,
                   max_passes=1000):
        """main's damage stage in every load step: updateDamageGeneral,
        updateCrack and the re-solves after broken bonds; broken bonds are
        appended to bondfile."""
        self.L.lpmh_set_damage(float(length), float(threshold), float(triax_coeff), float(critical_bstrain),
                               int(nbreak), os.fsencode(bondfile), int(max_passes))

    def init(self):
        self.L.lpmh_init()

    def load_step(self, disp_bcs, force_bcs=(), newton_tol=1e-8, maxiter=100):
        """Returns Newton iterations, |r0|, |reaction0|, |r|, 0, Newton
        passes, bonds broken (the last two with the damage stage on)."""
        nd, darr, nf, farr = G.bc_arrays(disp_bcs, list(force_bcs))
        st = np.zeros(7)
        self.L.lpmh_load_step(nd, darr, nf, farr, float(newton_tol), int(maxiter),
                              st.ctypes.data_as(C.POINTER(C.c_double)))
        return st

    def get(self, name):
        shape = {"xyz": (self.n, 3), "xyz_initial": (self.n, 3), "J2_alpha": (self.n,),
                 "F": (self.n, 18), "csz": (self.n, 18), "dL": (self.n, 18), "Kn": (self.n, 18),
                 "Tv": (self.n, 18), "damage_broken": (self.n, 18), "damage_w": (self.n, 18),
                 "damage_nonlocal": (self.n,), "nb": (self.n,),
                 "strain_tensor": (self.n, 6)}[name]
        out = np.zeros(shape)
        if self.L.lpmh_get(name.encode(), out.ctypes.data_as(C.POINTER(C.c_double))) != 0:
            raise KeyError(name)
        return out

    def compute_strain(self):
        """computeStrain through the reference-named drop-in."""
        self.L.computeStrain()
        return self.get("strain_tensor")

    def traffic(self, reset=False):
        a, b = C.c_longlong(), C.c_longlong()
        self.L.lpm_legacy_traffic(C.byref(a), C.byref(b), int(reset))
        return a.value, b.value
