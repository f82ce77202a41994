"""Python host binding of the GB300 LPM library (ctypes over include/lpm_gpu.h).

Mirrors the reference's operator boundary for the quasi-static solve path:
``Specimen.setup_lattice`` (createCuboid + neighbour search), ``set_material``
(calcKnTv), ``init_state`` (computedL / computeCab), ``load_step`` (one load
step of src/lpmc_project.c:385-471), and the single-function entry points
``assemble_stiffness`` / ``compute_force`` / ``solve`` / ``switch_state``.
Arrays come back in the reference's row-major [i][j] layout.

The library is loaded from lpm-c_gb300/_build/liblpmgpu.so (built by
build.py); there is no CPU fallback: if the shared object or a GPU is
missing, calls raise.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liblpmgpu.so")

PREC_FP64, PREC_MIXED = 0, 1
PRECOND_BJ, PRECOND_AMG = 0, 1
PL_J2, PL_CP, PL_PREDICTOR, PL_ELASTIC = 0, 1, 4, 6
STATUS_NEWTON_MAXIT, STATUS_CG_MAXIT, STATUS_NAN, STATUS_CP_SINGULAR = 1, 2, 4, 8

# every symbol declared in include/lpm_gpu.h
EXPORTED = [
    "lpm_create", "lpm_destroy", "lpm_last_error", "lpm_set_stream", "lpm_default_solver_opts",
    "lpm_set_solver", "lpm_setup_lattice", "lpm_setup_particles", "lpm_nparticle", "lpm_set_types",
    "lpm_set_material", "lpm_set_cp", "lpm_init_state", "lpm_load_step", "lpm_assemble_stiffness",
    "lpm_apply_bc", "lpm_compute_force", "lpm_switch_state", "lpm_solve", "lpm_begin_step", "lpm_get",
    "lpm_set", "lpm_get_sizes", "lpm_export_upper_csr", "lpm_spmv", "lpm_solve_rhs", "lpm_spmv_timing",
    "lpm_spmv_bytes", "lpm_update_rr_noalloc", "lpm_setup_batch", "lpm_batch_offsets",
    "lpm_batch_load_step", "lpm_autotune", "lpm_set_tuning", "lpm_get_tuning",
    "lpm_default_adjoint_opts", "lpm_adjoint_forward", "lpm_adjoint_backward", "lpm_force_vjp",
    "lpm_write_dump", "lpm_write_wait", "lpm_write_disp", "lpm_write_reaction", "lpm_write_stress",
    "lpm_format_dump", "lpm_format_disp", "lpm_format_reaction", "lpm_format_stress",
    "lpm_compute_strain", "lpm_write_strain", "lpm_format_strain",
    "lpm_default_damage_opts", "lpm_set_damage", "lpm_damage_log", "lpm_damage_brittle_select",
    "lpm_damage_update", "lpm_damage_crack",
]


class DispBC(C.Structure):
    """lpm_disp_bc == struct dispBCPara (include/lpm.h:83-88)."""
    _fields_ = [("type", C.c_int), ("flag", C.c_char), ("step", C.c_double)]


class ForceBC(C.Structure):
    """lpm_force_bc == struct forceBCPara (include/lpm.h:90-99)."""
    _fields_ = [("type", C.c_int), ("flag1", C.c_char), ("step1", C.c_double),
                ("flag2", C.c_char), ("step2", C.c_double), ("flag3", C.c_char), ("step3", C.c_double)]


class SolverOpts(C.Structure):
    _fields_ = [("precision", C.c_int), ("newton_tol", C.c_double), ("newton_maxiter", C.c_int),
                ("cg_rtol", C.c_double), ("cg_maxiter", C.c_int), ("inner_rtol", C.c_double),
                ("refine_maxiter", C.c_int), ("check_every", C.c_int), ("use_graphs", C.c_int),
                ("mixed_vectors", C.c_int), ("newton_accel", C.c_int), ("cg_forcing", C.c_double),
                ("preconditioner", C.c_int), ("amg_spacing", C.c_double), ("amg_rebuild", C.c_double),
                ("amg_sweeps", C.c_int), ("recycle", C.c_int)]


class Tuning(C.Structure):
    """lpm_tuning: launch shapes of the solve (include/lpm_gpu.h)."""
    _fields_ = [("spmv_variant", C.c_int), ("spmv_lanes", C.c_int), ("spmv_blocks", C.c_int),
                ("spmv_per_sm", C.c_int), ("cg_per_sm", C.c_int), ("spmv_ms", C.c_double),
                ("spmv_ms_default", C.c_double), ("smooth_lanes", C.c_int), ("smooth_ms", C.c_double),
                ("diff_stream", C.c_int), ("smooth_stream", C.c_int)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class AdjointOpts(C.Structure):
    _fields_ = [("checkpoint_every", C.c_int), ("gmres_restart", C.c_int), ("gmres_maxiter", C.c_int),
                ("gmres_rtol", C.c_double)]


class AdjointStats(C.Structure):
    _fields_ = [("steps", C.c_int), ("recomputed_steps", C.c_int), ("checkpoints", C.c_int),
                ("gmres_iters", C.c_int), ("cg_iters", C.c_int), ("cg_iters_backward", C.c_int),
                ("status", C.c_int), ("ms_forward", C.c_double), ("ms_backward", C.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class StepStats(C.Structure):
    _fields_ = [("newton_iters", C.c_int), ("cg_iters", C.c_int), ("refine_iters", C.c_int),
                ("spmv_calls", C.c_int), ("status", C.c_int), ("res0", C.c_double),
                ("reac0", C.c_double), ("res_final", C.c_double), ("ms_stiffness", C.c_double),
                ("ms_solve", C.c_double), ("ms_force", C.c_double), ("damage_passes", C.c_int),
                ("bonds_broken", C.c_int), ("amg_builds", C.c_int), ("ms_amg_build", C.c_double),
                ("fp64_fallbacks", C.c_int)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class DamageOpts(C.Structure):
    """lpm_damage_opts: the reference main's damage stage (include/lpm_gpu.h)."""
    _fields_ = [("enabled", C.c_int), ("length", C.c_double), ("threshold", C.c_double),
                ("triax_coeff", C.c_double), ("critical_bstrain", C.c_double), ("nbreak", C.c_int),
                ("max_passes", C.c_int)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class LPMError(RuntimeError):
    pass


_lib = None


def load(path=LIB_PATH):
    """Load the CUDA library (raises if it was not built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise LPMError(f"{path} not found: build the CUDA library first (lpm-c_gb300/build.py)")
    L = C.CDLL(path)
    vp, dp, ip = C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_int)
    sig = {
        "lpm_create": ([C.POINTER(vp), C.c_int], C.c_int),
        "lpm_destroy": ([vp], None),
        "lpm_last_error": ([], C.c_char_p),
        "lpm_set_stream": ([vp, vp], C.c_int),
        "lpm_default_solver_opts": ([C.POINTER(SolverOpts)], None),
        "lpm_set_solver": ([vp, C.POINTER(SolverOpts)], C.c_int),
        "lpm_setup_lattice": ([vp, C.c_int, C.c_double, dp], C.c_int),
        "lpm_setup_particles": ([vp, C.c_int, C.c_double, C.c_int, dp], C.c_int),
        "lpm_nparticle": ([vp], C.c_int),
        "lpm_set_types": ([vp, ip], C.c_int),
        "lpm_set_material": ([vp, dp, dp, dp, dp, dp, C.c_double, C.c_int], C.c_int),
        "lpm_set_cp": ([vp, dp], C.c_int),
        "lpm_init_state": ([vp], C.c_int),
        "lpm_load_step": ([vp, C.c_int, C.POINTER(DispBC), C.c_int, C.POINTER(ForceBC),
                           C.POINTER(StepStats)], C.c_int),
        "lpm_assemble_stiffness": ([vp], C.c_int),
        "lpm_apply_bc": ([vp, C.c_int, C.POINTER(DispBC), C.c_int, C.POINTER(ForceBC)], C.c_int),
        "lpm_compute_force": ([vp, C.c_int, dp], C.c_int),
        "lpm_switch_state": ([vp, C.c_int], C.c_int),
        "lpm_solve": ([vp, C.POINTER(StepStats)], C.c_int),
        "lpm_begin_step": ([vp], C.c_int),
        "lpm_get": ([vp, C.c_char_p, vp, C.c_size_t], C.c_int),
        "lpm_set": ([vp, C.c_char_p, vp, C.c_size_t], C.c_int),
        "lpm_get_sizes": ([vp, ip, ip, ip, C.POINTER(C.c_longlong)], C.c_int),
        "lpm_export_upper_csr": ([vp, dp, ip, ip, C.POINTER(C.c_longlong)], C.c_int),
        "lpm_spmv": ([vp, dp, dp], C.c_int),
        "lpm_solve_rhs": ([vp, dp, dp, C.POINTER(StepStats)], C.c_int),
        "lpm_spmv_timing": ([vp, dp, C.POINTER(C.c_longlong), C.c_int], C.c_int),
        "lpm_spmv_bytes": ([vp, C.c_int], C.c_double),
        "lpm_update_rr_noalloc": ([C.c_int, vp, vp, vp, vp, dp, vp], C.c_int),
        "lpm_setup_batch": ([vp, C.c_int, C.c_double, C.c_int, dp], C.c_int),
        "lpm_batch_offsets": ([vp, ip], C.c_int),
        "lpm_batch_load_step": ([vp, C.c_int, C.POINTER(DispBC), C.POINTER(StepStats)], C.c_int),
        "lpm_autotune": ([vp, C.POINTER(Tuning)], C.c_int),
        "lpm_set_tuning": ([vp, C.POINTER(Tuning)], C.c_int),
        "lpm_get_tuning": ([vp, C.POINTER(Tuning)], C.c_int),
        "lpm_default_adjoint_opts": ([C.POINTER(AdjointOpts)], None),
        "lpm_adjoint_forward": ([vp, dp, dp, dp, dp, C.c_int, C.c_int, C.POINTER(DispBC), C.c_int, C.c_int,
                                 C.POINTER(AdjointOpts), dp], C.c_int),
        "lpm_adjoint_backward": ([vp, dp, dp, dp, dp, dp, C.POINTER(AdjointStats)], C.c_int),
        "lpm_force_vjp": ([vp, dp, dp, dp, dp, dp, dp, dp], C.c_int),
        "lpm_write_dump": ([vp, C.c_char_p, C.c_int, C.c_char, dp], C.c_int),
        "lpm_write_wait": ([vp], C.c_int),
        "lpm_write_disp": ([vp, C.c_char_p, C.c_char, C.c_int, C.c_int], C.c_int),
        "lpm_write_reaction": ([vp, C.c_char_p, C.c_char, C.c_int, C.c_int], C.c_int),
        "lpm_write_stress": ([vp, C.c_char_p, C.c_int, C.c_int], C.c_int),
        "lpm_format_dump": ([C.c_char_p, C.c_int, C.c_char, C.c_int, dp, C.c_int, ip, dp, dp, dp, dp, ip, dp,
                             C.c_int, dp], C.c_int),
        "lpm_format_disp": ([C.c_char_p, C.c_char, C.c_int, C.c_int, C.c_int, ip, dp, dp], C.c_int),
        "lpm_format_reaction": ([C.c_char_p, C.c_char, C.c_int, C.c_int, C.c_int, C.c_int, ip, ip, dp, dp, dp, dp],
                                C.c_int),
        "lpm_format_stress": ([C.c_char_p, C.c_int, C.c_int, C.c_int, ip, dp], C.c_int),
        "lpm_compute_strain": ([vp], C.c_int),
        "lpm_write_strain": ([vp, C.c_char_p, C.c_int, C.c_int], C.c_int),
        "lpm_format_strain": ([C.c_char_p, C.c_int, C.c_int, C.c_int, ip, dp], C.c_int),
        "lpm_default_damage_opts": ([C.POINTER(DamageOpts)], None),
        "lpm_set_damage": ([vp, C.POINTER(DamageOpts)], C.c_int),
        "lpm_damage_log": ([vp, ip, C.c_int, ip], C.c_int),
        "lpm_damage_update": ([vp, ip], C.c_int),
        "lpm_damage_crack": ([vp], C.c_int),
        "lpm_damage_brittle_select": ([ip, dp, C.c_int, C.c_int, C.c_int, ip, ip], C.c_int),
    }
    for name, (args, res) in sig.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = res
    _lib = L
    return L


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _ip(a):
    return a.ctypes.data_as(C.POINTER(C.c_int))


def bc_arrays(disp_bcs, force_bcs):
    nd, nf = len(disp_bcs), len(force_bcs)
    darr = (DispBC * max(nd, 1))()
    for k, (t, f, s) in enumerate(disp_bcs):
        darr[k] = DispBC(int(t), f.encode(), float(s))
    farr = (ForceBC * max(nf, 1))()
    for k, (t, fx, fy, fz) in enumerate(force_bcs):
        farr[k] = ForceBC(int(t), b"x", float(fx), b"y", float(fy), b"z", float(fz))
    return nd, darr, nf, farr


def default_opts():
    o = SolverOpts()
    load().lpm_default_solver_opts(C.byref(o))
    return o


def brittle_select(bonds, strain, n, nbreak):
    """lpm_damage_brittle_select: the brittle pass's choice among candidate
    bonds (b = slot * n + particle, any order); host logic, no GPU needed."""
    L = load()
    b = np.ascontiguousarray(bonds, dtype=np.int32)
    v = np.ascontiguousarray(strain, dtype=np.float64)
    out = np.zeros(max(len(b), 1), dtype=np.int32)
    k = C.c_int()
    if L.lpm_damage_brittle_select(_ip(b), _dp(v), len(b), int(n), int(nbreak), _ip(out), C.byref(k)) != 0:
        raise LPMError(L.lpm_last_error().decode())
    return out[:k.value]


class Specimen:
    """One lattice specimen resident on one GPU (an lpm_ctx)."""

    def __init__(self, device=0):
        self.L = load()
        h = C.c_void_p()
        self._check(self.L.lpm_create(C.byref(h), device))
        self.h = h
        self.n = 0
        self.nn = 18
        self.nslip = 0

    def close(self):
        if getattr(self, "h", None):
            self.L.lpm_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def _check(self, rc):
        if rc < 0:
            raise LPMError(self.L.lpm_last_error().decode() or f"error {rc}")
        return rc

    # ---- setup
    def setup_lattice(self, lattice, radius, box):
        box = np.ascontiguousarray(box, dtype=np.float64)
        self.n = self._check(self.L.lpm_setup_lattice(self.h, lattice, radius, _dp(box)))
        return self.n

    def setup_batch(self, lattice, radius, boxes):
        """Concatenate len(boxes) specimens (lpm_setup_batch); returns the
        total particle count."""
        boxes = np.ascontiguousarray(boxes, dtype=np.float64).reshape(-1, 6)
        self.n = self._check(self.L.lpm_setup_batch(self.h, lattice, radius, len(boxes), _dp(boxes)))
        return self.n

    def batch_offsets(self):
        ns = self._check(self.L.lpm_batch_offsets(self.h, None))
        off = np.zeros(ns + 1, dtype=np.int32)
        self._check(self.L.lpm_batch_offsets(self.h, _ip(off)))
        return off

    def batch_load_step(self, disp_bcs):
        """disp_bcs: one list of (type, flag, step) per specimen, all of the
        same length.  Returns one statistics dict per specimen."""
        ns = len(disp_bcs)
        nbd = len(disp_bcs[0]) if ns else 0
        if any(len(b) != nbd for b in disp_bcs):
            raise LPMError("every specimen needs the same number of displacement BCs")
        arr = (DispBC * max(1, ns * nbd))()
        for s, bl in enumerate(disp_bcs):
            for k, (t, f, v) in enumerate(bl):
                arr[s * nbd + k] = DispBC(int(t), f.encode() if isinstance(f, str) else f, float(v))
        st = (StepStats * ns)()
        self._check(self.L.lpm_batch_load_step(self.h, nbd, arr, st))
        return [x.as_dict() for x in st]

    def autotune(self):
        t = Tuning()
        self._check(self.L.lpm_autotune(self.h, C.byref(t)))
        return t.as_dict()

    def set_tuning(self, spmv_variant=0, spmv_per_sm=8, cg_per_sm=8, diff_stream=0, smooth_stream=0):
        t = Tuning(spmv_variant=spmv_variant, spmv_per_sm=spmv_per_sm, cg_per_sm=cg_per_sm,
                   diff_stream=diff_stream, smooth_stream=smooth_stream)
        self._check(self.L.lpm_set_tuning(self.h, C.byref(t)))

    def get_tuning(self):
        t = Tuning()
        self._check(self.L.lpm_get_tuning(self.h, C.byref(t)))
        return t.as_dict()

    def adjoint_forward(self, E, nu, sigmay, H, step_bcs, rtype, rcomp, **opts):
        """Run the load steps (one BC list per step) and return the reaction
        curve; opts: checkpoint_every, gmres_restart, gmres_maxiter, gmres_rtol."""
        o = AdjointOpts()
        self.L.lpm_default_adjoint_opts(C.byref(o))
        for k, v in opts.items():
            setattr(o, k, v)
        nsteps = len(step_bcs)
        nbd = len(step_bcs[0]) if nsteps else 0
        arr = (DispBC * max(1, nsteps * nbd))()
        for s, bl in enumerate(step_bcs):
            for k, (t, f, v) in enumerate(bl):
                arr[s * nbd + k] = DispBC(int(t), f.encode() if isinstance(f, str) else f, float(v))
        vals = [np.ascontiguousarray(np.broadcast_to(np.asarray(x, dtype=np.float64), (self.n,)))
                for x in (E, nu, sigmay, H)]
        R = np.zeros(nsteps)
        comp = {"x": 0, "y": 1, "z": 2}.get(rcomp, rcomp)
        self._check(self.L.lpm_adjoint_forward(self.h, *[_dp(v) for v in vals], nsteps, nbd, arr, int(rtype),
                                               int(comp), C.byref(o), _dp(R)))
        return R

    def adjoint_backward(self, dLdR):
        dLdR = np.ascontiguousarray(dLdR, dtype=np.float64)
        out = [np.zeros(self.n) for _ in range(4)]
        st = AdjointStats()
        self._check(self.L.lpm_adjoint_backward(self.h, _dp(dLdR), *[_dp(o) for o in out], C.byref(st)))
        return dict(E=out[0], nu=out[1], sigmay=out[2], H=out[3]), st.as_dict()

    def force_vjp(self, Pbar, mu_dLp=None, mu_alpha=None):
        Pbar = np.ascontiguousarray(Pbar, dtype=np.float64).reshape(-1)
        mud = None if mu_dLp is None else _dp(np.ascontiguousarray(mu_dLp, dtype=np.float64))
        mua = None if mu_alpha is None else _dp(np.ascontiguousarray(mu_alpha, dtype=np.float64))
        xbar = np.zeros((self.n, 3))
        dlp = np.zeros((self.n, self.nn))
        ab = np.zeros(self.n)
        th = np.zeros((5, self.n))
        self._check(self.L.lpm_force_vjp(self.h, _dp(Pbar), mud, mua, _dp(xbar), _dp(dlp), _dp(ab), _dp(th)))
        return xbar, dlp, ab, th

    # ---- output in the reference's formats
    def write_dump(self, path, step, flag, box):
        self._check(self.L.lpm_write_dump(self.h, path.encode(), int(step), flag.encode(),
                                          _dp(np.ascontiguousarray(box, dtype=np.float64))))

    def write_wait(self):
        self._check(self.L.lpm_write_wait(self.h))

    def write_disp(self, path, c, t1, tstep):
        self._check(self.L.lpm_write_disp(self.h, path.encode(), c.encode(), int(t1), int(tstep)))

    def write_reaction(self, path, c, t1, tstep):
        self._check(self.L.lpm_write_reaction(self.h, path.encode(), c.encode(), int(t1), int(tstep)))

    def compute_strain(self):
        self._check(self.L.lpm_compute_strain(self.h))
        return self.get("strain_tensor")

    def write_strain(self, path, t1, tstep):
        self._check(self.L.lpm_write_strain(self.h, path.encode(), int(t1), int(tstep)))

    def write_stress(self, path, t1, tstep):
        self._check(self.L.lpm_write_stress(self.h, path.encode(), int(t1), int(tstep)))

    def setup_particles(self, lattice, radius, xyz):
        xyz = np.ascontiguousarray(xyz, dtype=np.float64)
        self.n = self._check(self.L.lpm_setup_particles(self.h, lattice, radius, xyz.shape[0], _dp(xyz)))
        return self.n

    def set_types(self, types):
        t = np.ascontiguousarray(types, dtype=np.int32)
        self._check(self.L.lpm_set_types(self.h, _ip(t)))

    def set_material(self, c11, c12, c44, sigmay=0.0, hardening=0.0, xi=0.0, plmode=PL_J2):
        arrs = [np.ascontiguousarray(np.broadcast_to(np.asarray(v, dtype=np.float64), (self.n,)))
                for v in (c11, c12, c44, sigmay, hardening)]
        self._check(self.L.lpm_set_material(self.h, *[_dp(a) for a in arrs], float(xi), int(plmode)))

    def set_cp(self, tau0, taus, h0, p, q, eta, maxloop, dtime):
        cp = np.array([tau0, taus, h0, p, q, eta, maxloop, dtime], dtype=np.float64)
        self._check(self.L.lpm_set_cp(self.h, _dp(cp)))

    def init_state(self):
        self._check(self.L.lpm_init_state(self.h))
        n, nn, ns = C.c_int(), C.c_int(), C.c_int()
        self._check(self.L.lpm_get_sizes(self.h, C.byref(n), C.byref(nn), C.byref(ns), None))
        self.nslip = ns.value

    def set_solver(self, **kw):
        o = default_opts()
        for k, v in kw.items():
            if not hasattr(o, k):
                raise KeyError(k)
            setattr(o, k, v)
        self._check(self.L.lpm_set_solver(self.h, C.byref(o)))
        return o

    def set_stream(self, stream_ptr):
        self._check(self.L.lpm_set_stream(self.h, C.c_void_p(stream_ptr)))

    # ---- hot path
    def load_step(self, disp_bcs, force_bcs=()):
        nd, darr, nf, farr = bc_arrays(disp_bcs, list(force_bcs))
        st = StepStats()
        self._check(self.L.lpm_load_step(self.h, nd, darr, nf, farr, C.byref(st)))
        return st.as_dict()

    def begin_step(self):
        self._check(self.L.lpm_begin_step(self.h))

    def assemble_stiffness(self):
        self._check(self.L.lpm_assemble_stiffness(self.h))

    def apply_bc(self, disp_bcs, force_bcs=()):
        nd, darr, nf, farr = bc_arrays(disp_bcs, list(force_bcs))
        self._check(self.L.lpm_apply_bc(self.h, nd, darr, nf, farr))

    def compute_force(self, plmode):
        norms = np.zeros(2)
        self._check(self.L.lpm_compute_force(self.h, plmode, _dp(norms)))
        return norms

    def switch_state(self, flag):
        self._check(self.L.lpm_switch_state(self.h, flag))

    def solve(self):
        st = StepStats()
        self._check(self.L.lpm_solve(self.h, C.byref(st)))
        return st.as_dict()

    def solve_rhs(self, b):
        b = np.ascontiguousarray(b, dtype=np.float64).reshape(-1)
        x = np.zeros_like(b)
        st = StepStats()
        self._check(self.L.lpm_solve_rhs(self.h, _dp(b), _dp(x), C.byref(st)))
        return x, st.as_dict()

    def spmv(self, x):
        x = np.ascontiguousarray(x, dtype=np.float64).reshape(-1)
        y = np.zeros_like(x)
        self._check(self.L.lpm_spmv(self.h, _dp(x), _dp(y)))
        return y

    # ---- data
    _SHAPES = {
        "xyz": ("p3", np.float64), "xyz_initial": ("p3", np.float64), "xyz_temp": ("p3", np.float64),
        "Pin": ("p3", np.float64), "Pex": ("p3", np.float64), "residual": ("p3", np.float64),
        "disp": ("p3", np.float64), "F": ("b", np.float64), "F_temp": ("b", np.float64),
        "dL": ("b", np.float64), "csx": ("b", np.float64), "csy": ("b", np.float64),
        "csz": ("b", np.float64), "Kn": ("b", np.float64), "Tv": ("b", np.float64),
        "distance_initial": ("b", np.float64), "dLp": ("b", np.float64), "dLp0": ("b", np.float64),
        "dLp2": ("b", np.float64), "J2_alpha": ("n1", np.float64), "J2_alpha0": ("n1", np.float64),
        "J2_alpha2": ("n1", np.float64), "J2_beta": ("n6", np.float64), "J2_beta2": ("n6", np.float64),
        "J2_dlambda": ("n1", np.float64), "stress_tensor": ("n6", np.float64),
        "strain_tensor": ("n6", np.float64),
        "neighbors": ("b", np.int32), "nsign": ("b", np.int32), "nb": ("n1", np.int32),
        "nb_conn": ("n1", np.int32), "conn": ("n61", np.int32), "K_pointer": ("kp", np.int32),
        "dispBC_index": ("p3", np.int32), "cs_initial": ("b3", np.float64),
        "type": ("n1", np.int32), "pl_flag": ("n1", np.int32),
        "cp_gy": ("ns", np.float64), "cp_gy2": ("ns", np.float64), "cp_A_single": ("ns", np.float64),
        "cp_A_single2": ("ns", np.float64), "cp_A": ("n1", np.float64), "cp_A2": ("n1", np.float64),
        "cp_Cab": ("nss", np.float64),
        "damage_broken": ("b", np.float64), "damage_w": ("b", np.float64), "damage_D": ("b", np.float64),
        "damage_nonlocal": ("n1", np.float64), "damage_visual": ("n1", np.float64),
        "nb_current": ("n1", np.int32),
    }

    def _shape(self, kind):
        n, nn, ns = self.n, self.nn, self.nslip
        return {"p3": (n, 3), "b": (n, nn), "n1": (n,), "n6": (n, 6), "n61": (n, 61), "kp": (n + 1, 2),
                "b3": (n, nn, 3), "ns": (n, ns), "nss": (n, ns * ns)}[kind]

    def get(self, name):
        kind, dt = self._SHAPES[name]
        out = np.zeros(self._shape(kind), dtype=dt)
        self._check(self.L.lpm_get(self.h, name.encode(), out.ctypes.data_as(C.c_void_p), out.nbytes))
        return out

    def set(self, name, arr):
        alias = {"dLp1": "dLp", "J2_alpha1": "J2_alpha", "J2_beta0": "J2_beta2", "J2_beta1": "J2_beta"}
        kind, dt = self._SHAPES.get(name, self._SHAPES.get(alias.get(name, ""), ("b", np.float64)))
        a = np.ascontiguousarray(arr, dtype=dt)
        self._check(self.L.lpm_set(self.h, name.encode(), a.ctypes.data_as(C.c_void_p), a.nbytes))

    # ---- damage stage (updateDamageGeneral, updateCrack, re-solve)
    def set_damage(self, enabled=True, **kw):
        """Switch the reference main's damage stage on (keyword overrides of
        lpm_default_damage_opts: length, threshold, triax_coeff,
        critical_bstrain, nbreak, max_passes) or off (enabled=False)."""
        o = DamageOpts()
        self.L.lpm_default_damage_opts(C.byref(o))
        o.enabled = 1 if enabled else 0
        for k, v in kw.items():
            if not hasattr(o, k):
                raise KeyError(k)
            setattr(o, k, v)
        self._check(self.L.lpm_set_damage(self.h, C.byref(o)))

    def damage_log(self):
        """Broken bonds so far as (particle, partner) rows, in the reference's order."""
        k = C.c_int()
        self._check(self.L.lpm_damage_log(self.h, None, 0, C.byref(k)))
        out = np.zeros((k.value, 2), dtype=np.int32)
        if k.value:
            self._check(self.L.lpm_damage_log(self.h, _ip(out), k.value, C.byref(k)))
        return out

    def export_upper_csr(self):
        nnz = C.c_longlong()
        self._check(self.L.lpm_export_upper_csr(self.h, None, None, None, C.byref(nnz)))
        K = np.zeros(nnz.value)
        IK = np.zeros(3 * self.n + 1, dtype=np.int32)
        JK = np.zeros(nnz.value, dtype=np.int32)
        self._check(self.L.lpm_export_upper_csr(self.h, _dp(K), _ip(IK), _ip(JK), C.byref(nnz)))
        return K, IK, JK

    def sizes(self):
        n, nn, ns, nb = C.c_int(), C.c_int(), C.c_int(), C.c_longlong()
        self._check(self.L.lpm_get_sizes(self.h, C.byref(n), C.byref(nn), C.byref(ns), C.byref(nb)))
        return dict(n=n.value, nn=nn.value, nslip=ns.value, nnz_blocks=nb.value)

    def spmv_timing(self, reset=0):
        ms, cnt = C.c_double(), C.c_longlong()
        self._check(self.L.lpm_spmv_timing(self.h, C.byref(ms), C.byref(cnt), int(reset)))
        return ms.value, cnt.value

    def spmv_bytes(self, precision):
        return self.L.lpm_spmv_bytes(self.h, int(precision))
