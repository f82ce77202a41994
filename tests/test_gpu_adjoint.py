"""Adjoint of the J2 load path against central finite differences.

1. lpm_force_vjp (reverse of one force evaluation) against central
   differences of the same evaluation, for every kind of input: positions,
   converged plastic stretch and hardening variable, C11/C12/C44, yield
   stress and hardening modulus.
2. lpm_adjoint_forward/backward on a small notched plate: directional
   derivatives of the reaction-misfit loss along smooth random perturbations
   of each field, and single (particle, field) pairs.
3. Checkpointed recomputation gives the same gradient as storing every step.
"""
import numpy as np
import pytest

import cases

pytestmark = pytest.mark.gpu

# finite differences of the loss need the forward converged to 1e-12;
# plain modified Newton needs hundreds of iterations per plastic step for
# that, the Anderson-accelerated loop tens
TIGHT = dict(newton_tol=1e-12, newton_maxiter=3000, cg_rtol=1e-13, cg_maxiter=100000, newton_accel=8)


def plate_specimen(G, plate, precision=0):
    s = G.Specimen(0)
    s.setup_particles(plate.lattice, plate.radius, plate.xyz)
    types = cases.sc_types(s.get("xyz"), s.get("nb"), plate.radius)
    s.set_types(types)
    s.set_solver(precision=precision, **TIGHT)
    return s


def plastic_state(G):
    """The point where the adjoint differentiates a force evaluation: the
    configuration after load step n with the converged state of step n - 1
    (here n = 3, deep enough into the plastic range that every particle
    yields, so the return map is smooth around it)."""
    case = cases.SCCase(n=6, sigmay=120.0)
    s = G.Specimen(0)
    n = s.setup_lattice(case.lattice, case.radius, case.box)
    types = cases.sc_types(s.get("xyz"), s.get("nb"), case.radius)
    s.set_types(types)
    c11, c12, c44 = cases.iso_cubic(case.E, case.nu)
    rng = np.random.default_rng(1)
    mat = [np.full(n, c11) * (1 + 0.05 * rng.uniform(-1, 1, n)), np.full(n, c12), np.full(n, c44),
           np.full(n, case.sigmay) * (1 + 0.1 * rng.uniform(-1, 1, n)), np.full(n, case.H)]
    s.set_material(*mat, 0.0, G.PL_J2)
    s.init_state()
    s.set_solver(precision=0, **TIGHT)
    for stp in [3 * case.schedule[0]] * 2:
        s.load_step(cases.sc_bcs(stp))
    dlp, al = s.get("dLp"), s.get("J2_alpha")
    s.load_step(cases.sc_bcs(3 * case.schedule[0]))
    s.set("dLp", dlp)
    s.set("J2_alpha", al)
    s.switch_state(0)
    return s, mat


def test_force_vjp_matches_central_differences(gpu_lib):
    G = gpu_lib
    s, mat = plastic_state(G)
    n, nn = s.n, s.nn
    assert s.get("J2_alpha").max() > 0.0  # some particles have yielded
    rng = np.random.default_rng(2)
    Pbar = rng.standard_normal((n, 3))
    mu_d = rng.standard_normal((n, nn)) * (s.get("neighbors") >= 0)
    mu_a = rng.standard_normal(n)
    x0 = s.get("xyz")
    dLp0, al0 = s.get("dLp"), s.get("J2_alpha")
    s.compute_force(G.PL_J2)
    xbar, dlpb, alb, th = s.force_vjp(Pbar, mu_d, mu_a)

    def objective():
        s.switch_state(0)
        s.compute_force(G.PL_J2)
        return float((Pbar * s.get("Pin")).sum() + (mu_d * s.get("dLp2")).sum() + (mu_a * s.get("J2_alpha2")).sum())

    def central(apply, h):
        """Richardson-extrapolated central difference (error O(h^4))."""
        def cd(hh):
            apply(hh)
            fp = objective()
            apply(-hh)
            fm = objective()
            apply(0.0)
            return (fp - fm) / (2 * hh)
        return (4.0 * cd(h) - cd(2.0 * h)) / 3.0

    # positions
    d = rng.standard_normal((n, 3))
    fd = central(lambda h: s.set("xyz", x0 + h * d), 1e-7)
    ad = float((xbar * d).sum())
    assert abs(fd - ad) <= 1e-6 * max(abs(ad), 1e-30), ("xyz", fd, ad)
    # converged plastic stretch and hardening variable
    dd = rng.standard_normal((n, nn)) * (s.get("neighbors") >= 0)
    fd = central(lambda h: s.set("dLp", dLp0 + h * dd), 1e-9)
    ad = float((dlpb * dd).sum())
    assert abs(fd - ad) <= 1e-6 * max(abs(ad), 1e-30), ("dLp", fd, ad)
    da = rng.uniform(0, 1, n)
    fd = central(lambda h: s.set("J2_alpha", al0 + h * da), 1e-9)
    ad = float((alb * da).sum())
    assert abs(fd - ad) <= 1e-6 * max(abs(ad), 1e-30), ("alpha", fd, ad)
    # material: C11, C12, C44, yield stress, hardening
    for k in range(5):
        dm = rng.uniform(0.5, 1.5, n) * mat[k]
        rel = 1e-7

        def setm(h, k=k, dm=dm):
            m = [x.copy() for x in mat]
            m[k] = mat[k] + h * dm
            s.set_material(*m, 0.0, G.PL_J2)

        fd = central(setm, rel)
        ad = float((th[k] * dm).sum())
        assert abs(fd - ad) <= 1e-6 * max(abs(ad), 1e-30), ("material", k, fd, ad)
    s.close()


def small_plate():
    return cases.NotchedPlate(nx=10, ny=2, nz=12, notch=4, steps=6, strain=0.006, corr=3.0)


def loss_and_grad(G, plate, fields, target, every=10):
    s = plate_specimen(G, plate)
    R = s.adjoint_forward(*fields, plate.step_bcs(), cases.T_TOP, "z", checkpoint_every=every)
    L = float(((R - target) ** 2).sum())
    grads, st = s.adjoint_backward(2.0 * (R - target))
    alpha = s.get("J2_alpha")
    s.close()
    return L, grads, st, alpha


def loss_only(G, plate, fields, target):
    s = plate_specimen(G, plate)
    R = s.adjoint_forward(*fields, plate.step_bcs(), cases.T_TOP, "z")
    alpha = s.get("J2_alpha")
    s.close()
    return float(((R - target) ** 2).sum()), alpha


def test_adjoint_gradient_matches_finite_differences(gpu_lib):
    G = gpu_lib
    plate = small_plate()
    f1, f2 = plate.fields(1), plate.fields(2)
    s = plate_specimen(G, plate)
    target = s.adjoint_forward(*f2, plate.step_bcs(), cases.T_TOP, "z")
    s.close()
    L, grads, st, alpha = loss_and_grad(G, plate, f1, target)
    assert L > 0.0 and alpha.max() > 0.0, (L, alpha.max())
    assert st["status"] == 0, st
    names = ["E", "nu", "sigmay", "H"]
    rng = np.random.default_rng(4)
    # directional derivatives along smooth fields (active sets unchanged for h = 1e-5)
    for k, name in enumerate(names):
        d = f1[k] * plate.fields(7 + k)[k] / plate.BASE[k]
        h = 1e-5
        fp = [x.copy() for x in f1]
        fm = [x.copy() for x in f1]
        fp[k] = f1[k] + h * d
        fm[k] = f1[k] - h * d
        Lp, ap = loss_only(G, plate, fp, target)
        Lm, am = loss_only(G, plate, fm, target)
        assert np.array_equal(ap > 0, am > 0) and np.array_equal(ap > 0, alpha > 0), name
        fd = (Lp - Lm) / (2 * h)
        ad = float((grads[name] * d).sum())
        assert abs(fd - ad) <= 1e-6 * abs(ad), (name, fd, ad)
    # single (particle, field) pairs, central h = 1e-4 relative
    for t in range(4):
        k = t % 4
        i = int(rng.integers(plate.n))
        h = 1e-4 * f1[k][i]
        fp = [x.copy() for x in f1]
        fm = [x.copy() for x in f1]
        fp[k][i] += h
        fm[k][i] -= h
        Lp, ap = loss_only(G, plate, fp, target)
        Lm, am = loss_only(G, plate, fm, target)
        if not (np.array_equal(ap > 0, am > 0) and np.array_equal(ap > 0, alpha > 0)):
            continue  # the perturbation moved the active set
        fd = (Lp - Lm) / (2 * h)
        ad = float(grads[names[k]][i])
        assert abs(fd - ad) <= 1e-4 * max(abs(ad), 1e-3 * np.abs(grads[names[k]]).max()), (names[k], i, fd, ad)


def test_checkpointed_recomputation_is_exact(gpu_lib):
    G = gpu_lib
    plate = small_plate()
    f1, f2 = plate.fields(1), plate.fields(2)
    s = plate_specimen(G, plate)
    target = s.adjoint_forward(*f2, plate.step_bcs(), cases.T_TOP, "z")
    s.close()
    _, g_all, st_all, _ = loss_and_grad(G, plate, f1, target, every=100)
    _, g_ck, st_ck, _ = loss_and_grad(G, plate, f1, target, every=2)
    assert st_ck["checkpoints"] == 3 and st_ck["recomputed_steps"] == plate.steps
    for name in g_all:
        assert np.array_equal(g_all[name], g_ck[name]), name


def test_adjoint_matches_cpu_reference_gradient(oracle_mod, gpu_lib):
    """The GPU adjoint gradient against a reference gradient from the FP64 CPU
    path: central differences of the loss computed by the oracle (the C
    restatement of the reference, bit-exact with it), along a smooth direction
    of each field."""
    G = gpu_lib
    # two steps into the plastic range (74 of 154 particles yield): the
    # reference's plain modified Newton, run by the oracle, converges there
    # to 1e-12 (it diverges on the third step of this plate)
    plate = cases.NotchedPlate(nx=8, ny=2, nz=10, notch=3, steps=2, strain=0.002, corr=2.0)
    f1, f2 = plate.fields(1), plate.fields(2)
    s = plate_specimen(G, plate)
    target = s.adjoint_forward(*f2, plate.step_bcs(), cases.T_TOP, "z")
    s.close()
    L_gpu, grads, st, _ = loss_and_grad(G, plate, f1, target)
    assert st["status"] == 0

    def oracle_loss(fields):
        o = oracle_mod.Oracle()
        n = o.setup_particles(plate.lattice, plate.radius, plate.xyz)
        o.set_types(cases.sc_types(o.d("xyz", (n, 3)), o.i("nb", (n,)), plate.radius))
        E, nu, sy, H = fields
        c11, c12, c44 = cases.iso_cubic(E, nu)
        o.set_material(c11, c12, c44, sy, H, 0.0, 0)
        o.init_state()
        top = o.i("type", (n,)) == cases.T_TOP
        R = []
        for b in plate.step_bcs():
            o.load_step(b, [], 1e-12, 3000, 1e-20, 0.0)
            R.append(-o.d("Pin", (n, 3))[top, 2].sum())
        return float(((np.array(R) - target) ** 2).sum())

    assert abs(oracle_loss(f1) - L_gpu) <= 1e-8 * L_gpu
    for k, name in enumerate(["E", "nu", "sigmay", "H"]):
        d = f1[k] * plate.fields(7 + k)[k] / plate.BASE[k]
        h = 1e-5
        fp = [x.copy() for x in f1]
        fm = [x.copy() for x in f1]
        fp[k] = f1[k] + h * d
        fm[k] = f1[k] - h * d
        fd = (oracle_loss(fp) - oracle_loss(fm)) / (2 * h)
        ad = float((grads[name] * d).sum())
        assert abs(fd - ad) <= 1e-5 * abs(ad), (name, fd, ad)
