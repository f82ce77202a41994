"""Generate the golden vectors under tests/golden/ from the LPM-C reference itself.

Runs the reference's own C sources (built by oracle/build_ref.sh into
oracle/_ref/libref_lpm.so, MKL replaced by the public-API shim) on the SC
cyclic case at 10x10x10 (C1), a small FCC crystal-plasticity case, a
force-controlled SC case (setForceBC) and two cases of the main loop's damage
stage (ductile nonlocal for J2, brittle for elastic), and
stores inputs and outputs as compressed .npz fixtures.  The reference runs
single-threaded (its OpenMP loops race, see src/constitutive.c:95 with
:495-515,625-645), so the fixtures are deterministic.

    python tests/golden/make_golden.py [--steps N]

Reference CG tolerances are overridden to |r|^2 <= 1e-20 |r0|^2 (1e-10 on the
norm, absolute 0) because the hard-coded 1e-8 / 1e-12 (src/solver.c:221-222)
makes a Newton tolerance of 1e-8 unreachable at these force levels.
"""
import argparse
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, HERE)

import refdrv as R  # noqa: E402
import cases  # noqa: E402


def snapshot(n, nn):
    """State the reference keeps after a converged step (slot 1 = converged)."""
    return dict(
        xyz=R.get_d2("xyz", n, 3),
        F=R.get_d2("F", n, nn),
        csx=R.get_d2("csx", n, nn), csy=R.get_d2("csy", n, nn), csz=R.get_d2("csz", n, nn),
        dLp=R.get_d3("dLp", n, nn, 1),
        alpha=R.get_d2("J2_alpha", n, 3)[:, 1],
        beta=R.get_d3("J2_beta", n, 6, 1),
        Pin=R.get_d1("Pin", 3 * n),
        Pex=R.get_d1("Pex", 3 * n),
        stress=R.get_d2("stress_tensor", n, 6),
    )


def sc_case(out, nsteps, tag="sc10"):
    case = cases.SCCase(n=10)
    t0 = time.time()
    n = R.setup(case.lattice, case.radius, case.box)
    nn = R.gint("nneighbors")
    xyz0 = R.get_d2("xyz", n, 3)
    nb = R.get_i1("nb", n)
    types = cases.sc_types(xyz0, nb, case.radius)
    R.set_types(types, cases.NTYPE)
    R.material(case.ce_per_type(), 0, np.full(n, case.sigmay), 0.0, case.H)
    R.init_state()
    R.set_cg_tol(1e-20, 0.0)
    kp = R.get_i2("K_pointer", n + 1, 2)
    nnz = int(kp[n, 1])
    setup = dict(
        box=np.array(case.box), radius=case.radius, types=types, xyz=xyz0,
        neighbors=R.get_i2("neighbors", n, nn), nsign=R.get_i2("nsign", n, nn), nb=nb,
        distance_initial=R.get_d2("distance_initial", n, nn),
        csx_initial=R.get_d2("csx_initial", n, nn), csy_initial=R.get_d2("csy_initial", n, nn),
        csz_initial=R.get_d2("csz_initial", n, nn),
        conn=R.get_i2("conn", n, R.gint("nneighbors_AFEM") + 1), nb_conn=R.get_i1("nb_conn", n),
        K_pointer=kp, Kn=R.get_d2("Kn", n, nn), Tv=R.get_d2("Tv", n, nn),
    )
    np.savez_compressed(os.path.join(out, f"{tag}_setup.npz"), **setup)

    sched = case.schedule[:nsteps]
    rec = {k: [] for k in ("iters", "nres0", "nreac0", "nres", "cg", "disp_top", "react_top")}
    snaps = {}
    # every 20 steps (each quarter cycle's end), so that the whole run can be
    # replayed in independent segments
    snap_steps = {1, 13, 14, len(sched)} | set(range(20, len(sched) + 1, 20))
    for s, stp in enumerate(sched, start=1):
        if s == 1 or s == 14:
            # stiffness at the converged state entering this step (FD, upper CSR)
            state_in = snapshot(n, nn)
            with R.quiet():
                R.lib().calcStiffness3DFiniteDifference(6)
            # the finite-difference sweep overwrites F (src/constitutive.c:270), which
            # the load step copies into F_temp for its predictor: put it back
            R.set_d2("F", state_in["F"])
            K = R.get_d1("K_global", nnz)
            IK = R.get_i1("IK", 3 * n + 1)
            JK = R.get_i1("JK", nnz)
            np.savez_compressed(os.path.join(out, f"{tag}_K_step{s}.npz"), K_global=K, IK=IK, JK=JK,
                                **{"in_" + k: v for k, v in state_in.items()})
        with R.quiet():
            st = R.load_step(cases.sc_bcs(stp), [], case.newton_tol)
        xyz = R.get_d2("xyz", n, 3)
        F = R.get_d2("F", n, nn)
        csz = R.get_d2("csz", n, nn)
        top = types == cases.T_TOP
        rec["iters"].append(st[0])
        rec["nres0"].append(st[1])
        rec["nreac0"].append(st[2])
        rec["nres"].append(st[3])
        rec["cg"].append(st[4])
        rec["disp_top"].append((xyz[top, 2].sum() - xyz0[top, 2].sum()) / top.sum())
        rec["react_top"].append(np.sum(-csz[top] * F[top]))
        if s in snap_steps:
            snaps[s] = snapshot(n, nn)
        print(f"{tag} step {s}: iters {int(st[0])} res {st[3]:.3e} t={time.time() - t0:.1f}s", flush=True)
    arrs = {k: np.array(v) for k, v in rec.items()}
    arrs["schedule"] = np.array(sched)
    for s, d in snaps.items():
        for k, v in d.items():
            arrs[f"s{s}_{k}"] = v
    arrs["snap_steps"] = np.array(sorted(snaps))
    np.savez_compressed(os.path.join(out, f"{tag}_cyclic.npz"), **arrs)


def fcc_case(out, nsteps, tag="fcc4", case=None):
    """FCC crystal plasticity (computeBondForceCPMiehe), [001] tension, 4^3 cells."""
    case = case or cases.FCCCase(ncell=4)
    t0 = time.time()
    n = R.setup(case.lattice, case.radius, case.box)
    nn = R.gint("nneighbors")
    xyz0 = R.get_d2("xyz", n, 3)
    nb = R.get_i1("nb", n)
    types = cases.sc_types(xyz0, nb, case.radius)
    R.set_types(types, cases.NTYPE)
    R.material(case.ce_per_type(), 1, np.zeros(n), 0.0, 0.0, np.array(case.cp))
    R.init_state()
    R.set_cg_tol(1e-20, 0.0)
    ns = R.gint("nslipSys")
    arrs = dict(box=np.array(case.box), types=types, xyz=xyz0, cp=np.array(case.cp),
                schmid=R.get_d2("schmid_tensor", ns, 6),
                neighbors=R.get_i2("neighbors", n, nn), nsign=R.get_i2("nsign", n, nn),
                distance_initial=R.get_d2("distance_initial", n, nn),
                Kn=R.get_d2("Kn", n, nn), Tv=R.get_d2("Tv", n, nn),
                cp_Cab=R.get_d2("cp_Cab", n, ns * ns))
    rec = {k: [] for k in ("iters", "nres", "disp_top", "react_top")}
    top = types == cases.T_TOP
    for s, stp in enumerate(case.schedule[:nsteps], start=1):
        with R.quiet():
            st = R.load_step(cases.sc_bcs(stp), [], case.newton_tol)
        xyz = R.get_d2("xyz", n, 3)
        F = R.get_d2("F", n, nn)
        csz = R.get_d2("csz", n, nn)
        rec["iters"].append(st[0])
        rec["nres"].append(st[3])
        rec["disp_top"].append((xyz[top, 2].sum() - xyz0[top, 2].sum()) / top.sum())
        rec["react_top"].append(np.sum(-csz[top] * F[top]))
        if s in (5, nsteps):
            arrs[f"s{s}_xyz"] = xyz
            arrs[f"s{s}_F"] = F
            for c in ("csx", "csy", "csz"):
                arrs[f"s{s}_{c}"] = R.get_d2(c, n, nn)
            arrs[f"s{s}_dLp"] = R.get_d3("dLp", n, nn, 1)
            arrs[f"s{s}_cp_gy"] = R.get_d3("cp_gy", n, ns, 1)
            arrs[f"s{s}_cp_A_single"] = R.get_d3("cp_A_single", n, ns, 1)
            arrs[f"s{s}_cp_A"] = R.get_d2("cp_A", n, 3)[:, 1]
        print(f"{tag} step {s}: iters {int(st[0])} res {st[3]:.3e} t={time.time() - t0:.1f}s", flush=True)
    for k, v in rec.items():
        arrs[k] = np.array(v)
    arrs["schedule"] = np.array(case.schedule[:nsteps])
    np.savez_compressed(os.path.join(out, f"{tag}_cp.npz"), **arrs)


def force_case(out, tag="sc_force"):
    """Force-controlled SC J2 case (setForceBC): top-face force ramp into the
    plastic range, x and z components."""
    case = cases.ForceCase()
    t0 = time.time()
    n = R.setup(case.lattice, case.radius, case.box)
    nn = R.gint("nneighbors")
    xyz0 = R.get_d2("xyz", n, 3)
    types = cases.sc_types(xyz0, R.get_i1("nb", n), case.radius)
    R.set_types(types, cases.NTYPE)
    R.material(case.ce_per_type(), 0, np.full(n, case.sigmay), 0.0, case.H)
    R.init_state()
    R.set_cg_tol(1e-20, 0.0)
    disp, force = case.bcs()
    rec = {k: [] for k in ("iters", "nres0", "nreac0", "nres", "disp_top_x", "disp_top_z")}
    top = types == cases.T_TOP
    arrs = dict(box=np.array(case.box), types=types, xyz=xyz0)
    for s in range(1, case.steps + 1):
        with R.quiet():
            st = R.load_step(disp, force, case.newton_tol)
        xyz = R.get_d2("xyz", n, 3)
        rec["iters"].append(st[0])
        rec["nres0"].append(st[1])
        rec["nreac0"].append(st[2])
        rec["nres"].append(st[3])
        rec["disp_top_x"].append((xyz[top, 0].sum() - xyz0[top, 0].sum()) / top.sum())
        rec["disp_top_z"].append((xyz[top, 2].sum() - xyz0[top, 2].sum()) / top.sum())
        print(f"{tag} step {s}: iters {int(st[0])} res {st[3]:.3e} t={time.time() - t0:.1f}s", flush=True)
    for k, v in rec.items():
        arrs[k] = np.array(v)
    arrs["s_xyz"] = R.get_d2("xyz", n, 3)
    arrs["s_alpha"] = R.get_d2("J2_alpha", n, 3)[:, 1]
    arrs["s_dLp"] = R.get_d3("dLp", n, nn, 1)
    arrs["s_Pex"] = R.get_d1("Pex", 3 * n)
    arrs["s_F"] = R.get_d2("F", n, nn)
    np.savez_compressed(os.path.join(out, f"{tag}.npz"), **arrs)


def _damage_record(n, nn, bondfile):
    """Arrays after a damaged load step and the broken pairs the reference
    logged (TIMESTEP lines dropped)."""
    pairs = [tuple(int(v) for v in line.split()) for line in open(bondfile).read().splitlines()
             if line and not line.startswith("TIMESTEP")]
    return dict(
        xyz=R.get_d2("xyz", n, 3), F=R.get_d2("F", n, nn), Pin=R.get_d1("Pin", 3 * n),
        brk=R.get_d2("damage_broken", n, nn), w=R.get_d2("damage_w", n, nn),
        D=R.get_d3("damage_D", n, nn, 1), dnl=R.get_d2("damage_nonlocal", n, 2)[:, 1],
        dvis=R.get_d1("damage_visual", n), nb=R.get_i1("nb", n), fix=R.get_i1("fix_index", 3 * n),
        alpha=R.get_d2("J2_alpha", n, 3)[:, 1], dLp=R.get_d3("dLp", n, nn, 1),
        pairs=np.array(pairs, dtype=np.int32).reshape(-1, 2))


def damage_case(out, which):
    """The reference's main loop with its damage stage: ductile nonlocal (J2)
    or brittle (elastic); per step the stats, the broken-bond log and the
    damage state."""
    import tempfile
    if which == "ductile":
        case = cases.DuctileDamageCase()
        n = R.setup(case.lattice, case.radius, case.box)
        xyz0 = R.get_d2("xyz", n, 3)
        types = cases.sc_types(xyz0, R.get_i1("nb", n), case.radius)
        R.set_types(types, cases.NTYPE)
        R.material(case.ce_per_type(), 0, case.sigmay(xyz0), 0.0, case.H)
        R.init_state()
        R.set_damage(L=case.L, threshold=case.threshold, cA=0.0)
        step_bcs = [cases.sc_bcs(v) for v in case.schedule]
        tag = "damage_ductile"
        full_steps = {5, 6, 7}
    else:
        case = cases.BrittleCase()
        n = R.setup(case.lattice, case.radius, case.box)
        xyz0 = R.get_d2("xyz", n, 3)
        types = case.types(xyz0, R.get_i1("nb", n))
        R.set_types(types, cases.NTYPE + 1)
        ce = np.tile(cases.iso_cubic(case.E, case.nu), (cases.NTYPE + 1, 1))
        R.material(ce, 6, np.full(n, 1e30), 0.0, 0.0)
        R.init_state()
        R.set_damage(crit_bstrain=case.crit, nbreak=case.nbreak)
        step_bcs = [case.bcs(v) for v in case.schedule]
        tag = "damage_brittle"
        full_steps = {3, 6, 12}
    R.set_cg_tol(1e-20, 0.0)
    nn = R.gint("nneighbors")
    arrs = dict(types=types, xyz0=xyz0)
    stats = []
    t0 = time.time()
    with tempfile.TemporaryDirectory() as tmp:
        for s, bcs in enumerate(step_bcs, start=1):
            bondfile = os.path.join(tmp, f"bonds{s}.txt")
            with R.quiet():
                st = R.load_step_damage(bcs, [], case.newton_tol, bondfile, s, maxiter=200, max_passes=50)
            stats.append(st)
            rec = _damage_record(n, nn, bondfile)
            arrs[f"s{s}_pairs"] = rec.pop("pairs")
            if s in full_steps:  # the whole state only where damage changes course
                for k, v in rec.items():
                    arrs[f"s{s}_{k}"] = v
            print(f"{tag} step {s}: newton {int(st[0])} passes {int(st[5])} candidates {int(st[6])} "
                  f"res {st[3]:.2e} t={time.time() - t0:.1f}s", flush=True)
    arrs["stats"] = np.array(stats)
    np.savez_compressed(os.path.join(out, f"{tag}.npz"), **arrs)


def setup_case(out, name):
    """Bond lists, AFEM connectivity and K_pointer of a setup-only shape
    (searchNormalNeighbor, searchAFEMNeighbor), with the generated lattice."""
    lattice, radius, box = cases.SETUP_SHAPES[name]
    n = R.setup(lattice, radius, box)
    nn = R.gint("nneighbors")
    arrs = dict(
        box=np.array(box), xyz=R.get_d2("xyz", n, 3),
        neighbors=R.get_i2("neighbors", n, nn), nsign=R.get_i2("nsign", n, nn), nb=R.get_i1("nb", n),
        distance_initial=R.get_d2("distance_initial", n, nn),
        csx_initial=R.get_d2("csx_initial", n, nn), csy_initial=R.get_d2("csy_initial", n, nn),
        csz_initial=R.get_d2("csz_initial", n, nn),
        conn=R.get_i2("conn", n, R.gint("nneighbors_AFEM") + 1), nb_conn=R.get_i1("nb_conn", n),
        K_pointer=R.get_i2("K_pointer", n + 1, 2))
    np.savez_compressed(os.path.join(out, f"setup_{name}.npz"), **arrs)
    print(f"setup {name}: {n} particles", flush=True)


def noise_case(out, tag="sc8_enoise"):
    """Per-particle moduli (the C2 material model at small size): E = 200 GPa
    (1 + 0.05 U[-1, 1]) per particle, seed 1, as unique reference types (one
    Ce row per particle) with the usual types as BC groups; bond Kn/Tv are the
    two end particles' averages (src/stiffness.c:186-200).  14 cyclic steps
    into the plastic range."""
    case = cases.SCCase(n=8, sigmay=150.0, e_noise=0.05, seed=1)
    n = R.setup(case.lattice, case.radius, case.box)
    nn = R.gint("nneighbors")
    xyz0 = R.get_d2("xyz", n, 3)
    groups = cases.sc_types(xyz0, R.get_i1("nb", n), case.radius)
    u = cases.splitmix64_uniform(case.seed, n)
    scale = 1.0 + case.e_noise * (2.0 * u - 1.0)
    c11, c12, c44 = cases.iso_cubic(case.E, case.nu)
    ce = np.stack([c11 * scale, c12 * scale, c44 * scale], axis=1)
    R.set_types(np.arange(n, dtype=np.int32), n)
    R.set_bc_groups(groups)
    R.material(ce, 0, np.full(n, case.sigmay), 0.0, case.H)
    R.init_state()
    R.set_cg_tol(1e-20, 0.0)
    arrs = dict(groups=groups, xyz=xyz0, Kn=R.get_d2("Kn", n, nn), Tv=R.get_d2("Tv", n, nn))
    top = groups == cases.T_TOP
    rec = {k: [] for k in ("iters", "nres", "disp_top")}
    for s_, stp in enumerate(case.schedule[:14], start=1):
        with R.quiet():
            st = R.load_step(cases.sc_bcs(stp), [], case.newton_tol)
        xyz = R.get_d2("xyz", n, 3)
        rec["iters"].append(st[0])
        rec["nres"].append(st[3])
        rec["disp_top"].append((xyz[top, 2].sum() - xyz0[top, 2].sum()) / top.sum())
    for k, v in rec.items():
        arrs[k] = np.array(v)
    arrs["s_xyz"] = R.get_d2("xyz", n, 3)
    arrs["s_alpha"] = R.get_d2("J2_alpha", n, 3)[:, 1]
    arrs["s_F"] = R.get_d2("F", n, nn)
    np.savez_compressed(os.path.join(out, f"{tag}.npz"), **arrs)
    print(f"{tag}: {n} particles, alpha max {arrs['s_alpha'].max():.3e}", flush=True)


def kinematic_case(out, tag="sc6_kinematic"):
    """Mixed linear hardening (J2_xi = 0.5: half kinematic, half isotropic)
    over three quarters of a load cycle of SC 6^3 (8 steps per quarter: up to
    +A, back to 0, on to -A, with reverse yielding): per-step iterations,
    residuals and top displacement, and the final state with the back
    stress."""
    case = cases.SCCase(n=6, sigmay=150.0, xi=0.5, steps_per_quarter=8, cycles=1)
    n = R.setup(case.lattice, case.radius, case.box)
    nn = R.gint("nneighbors")
    xyz0 = R.get_d2("xyz", n, 3)
    types = cases.sc_types(xyz0, R.get_i1("nb", n), case.radius)
    R.set_types(types, cases.NTYPE)
    R.material(case.ce_per_type(), 0, np.full(n, case.sigmay), case.xi, case.H)
    R.init_state()
    R.set_cg_tol(1e-20, 0.0)
    top = types == cases.T_TOP
    rec = {k: [] for k in ("iters", "nres", "disp_top")}
    alpha_max = []
    for s_, stp in enumerate(case.schedule[:24], start=1):
        with R.quiet():
            st = R.load_step(cases.sc_bcs(stp), [], case.newton_tol)
        xyz = R.get_d2("xyz", n, 3)
        rec["iters"].append(st[0])
        rec["nres"].append(st[3])
        rec["disp_top"].append((xyz[top, 2].sum() - xyz0[top, 2].sum()) / top.sum())
        alpha_max.append(R.get_d2("J2_alpha", n, 3)[:, 1].max())
    print(f"{tag}: plastic strain max per step {np.array2string(np.array(alpha_max), precision=2)}", flush=True)
    arrs = {k: np.array(v) for k, v in rec.items()}
    arrs["types"] = types
    arrs["s_xyz"] = R.get_d2("xyz", n, 3)
    arrs["s_alpha"] = R.get_d2("J2_alpha", n, 3)[:, 1]
    arrs["s_beta"] = R.get_d3("J2_beta", n, 6, 1)
    arrs["s_F"] = R.get_d2("F", n, nn)
    np.savez_compressed(os.path.join(out, f"{tag}.npz"), **arrs)
    print(f"{tag}: {n} particles, {len(rec['iters'])} steps, alpha max {arrs['s_alpha'].max():.3e}, "
          f"|beta| max {np.abs(arrs['s_beta']).max():.3e}", flush=True)


def sigmay_case(out, tag="sc8_sigmay"):
    """Per-particle yield stress (the reference's sigmay[i],
    src/constitutive.c:591): sigma_y = 200 + 200 U[0, 1) MPa per particle
    (splitmix64 seed 3), the batch workload's range; 20 cyclic steps of SC 8^3
    with progressive yielding."""
    case = cases.SCCase(n=8)
    n = R.setup(case.lattice, case.radius, case.box)
    nn = R.gint("nneighbors")
    xyz0 = R.get_d2("xyz", n, 3)
    types = cases.sc_types(xyz0, R.get_i1("nb", n), case.radius)
    R.set_types(types, cases.NTYPE)
    sy = cases.sigmay_field(n)
    R.material(case.ce_per_type(), 0, sy, 0.0, case.H)
    R.init_state()
    R.set_cg_tol(1e-20, 0.0)
    top = types == cases.T_TOP
    rec = {k: [] for k in ("iters", "nres", "disp_top")}
    for s_, stp in enumerate(case.schedule[:20], start=1):
        with R.quiet():
            st = R.load_step(cases.sc_bcs(stp), [], case.newton_tol)
        xyz = R.get_d2("xyz", n, 3)
        rec["iters"].append(st[0])
        rec["nres"].append(st[3])
        rec["disp_top"].append((xyz[top, 2].sum() - xyz0[top, 2].sum()) / top.sum())
    arrs = {k: np.array(v) for k, v in rec.items()}
    arrs["types"] = types
    arrs["sigmay"] = sy
    arrs["s_xyz"] = R.get_d2("xyz", n, 3)
    arrs["s_alpha"] = R.get_d2("J2_alpha", n, 3)[:, 1]
    arrs["s_F"] = R.get_d2("F", n, nn)
    np.savez_compressed(os.path.join(out, f"{tag}.npz"), **arrs)
    print(f"{tag}: {n} particles, yielded {(arrs['s_alpha'] > 0).sum()}, alpha max {arrs['s_alpha'].max():.3e}",
          flush=True)


def fcc_j2_case(out, tag="fcc4_j2"):
    """J2 plasticity on the FCC lattice (plmode 0 on lattice 3: 12 first- and
    6 second-shell bonds, the FCC branch of calcKnTv): 4^3 cells with the Al
    constants, sigma_y = 100 MPa, H = 1000 MPa, [001] tension, 12 steps
    (yield near step 7)."""
    case = cases.FCCCase(ncell=4)
    n = R.setup(case.lattice, case.radius, case.box)
    nn = R.gint("nneighbors")
    xyz0 = R.get_d2("xyz", n, 3)
    types = cases.sc_types(xyz0, R.get_i1("nb", n), case.radius)
    R.set_types(types, cases.NTYPE)
    R.material(case.ce_per_type(), 0, np.full(n, cases.FCC_J2["sigmay"]), 0.0, cases.FCC_J2["H"])
    R.init_state()
    R.set_cg_tol(1e-20, 0.0)
    top = types == cases.T_TOP
    rec = {k: [] for k in ("iters", "nres", "disp_top")}
    for s_, stp in enumerate(case.schedule[:12], start=1):
        with R.quiet():
            st = R.load_step(cases.sc_bcs(stp), [], case.newton_tol)
        xyz = R.get_d2("xyz", n, 3)
        rec["iters"].append(st[0])
        rec["nres"].append(st[3])
        rec["disp_top"].append((xyz[top, 2].sum() - xyz0[top, 2].sum()) / top.sum())
    arrs = {k: np.array(v) for k, v in rec.items()}
    arrs["types"] = types
    arrs["s_xyz"] = R.get_d2("xyz", n, 3)
    arrs["s_alpha"] = R.get_d2("J2_alpha", n, 3)[:, 1]
    arrs["s_dLp"] = R.get_d3("dLp", n, nn, 1)
    arrs["s_F"] = R.get_d2("F", n, nn)
    np.savez_compressed(os.path.join(out, f"{tag}.npz"), **arrs)
    print(f"{tag}: {n} particles, iters {arrs['iters'].astype(int).tolist()}, alpha max {arrs['s_alpha'].max():.3e}",
          flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--steps", type=int, default=160)
    ap.add_argument("--fcc-steps", type=int, default=12)
    ap.add_argument("--only", choices=["sc", "fcc", "force", "ductile", "brittle", "enoise", "kinematic", "fcc_sat", "sigmay", "fcc_j2"] +
                    ["setup_" + k for k in cases.SETUP_SHAPES], default=None)
    ap.add_argument("--out", default=HERE)
    args = ap.parse_args()
    if not R.available():
        sys.exit("oracle/_ref/libref_lpm.so missing: run oracle/build_ref.sh first")
    # the reference keeps all state in process globals: one case per process
    if args.only == "fcc":
        fcc_case(args.out, args.fcc_steps)
    elif args.only == "force":
        force_case(args.out)
    elif args.only == "enoise":
        noise_case(args.out)
    elif args.only == "kinematic":
        kinematic_case(args.out)
    elif args.only == "sigmay":
        sigmay_case(args.out)
    elif args.only == "fcc_j2":
        fcc_j2_case(args.out)
    elif args.only == "fcc_sat":
        fcc_case(args.out, args.fcc_steps, tag="fcc4_sat", case=cases.FCCCase(ncell=4, **cases.FCC_SAT))
    elif args.only in ("ductile", "brittle"):
        damage_case(args.out, args.only)
    elif args.only and args.only.startswith("setup_"):
        setup_case(args.out, args.only[len("setup_"):])
    elif args.only == "sc":
        sc_case(args.out, args.steps)
    else:
        import subprocess
        for which in ["sc", "fcc", "force", "ductile", "brittle", "enoise", "kinematic", "fcc_sat", "sigmay",
                      "fcc_j2"] + \
                ["setup_" + k for k in cases.SETUP_SHAPES]:
            subprocess.check_call([sys.executable, __file__, "--only", which, "--steps", str(args.steps),
                                   "--fcc-steps", str(args.fcc_steps), "--out", args.out])


if __name__ == "__main__":
    main()
