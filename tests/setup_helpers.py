"""Build the same specimen in the oracle (CPU restatement) and on the GPU."""
import numpy as np

import cases


def sc_oracle(O, case, threads=4):
    O.set_threads(threads)
    o = O.Oracle()
    n = o.setup_lattice(case.lattice, case.radius, case.box)
    xyz = o.d("xyz", (n, 3))
    nb = o.i("nb", (n,))
    types = cases.sc_types(xyz, nb, case.radius)
    o.set_types(types)
    c11, c12, c44 = material_arrays(case, n)
    o.set_material(c11, c12, c44, case.sigmay, case.H, getattr(case, "xi", 0.0), 0)
    o.init_state()
    return o, types


def sc_gpu(G, case, precision=0, **solver):
    s = G.Specimen(0)
    n = s.setup_lattice(case.lattice, case.radius, case.box)
    xyz = s.get("xyz")
    nb = s.get("nb")
    types = cases.sc_types(xyz, nb, case.radius)
    s.set_types(types)
    c11, c12, c44 = material_arrays(case, n)
    s.set_material(c11, c12, c44, case.sigmay, case.H, getattr(case, "xi", 0.0), G.PL_J2)
    s.init_state()
    s.set_solver(precision=precision, newton_tol=case.newton_tol, **solver)
    return s, types


def material_arrays(case, n):
    c11, c12, c44 = cases.iso_cubic(case.E, case.nu)
    if case.e_noise:
        u = cases.splitmix64_uniform(case.seed, n)
        scale = 1.0 + case.e_noise * (2.0 * u - 1.0)
        return c11 * scale, c12 * scale, c44 * scale
    return np.full(n, c11), np.full(n, c12), np.full(n, c44)


def batch_gpu(G, case, precision=0, **solver):
    """All specimens of a cases.BatchCase in one batch context."""
    s = G.Specimen(0)
    n = s.setup_batch(case.lattice, case.radius, case.boxes)
    off = s.batch_offsets()
    xyz, nb = s.get("xyz"), s.get("nb")
    types = np.concatenate([cases.sc_types(xyz[off[k]:off[k + 1]], nb[off[k]:off[k + 1]], case.radius)
                            for k in range(case.nspec)])
    reps = np.diff(off)
    E = np.repeat(case.E, reps)
    c11, c12, c44 = cases.iso_cubic(E, case.nu)
    s.set_types(types)
    s.set_material(c11, c12, c44, np.repeat(case.sigmay, reps), np.full(n, case.H), 0.0, G.PL_J2)
    s.init_state()
    s.set_solver(precision=precision, newton_tol=case.newton_tol, **solver)
    return s, off


def single_of_batch(G, case, k, precision=0, **solver):
    """Specimen k of a cases.BatchCase alone in its own context."""
    s = G.Specimen(0)
    n = s.setup_lattice(case.lattice, case.radius, case.boxes[k])
    types = cases.sc_types(s.get("xyz"), s.get("nb"), case.radius)
    c11, c12, c44 = cases.iso_cubic(case.E[k], case.nu)
    s.set_types(types)
    s.set_material(np.full(n, c11), np.full(n, c12), np.full(n, c44), np.full(n, case.sigmay[k]),
                   np.full(n, case.H), 0.0, G.PL_J2)
    s.init_state()
    s.set_solver(precision=precision, newton_tol=case.newton_tol, **solver)
    return s
