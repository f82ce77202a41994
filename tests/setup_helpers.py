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
    o.set_material(c11, c12, c44, case.sigmay, case.H, 0.0, 0)
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
    s.set_material(c11, c12, c44, case.sigmay, case.H, 0.0, G.PL_J2)
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
