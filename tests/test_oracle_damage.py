"""The oracle's restatement of the reference main's damage stage against
golden data written by the reference itself (tests/golden/make_golden.py,
reference built from its own sources): updateDuctileDamagePwiseNonlocal for
J2 and updateBrittleDamage for elastic bonds (src/constitutive.c:1437-1527,
:1757-1862), updateCrack (:1399-1434) and the re-solve of a load step after
bonds break (src/lpmc_project.c:528-546).  Bit-exact: per step the Newton
iterations, residual norms, passes, the broken-bond log in order, and the
damage, force and plastic state."""
import numpy as np
import pytest

import cases
from conftest import golden


def _ductile(O):
    case = cases.DuctileDamageCase()
    O.set_threads(1)
    o = O.Oracle()
    n = o.setup_lattice(case.lattice, case.radius, case.box)
    xyz0 = o.d("xyz", (n, 3))
    types = cases.sc_types(xyz0, o.i("nb", (n,)), case.radius)
    o.set_types(types)
    c11, c12, c44 = cases.iso_cubic(case.E, case.nu)
    o.set_material(c11, c12, c44, case.sigmay(xyz0), case.H, 0.0, 0)
    o.init_state()
    o.set_damage(L=case.L, threshold=case.threshold, cA=0.0)
    return o, types, [cases.sc_bcs(v) for v in case.schedule], case.newton_tol


def _brittle(O):
    case = cases.BrittleCase()
    O.set_threads(1)
    o = O.Oracle()
    n = o.setup_lattice(case.lattice, case.radius, case.box)
    xyz0 = o.d("xyz", (n, 3))
    types = case.types(xyz0, o.i("nb", (n,)))
    o.set_types(types)
    c11, c12, c44 = cases.iso_cubic(case.E, case.nu)
    o.set_material(c11, c12, c44, 1e30, 0.0, 0.0, 6)
    o.init_state()
    o.set_damage(crit_bstrain=case.crit, nbreak=case.nbreak)
    return o, types, [case.bcs(v) for v in case.schedule], case.newton_tol


@pytest.mark.parametrize("which", ["ductile", "brittle"])
def test_damage_stage_bit_exact(oracle_mod, which):
    g = golden(f"damage_{which}.npz")
    o, types, step_bcs, tol = (_ductile if which == "ductile" else _brittle)(oracle_mod)
    n, nn = o.n, o.nn
    assert np.array_equal(types, g["types"])
    logged = 0
    for s, bcs in enumerate(step_bcs, start=1):
        st = o.load_step_damage(bcs, [], tol, 200, 1e-20, 0.0, 50)
        ref = g["stats"][s - 1]
        assert np.array_equal(st, ref), (s, st, ref)
        log = o.broken_log()
        assert np.array_equal(log[logged:], g[f"s{s}_pairs"]), s
        logged = log.shape[0]
        if f"s{s}_brk" not in g:
            continue
        assert np.array_equal(o.d("xyz", (n, 3)), g[f"s{s}_xyz"]), s
        assert np.array_equal(o.d("F", (n, nn)), g[f"s{s}_F"]), s
        assert np.array_equal(o.d("Pin", (3 * n,)), g[f"s{s}_Pin"]), s
        assert np.array_equal(o.d("damage_broken", (n, nn)), g[f"s{s}_brk"]), s
        assert np.array_equal(o.d("damage_w", (n, nn)), g[f"s{s}_w"]), s
        assert np.array_equal(o.d("damage_D1", (n, nn)), g[f"s{s}_D"]), s
        assert np.array_equal(o.d("damage_nonlocal1", (n,)), g[f"s{s}_dnl"]), s
        assert np.array_equal(o.d("damage_visual", (n,)), g[f"s{s}_dvis"]), s
        assert np.array_equal(o.i("nb_current", (n,)), g[f"s{s}_nb"]), s
        assert np.array_equal(o.i("fix_index", (3 * n,)), g[f"s{s}_fix"]), s
        assert np.array_equal(o.d("alpha1", (n,)), g[f"s{s}_alpha"]), s
        assert np.array_equal(o.d("dLp1", (n, nn)), g[f"s{s}_dLp"]), s
    # the case reached what it is meant to exercise
    assert g["stats"][:, 6].sum() > 0 and g["stats"][:, 5].max() > 1
    if which == "ductile":
        assert o.d("damage_nonlocal1", (n,)).max() > 0.0
    else:
        assert g["stats"][:, 6].max() > cases.BrittleCase().nbreak  # the sorted, limited branch
