"""Host logic of the GPU damage stage, on the CPU: the brittle pass's choice
of bonds (lpm_damage_brittle_select, used by lpm_load_step after the
candidate kernel) against the oracle's restatement of updateBrittleDamage
(src/constitutive.c:1437-1527), which reproduces the reference bit for bit
(tests/test_oracle_damage.py).  Candidates arrive from the GPU in any order;
ties in strain are frequent (a bond and its reverse always tie)."""
import numpy as np
import pytest


@pytest.mark.parametrize("seed", range(12))
def test_brittle_choice_matches_oracle(oracle_mod, gpu_lib, seed):
    rng = np.random.default_rng(seed)
    n = int(rng.integers(5, 400))
    k = int(rng.integers(0, min(18 * n, 900)))
    bonds = rng.choice(18 * n, size=k, replace=False).astype(np.int32)
    # strains from a small set of values: many exact ties, as for reverse bonds
    levels = rng.uniform(2e-3, 3e-3, size=max(1, k // 3))
    strain = levels[rng.integers(0, len(levels), size=k)]
    nbreak = int(rng.integers(0, 30))
    got = gpu_lib.brittle_select(bonds, strain, n, nbreak)
    # the oracle takes the candidates in the reference's scan order (i, then j)
    i, j = bonds % n, bonds // n
    order = np.lexsort((j, i))
    ref = oracle_mod.brittle_select(i[order], j[order], strain[order], nbreak)
    assert np.array_equal(np.stack([got % n, got // n], axis=1).reshape(-1, 2), ref.reshape(-1, 2))
    assert len(got) == min(k, nbreak) if k > nbreak else len(got) == k
