"""CPU checks: computeStrain's weighted least squares (src/lpm_basic.c:127-249)
restated with numpy reproduces the reference's strain tensor from its own
bond stretches; the synthetic case generators build what they promise."""
import numpy as np

import cases
from conftest import golden


def lsq_strain(x0, nbr, shell, L0, dL):
    """e (6: e11 e22 e33 e23 e13 e12) minimising sum_b w_b (n.e.n - dL/L0)^2,
    w = 0.1 first shell, 0.9 second; normal equations in the reference's
    unknown order (e11 e12 e13 e22 e23 e33)."""
    n = x0.shape[0]
    out = np.zeros((n, 6))
    pairs = [(0, 0), (0, 1), (0, 2), (1, 1), (1, 2), (2, 2)]
    for i in range(n):
        A = np.zeros((6, 6))
        b = np.zeros(6)
        for j in range(nbr.shape[1]):
            p = nbr[i, j]
            if p < 0 or shell[i, j] not in (0, 1):
                continue
            w = 0.1 if shell[i, j] == 0 else 0.9
            u = (x0[p] - x0[i]) / L0[i, j]
            m = np.array([u[a] * u[c] for a, c in pairs])
            A += w * np.outer(m, m)
            b += w * dL[i, j] / L0[i, j] * m
        e = np.linalg.solve(A, b)
        out[i] = [e[0], e[3], e[5], e[4], e[2], e[1]]
    return out


def test_strain_restatement_matches_reference():
    d = golden("output_sc6_j2.npz")
    case = cases.SCCase(n=6)
    x0 = d["xyz0"]
    n = x0.shape[0]
    # bond lists of the 6^3 lattice from positions (the reference's order: ascending partner index)
    h = 2 * case.radius
    nbr = -np.ones((n, 18), dtype=int)
    shell = -np.ones((n, 18), dtype=int)
    for i in range(n):
        dist = np.linalg.norm(x0 - x0[i], axis=1)
        cand = [j for j in range(n) if j != i and dist[j] < 1.01 * np.sqrt(2) * h]
        for k, j in enumerate(cand):
            nbr[i, k] = j
            shell[i, k] = 0 if dist[j] < 1.01 * h else 1
    e = lsq_strain(x0, nbr, shell, d["distance_initial"], d["dL"])
    ref = d["strain"]
    ok = np.abs(ref).max(axis=1) > 0  # particle 0 keeps its previous value when its system is singular
    assert np.allclose(e[ok], ref[ok], rtol=1e-9, atol=1e-12 * np.abs(ref).max())


def test_sc_box_exact_counts():
    for nx, ny, nz in [(3, 4, 5), (20, 33, 41), (60, 21, 37)]:
        box = cases.sc_box_exact(nx, ny, nz, 0.1)
        h = 0.2
        bx = box[1] - box[0]
        # y/z ranges centred on grid lines: a half spacing of margin on both sides
        for lo, hi, m in ((box[2], box[3], ny), (box[4], box[5], nz)):
            assert abs((hi - lo) - m * h) < 1e-12
        assert abs(bx - ((nx - 1) * h + 0.5 * h)) < 1e-12


def test_batch_case_distributions():
    c = cases.BatchCase(nspec=256, seed=1)
    assert c.edges.min() >= 20 and c.edges.max() <= 60
    assert 180e3 <= c.E.min() and c.E.max() <= 220e3
    assert 200.0 <= c.sigmay.min() and c.sigmay.max() <= 400.0
    assert c.particles() == int(np.prod(c.edges, axis=1).sum())


def test_notched_plate_geometry():
    p = cases.NotchedPlate(nx=20, ny=3, nz=20, notch=5)
    g = p.grid
    assert p.n == 20 * 3 * 20 - 5 * 3
    cut = (g[:, 2] == 10) & (g[:, 0] < 5)
    assert not cut.any()
    E, nu, sy, H = p.fields(1)
    for f, base in zip((E, nu, sy, H), p.BASE):
        assert np.all(np.abs(f / base - 1.0) <= 0.1 + 1e-12)
