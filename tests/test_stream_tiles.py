"""The tile arithmetic of the streamed kernels (k_spmv_diff_stream in
k_solve.cu, k_amg_k0_stream in k_amg.cu), restated on the CPU for the block-CSR
patterns the GPU builds, and checked against the buffers it addresses.  No GPU:
the streamed kernels copy with cp.async.bulk, which faults on a misaligned or
out-of-range copy, so every copy and every shared-memory read of every tile is
checked here, for each variant's shape.

Restated from the kernels and their host layouts (init_stream_product,
init_stream_smoother):
- tile t of ROWS rows starts at row r0 = ROWS t; it copies the row offsets
  r0 .. r0 + ROWS + 1 ((ROWS + 2) x 8 B; the device row-offset array holds
  ceil(n / 16) 16 + 2 entries, padded with the total), the column indices
  [b0, b1) (4 B each) and the values: 36 B per block for the product; for
  the smoother the FP16 values' bytes [18 b0, 18 b1) widened to 16-byte
  boundaries (the FP16 array is padded by 16 bytes);
- stage layout: columns at round_up((ROWS + 2) 8, 128), values after
  round_up(ROWS max_npad 4, 128), stage bytes a multiple of 128;
- stages per CTA: min(8, (min(optin, per_sm / CTAs) - 2048) / stage bytes),
  at least 2 (GB300: 232,448 B per block opt-in, 233,472 B per SM).
"""
import numpy as np
import pytest

import cases

OPTIN, PER_SM = 232448, 233472
VARIANTS = {  # name: (rows per tile, CTAs per SM)
    "product 16x1": (16, 1), "product 16x2": (16, 2), "product 8x5": (8, 5),
    "smoother 16x1": (16, 1), "smoother 16x2": (16, 2), "smoother 8x6": (8, 6),
}


def _up(v, a):
    return (v + a - 1) // a * a


def _pattern(oracle_mod, which):
    if which[0] == "sc":
        case = cases.SCCase(n=which[1])
    else:
        case = cases.FCCCase(ncell=which[1])
    o = oracle_mod.Oracle()
    n = o.setup_lattice(case.lattice, case.radius, case.box)
    nconn = o.i("nb_conn", (n,)).astype(np.int64)
    return (nconn + 3) & ~3  # rows padded to multiples of 4 blocks (setup.cpp)


@pytest.mark.parametrize("which", [("sc", 12), ("sc", 23), ("fcc", 7)])
@pytest.mark.parametrize("variant", list(VARIANTS))
def test_stream_tiles_stay_in_bounds(oracle_mod, which, variant):
    npad = _pattern(oracle_mod, which)
    rows, ctas = VARIANTS[variant]
    smoother = variant.startswith("smoother")
    n = npad.size
    rowoff = np.zeros(n + 1, np.int64)
    rowoff[1:] = np.cumsum(npad)
    nblk = int(rowoff[n])
    nro = (n + 15) // 16 * 16 + 2
    ro = np.full(nro, rowoff[n])
    ro[:n + 1] = rowoff
    maxnp = int(npad.max())
    assert maxnp <= 64 and np.all(npad % 4 == 0)
    cols_off = _up((rows + 2) * 8, 128)
    vals_off = cols_off + _up(rows * maxnp * 4, 128)
    stage = vals_off + (_up(rows * maxnp * 18 + 16, 128) if smoother else _up(rows * maxnp * 36, 128))
    stages = min(8, (min(OPTIN, PER_SM // ctas) - 2048) // stage)
    assert stages >= 2, "two stages must fit"
    assert ctas * (stages * stage + 256 + 1024) <= PER_SM  # dynamic + static + per-block reservation
    ntiles = (n + rows - 1) // rows
    r0 = np.arange(ntiles) * rows
    r1 = np.minimum(r0 + rows, n)
    b0, b1 = rowoff[r0], rowoff[r1]
    nb = b1 - b0
    # row-offset copy: (rows + 2) entries from r0, 16-byte aligned, inside the padded array
    assert ((rows + 2) * 8) % 16 == 0 and np.all((r0 * 8) % 16 == 0) and np.all(r0 + rows + 1 < nro)
    # column copy
    assert np.all((4 * b0) % 16 == 0) and np.all((4 * nb) % 16 == 0) and np.all(4 * nb <= vals_off - cols_off)
    if smoother:
        v0 = (18 * b0) & ~15
        v1 = (18 * b1 + 15) & ~15
        vb = np.where(nb > 0, v1 - v0, 0)
        assert np.all(v1 <= 2 * (9 * nblk + 8)) and np.all(vb % 16 == 0) and np.all(vb <= stage - vals_off)
        delta = (18 * b0) & 15
        assert set(np.unique(delta)) <= {0, 8}
    else:
        assert np.all((36 * b0) % 16 == 0) and np.all(36 * nb <= stage - vals_off)
        assert np.all((rows + 2) * 8 + 40 * nb < (1 << 20))  # mbarrier transaction count
    # shared-memory reads of every row: the tile-local block offset o and
    # count np from the copied row offsets, 16-byte column reads and 16-byte
    # (product) or 8-byte (smoother) value reads per component
    for t in range(ntiles):
        sl = ro[r0[t]:r0[t] + rows + 2]
        for rl in range(rows):
            if r0[t] + rl >= n:
                continue
            o = int(sl[rl] - sl[0])
            npr = int(sl[rl + 1] - sl[rl])
            assert npr == npad[r0[t] + rl] and o % 4 == 0
            assert o + npr <= nb[t]  # columns inside the copied range
            last = 9 * o + 8 * npr + npr - 4  # last value group read
            if smoother:
                a = int(delta[t]) + 2 * last
                assert a % 8 == 0 and a + 8 <= vb[t]
            else:
                assert (4 * last) % 16 == 0 and 4 * (last + 4) <= 36 * nb[t]
