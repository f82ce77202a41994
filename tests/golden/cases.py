"""Workload definitions shared by the golden-vector generator, the tests and bench.py.

Each case names a lattice, its material and its load schedule in the terms the
LPM-C reference uses (src/lpmc_project.c:75-335): lattice id, particle radius,
box (createCuboid input), per-type elastic constants, J2 parameters and
per-step displacement boundary conditions given as (type, axis, step).

Rigid-body pin: the SC cases fix only z on the bottom face, which leaves x/y
translation and z-rotation free (a singular stiffness).  Two bottom particles
are additionally pinned (one in x and y, one in y), removing exactly those
three modes without loading the specimen.
"""
import numpy as np

# particle types (reference convention: type selects BCs and Ce rows)
T_INTERIOR, T_TOP, T_BOTTOM, T_FULL, T_PIN_XY, T_PIN_Y = 0, 1, 2, 3, 4, 5
NTYPE = 6


def iso_cubic(E, nu):
    """C11, C12, C44 of an isotropic solid (src/lpmc_project.c:188-190)."""
    C11 = E * (1.0 - nu) / (1.0 + nu) / (1.0 - 2.0 * nu)
    C12 = E * nu / (1.0 + nu) / (1.0 - 2.0 * nu)
    C44 = E / 2.0 / (1.0 + nu)
    return C11, C12, C44


def sc_box(nx, ny, nz, radius):
    """Box for createCuboid (lattice 2) that holds exactly nx*ny*nz particles.

    x starts at box[0]; y and z start at -|box diagonal| (src/initialization.c:247-282),
    so the y/z boxes are widened by half a spacing on both sides to capture
    exactly ny/nz grid lines whatever their offset.
    """
    h = 2.0 * radius
    return [0.0, (nx - 1) * h + 0.5 * h, -0.5 * h, (ny - 1) * h + 0.5 * h,
            -0.5 * h, (nz - 1) * h + 0.5 * h]


def sc_box_exact(nx, ny, nz, radius):
    """Box for createCuboid (lattice 2) holding exactly nx*ny*nz particles for
    any edge lengths.  The generator's y/z grid lines sit at -a + 2r k with a
    the box diagonal (src/initialization.c:241-284), and a depends only on the
    box's edge lengths, so the y/z ranges are centred on grid lines: no line
    falls on a face."""
    h = 2.0 * radius
    bx, by, bz = (nx - 1) * h + 0.5 * h, ny * h, nz * h
    a = np.sqrt(bx * bx + by * by + bz * bz)
    line0 = -a + h * np.ceil(a / h)  # first grid line at or above 0
    return [0.0, bx, line0 - 0.5 * h, line0 - 0.5 * h + by, line0 - 0.5 * h, line0 - 0.5 * h + bz]


def sc_types(xyz, nb, radius, nneighbors=18):
    """Types: top/bottom layers, full-neighbour interior, and the two pins."""
    n = xyz.shape[0]
    t = np.full(n, T_INTERIOR, dtype=np.int32)
    zmax, zmin = xyz[:, 2].max(), xyz[:, 2].min()
    top = xyz[:, 2] >= zmax - 1.2 * radius
    bot = xyz[:, 2] <= zmin + 1.2 * radius
    t[top] = T_TOP
    t[bot] = T_BOTTOM
    t[nb == nneighbors] = T_FULL
    bidx = np.nonzero(bot)[0]
    p1 = bidx[np.lexsort((xyz[bidx, 0], xyz[bidx, 1]))[0]]          # min y, then min x
    cand = bidx[np.isclose(xyz[bidx, 1], xyz[p1, 1])]
    p2 = cand[np.argmax(xyz[cand, 0])]                               # same row, max x
    t[p1] = T_PIN_XY
    t[p2] = T_PIN_Y
    return t


def sc_bcs(step_z):
    """Per-step BCs: bottom z fixed, pins, top z displaced by step_z."""
    return [(T_BOTTOM, "z", 0.0), (T_PIN_XY, "x", 0.0), (T_PIN_XY, "y", 0.0),
            (T_PIN_XY, "z", 0.0), (T_PIN_Y, "y", 0.0), (T_PIN_Y, "z", 0.0),
            (T_TOP, "z", step_z)]


def sc_force_bcs(fx, fz):
    """Force-controlled variant (setForceBC, src/boundary.c:50-70): bottom z
    fixed and the pins as in sc_bcs; the top layer carries the per-step force
    increment (fx, 0, fz), shared equally by its particles.
    Returns (displacement BCs, force BCs)."""
    disp = [(T_BOTTOM, "z", 0.0), (T_PIN_XY, "x", 0.0), (T_PIN_XY, "y", 0.0),
            (T_PIN_XY, "z", 0.0), (T_PIN_Y, "y", 0.0), (T_PIN_Y, "z", 0.0)]
    return disp, [(T_TOP, fx, 0.0, fz)]


class ForceCase:
    """SC J2 specimen nx x ny x nz under a top-face force ramp: `steps` equal
    increments of (fx, 0, fz) N.  Yield starts at step 4; the reference's
    modified Newton converges through step 8 (96 iterations there) and not
    beyond, where the force approaches the specimen's limit load."""

    def __init__(self, nx=6, ny=6, nz=8, radius=0.1, E=200e3, nu=0.3, sigmay=150.0, H=2000.0,
                 fz=20.0, fx=2.0, steps=8, newton_tol=1e-8):
        self.lattice, self.radius = 2, radius
        self.box = sc_box(nx, ny, nz, radius)
        self.E, self.nu, self.sigmay, self.H = E, nu, sigmay, H
        self.fz, self.fx, self.steps = fz, fx, steps
        self.newton_tol = newton_tol
        self.e_noise, self.seed = 0.0, 1

    def ce_per_type(self):
        return np.tile(iso_cubic(self.E, self.nu), (NTYPE, 1))

    def bcs(self):
        return sc_force_bcs(self.fx, self.fz)


class DuctileDamageCase:
    """J2 with the reference main's ductile nonlocal damage
    (updateDuctileDamagePwiseNonlocal): SC 8^3 in z tension, yield stress
    400 MPa except 60 MPa within 0.25 mm of the centre, nonlocal length
    0.15 mm, damage threshold 1e-3.  Damage accumulates around the weak zone
    from step 1; step 6 breaks the first bonds (one re-solve pass), step 7
    cascades over several passes."""

    def __init__(self, n=8, radius=0.1, E=200e3, nu=0.3, H=2000.0, inc=0.0005, steps=7,
                 L=0.15, threshold=1e-3, newton_tol=1e-8):
        self.n, self.radius, self.lattice = n, radius, 2
        self.box = sc_box(n, n, n, radius)
        self.E, self.nu, self.H = E, nu, H
        self.schedule = [inc] * steps
        self.L, self.threshold = L, threshold
        self.newton_tol = newton_tol
        self.e_noise, self.seed = 0.0, 1

    def sigmay(self, xyz0):
        c = xyz0.mean(axis=0)
        return np.where(np.linalg.norm(xyz0 - c, axis=1) < 0.25, 60.0, 400.0)

    def ce_per_type(self):
        return np.tile(iso_cubic(self.E, self.nu), (NTYPE, 1))


T_PATCH = 6  # a loaded patch of the top face (brittle case)


class BrittleCase:
    """Elastic SC 8^3 with the reference's brittle bond breaking
    (updateBrittleDamage): only a 3 x 3 corner patch of the top face is
    pulled along z (type T_PATCH), the rest of the top is free; bonds break
    at an elastic bond strain of 2e-3, at most 6 per pass.  Breaking starts at
    step 3 and spreads under the patch, with up to 11 passes per step."""

    def __init__(self, n=8, radius=0.1, E=200e3, nu=0.3, inc=0.0004, steps=12, crit=2e-3, nbreak=6,
                 newton_tol=1e-8):
        self.n, self.radius, self.lattice = n, radius, 2
        self.box = sc_box(n, n, n, radius)
        self.E, self.nu = E, nu
        self.schedule = [inc] * steps
        self.crit, self.nbreak = crit, nbreak
        self.newton_tol = newton_tol

    def types(self, xyz0, nb):
        t = sc_types(xyz0, nb, self.radius)
        patch = (t == T_TOP) & (xyz0[:, 0] < 0.5) & (xyz0[:, 1] < 0.5)
        t[patch] = T_PATCH
        return t

    def bcs(self, inc):
        return [b for b in sc_bcs(0.0) if b[0] != T_TOP] + [(T_PATCH, "z", inc)]


# Setup-only shapes (lattice, radius, box) whose bond lists, AFEM
# connectivity and CSR pattern are pinned against the reference: the 20^3
# SC cube, a ragged SC box and a ragged FCC box.
SETUP_SHAPES = {
    "sc20": (2, 0.1, sc_box(20, 20, 20, 0.1)),
    "sc7x3x11": (2, 0.1, sc_box_exact(7, 3, 11, 0.1)),
    "fcc_ragged": (3, 0.1, [-0.07, 1.2, -0.07, 0.5, -0.07, 0.9]),
}


def cyclic_schedule(amplitude, steps_per_quarter, cycles):
    """Increments 0->+A->0->-A->0 per cycle, steps_per_quarter equal steps each."""
    inc = amplitude / steps_per_quarter
    one = [inc] * steps_per_quarter + [-inc] * (2 * steps_per_quarter) + [inc] * steps_per_quarter
    return one * cycles


class SCCase:
    """SC elastoplastic cyclic case (C1 at n=10, C2 at n=100)."""

    def __init__(self, n=10, radius=0.1, E=200e3, nu=0.3, sigmay=250.0, H=2000.0,
                 strain=0.002, steps_per_quarter=20, cycles=2, newton_tol=1e-8,
                 e_noise=0.0, seed=1, xi=0.0):
        self.n = n
        self.xi = xi  # kinematic share of the linear hardening (J2_xi)
        self.radius = radius
        self.lattice = 2
        self.box = sc_box(n, n, n, radius)
        self.E, self.nu, self.sigmay, self.H = E, nu, sigmay, H
        self.height = (n - 1) * 2.0 * radius
        self.schedule = cyclic_schedule(strain * self.height, steps_per_quarter, cycles)
        self.newton_tol = newton_tol
        self.e_noise = e_noise
        self.seed = seed

    def ce_per_type(self):
        return np.tile(iso_cubic(self.E, self.nu), (NTYPE, 1))


def sigmay_field(n, seed=3):
    """Per-particle yield stress 200 + 200 U[0, 1) MPa (splitmix64, seed 3)."""
    return 200.0 + 200.0 * splitmix64_uniform(seed, n)


def splitmix64_uniform(seed, count):
    """Counter-based uniform doubles in [0,1): splitmix64(seed*2^32 + k) >> 11 * 2^-53."""
    out = np.empty(count, dtype=np.float64)
    mask = (1 << 64) - 1
    for k in range(count):
        z = ((seed << 32) + k + 0x9E3779B97F4A7C15) & mask
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & mask
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & mask
        z = z ^ (z >> 31)
        out[k] = (z >> 11) * (1.0 / 9007199254740992.0)
    return out


def fcc_box(ncell, radius):
    """Box for createCuboid (lattice 3) holding ncell^3 FCC cells of edge 2*sqrt(2)*radius.

    FCC sites start at -|box diagonal| on all axes (src/initialization.c:359-415);
    the box is widened by a quarter cell on each side so it captures the sites
    of exactly ncell cells plus their closing faces whatever the offset."""
    a = 4 * radius / np.sqrt(2.0)
    return [-0.25 * a, ncell * a + 0.25 * a] * 3


class FCCCase:
    """FCC single crystal, crystal plasticity, [001] tension (C3 at ncell=80)."""

    def __init__(self, ncell=4, radius=0.1, strain=0.02, steps=100, newton_tol=1e-8,
                 tau0=50.0, h0=500.0, p=20.0, q=1.0, eta=10.0, maxloop=10, dtime=1.0, taus=1e30):
        self.lattice = 3
        self.radius = radius
        self.box = fcc_box(ncell, radius)
        # Al constants (examples/FCC_Al_R0.3_001_tension.c:200-202)
        self.C11, self.C12, self.C44 = 107.3e3, 60.8e3, 28.3e3
        # linear hardening by default: taus -> infinity makes h = h0
        # (src/constitutive.c:1125-1126); a finite taus saturates it
        self.cp = [tau0, taus, h0, p, q, eta, maxloop, dtime]
        self.height = ncell * 4 * radius / np.sqrt(2.0)
        self.schedule = [strain * self.height / steps] * steps
        self.newton_tol = newton_tol

    def ce_per_type(self):
        return np.tile([self.C11, self.C12, self.C44], (NTYPE, 1))


# Saturating, latent-hardening, more rate-sensitive crystal plasticity: the
# hardening modulus h0 / cosh^2(h0 A / (taus - tau0)) of
# src/constitutive.c:1124-1125 falls from h0 towards zero as the accumulated
# slip A grows (with taus -> infinity it stays h0), and latent hardening
# ratio q = 1.4.
FCC_SAT = dict(tau0=50.0, taus=150.0, h0=500.0, p=20.0, q=1.2)


# J2 plasticity on the FCC lattice (plmode 0 on lattice 3)
FCC_J2 = dict(sigmay=100.0, H=1000.0)


class BatchCase:
    """Batch of independent SC specimens of uneven size (C4 at nspec=256,
    edges 20..60): each edge drawn independently from U{lo..hi}, per-specimen
    E ~ U[180e3, 220e3], yield ~ U[200, 400], H = 2000; monotonic tension to
    `strain` over `steps` equal steps (top layer displaced along z)."""

    def __init__(self, nspec=256, edge_lo=20, edge_hi=60, radius=0.1, nu=0.3, H=2000.0,
                 strain=0.01, steps=50, newton_tol=1e-8, seed=1):
        self.nspec, self.radius, self.lattice = nspec, radius, 2
        u = splitmix64_uniform(seed, 3 * nspec).reshape(nspec, 3)
        self.edges = (edge_lo + np.floor(u * (edge_hi - edge_lo + 1))).astype(int)
        self.E = 180e3 + 40e3 * splitmix64_uniform(seed + 1, nspec)
        self.sigmay = 200.0 + 200.0 * splitmix64_uniform(seed + 2, nspec)
        self.nu, self.H = nu, H
        self.boxes = np.array([sc_box_exact(nx, ny, nz, radius) for nx, ny, nz in self.edges])
        self.heights = (self.edges[:, 2] - 1) * 2.0 * radius
        self.strain, self.steps = strain, steps
        self.newton_tol = newton_tol

    def particles(self):
        return int(np.prod(self.edges, axis=1).sum())

    def step_bcs(self):
        """Per-specimen BC lists of one load step."""
        return [sc_bcs(self.strain * h / self.steps) for h in self.heights]


def splitmix64_uniform_np(seed, count):
    """Vectorised splitmix64_uniform (same values)."""
    k = np.arange(count, dtype=np.uint64)
    with np.errstate(over="ignore"):
        z = np.uint64((seed << 32) & ((1 << 64) - 1)) + k + np.uint64(0x9E3779B97F4A7C15)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        z = z ^ (z >> np.uint64(31))
    return (z >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)


def gaussian_filter3(a, sigma):
    """Separable Gaussian filter (truncated at 4 sigma, reflected edges)."""
    r = int(4 * sigma + 0.5)
    x = np.arange(-r, r + 1, dtype=np.float64)
    k = np.exp(-0.5 * (x / sigma) ** 2)
    k /= k.sum()
    out = a
    for ax in range(3):
        pad = [(0, 0)] * 3
        pad[ax] = (r, r)
        p = np.pad(out, pad, mode="reflect")
        acc = np.zeros_like(out)
        for t in range(2 * r + 1):
            sl = [slice(None)] * 3
            sl[ax] = slice(t, t + out.shape[ax])
            acc += k[t] * p[tuple(sl)]
        out = acc
    return out


class NotchedPlate:
    """SC notched plate (C5 at 200 x 10 x 200): loading along z, thickness
    along y; a single-edge notch one particle layer wide at mid-height, cut
    from the x = 0 edge `notch` particles deep through the thickness.
    Per-particle E, nu, yield stress and H are smooth random fields
    (Gaussian-filtered white noise, correlation length `corr` particles,
    min-max scaled to +-amp about 200 GPa / 0.3 / 250 MPa / 2 GPa)."""

    BASE = (200e3, 0.3, 250.0, 2000.0)

    def __init__(self, nx=200, ny=10, nz=200, notch=40, radius=0.1, steps=60, strain=0.01, corr=10.0, amp=0.1,
                 newton_tol=1e-8):
        self.nx, self.ny, self.nz, self.notch = nx, ny, nz, notch
        self.radius, self.lattice = radius, 2
        h = 2.0 * radius
        iz, iy, ix = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
        keep = ~((iz == nz // 2) & (ix < notch))
        self.grid = np.stack([ix[keep], iy[keep], iz[keep]], axis=1)
        self.xyz = self.grid.astype(np.float64) * h
        self.height = (nz - 1) * h
        self.steps, self.strain = steps, strain
        self.schedule = [strain * self.height / steps] * steps
        self.corr, self.amp = corr, amp
        self.newton_tol = newton_tol

    @property
    def n(self):
        return self.xyz.shape[0]

    def fields(self, seed):
        """E, nu, sigmay, H per particle for a seed."""
        out = []
        for k, base in enumerate(self.BASE):
            w = splitmix64_uniform_np(seed * 16 + k, self.nx * self.ny * self.nz) - 0.5
            g = gaussian_filter3(w.reshape(self.nz, self.ny, self.nx), self.corr)
            g = 2.0 * (g - g.min()) / (g.max() - g.min()) - 1.0
            v = g[self.grid[:, 2], self.grid[:, 1], self.grid[:, 0]]
            out.append(base * (1.0 + self.amp * v))
        return out

    def step_bcs(self):
        return [sc_bcs(s) for s in self.schedule]
