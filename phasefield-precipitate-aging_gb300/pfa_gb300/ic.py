"""Seeded synthetic initial conditions for the benchmark configurations.

The reference generates its initial grids with MMSP (src/alloy625.cpp:520-739);
the workloads here are specified by composition, stripe and particle recipes,
so these generators produce them directly as numpy arrays in the reference's
halo layout: shape (Ny + 2, Nx + 2) in 2D and (Nz + 2, Ny + 2, Nx + 2) in 3D,
with the one-cell ghost ring filled by the zero-flux mirror.

Particles follow the reference's embedding recipe (embed_OPC,
src/alloy625.cpp:262-294): phi = 0.5 - 0.5 tanh(z / (w/2)) with
z = dx (r - R) (tanh_interp, thermo/nucleation.c:12-16), and the composition
is blended toward the precipitate's equilibrium composition by p(phi).
"""
import numpy as np

# equilibrium compositions, thermo/parabola625.c:65-117
XE = {"gam": (0.52421634830562147, 0.01299272922003303),
      "del": (0.022966218927631978, 0.24984563695705883),
      "lav": (0.37392129441013022, 0.25826261799015571)}

MATRIX = (0.3041, 0.0235)
ENRICH = (0.2720, 0.1692)
MATRIX_RANGE = ((0.2794, 0.3288), (0.0202, 0.0269))
ENRICH_RANGE = ((0.2473, 0.2967), (0.1659, 0.1726))


def p(x):
    return x ** 3 * (6.0 * x ** 2 - 15.0 * x + 10.0)


def mirror_halo(a):
    """Fill the ghost ring with the adjacent interior values (in place)."""
    if a.ndim == 2:
        a[:, 0] = a[:, 1]
        a[:, -1] = a[:, -2]
        a[0, :] = a[1, :]
        a[-1, :] = a[-2, :]
    else:
        a[:, :, 0] = a[:, :, 1]
        a[:, :, -1] = a[:, :, -2]
        a[:, 0, :] = a[:, 1, :]
        a[:, -1, :] = a[:, -2, :]
        a[0] = a[1]
        a[-1] = a[-2]
    return a


def _embed(fields, centre, radius, phase, dx, width, grid_shape):
    """Blend one particle (circle / sphere) into the interior fields."""
    xcr, xnb, phd, phl = fields
    pad = int(np.ceil(radius + 6 * (width / 2) / dx)) + 1
    sl = []
    coords = []
    for d, (c, n) in enumerate(zip(centre, grid_shape)):
        lo = max(0, int(np.floor(c)) - pad)
        hi = min(n, int(np.floor(c)) + pad + 1)
        sl.append(slice(lo, hi))
        coords.append(np.arange(lo, hi, dtype=np.float64) - c)
    mesh = np.meshgrid(*coords, indexing="ij")
    r = np.sqrt(sum(m * m for m in mesh))
    z = dx * (r - radius)
    phi = 0.5 - 0.5 * np.tanh(z / (width / 2))
    pp = p(phi)
    sl = tuple(sl)
    xe = XE["del"] if phase == 0 else XE["lav"]
    target = phd if phase == 0 else phl
    xcr[sl] = pp * xe[0] + (1.0 - pp) * xcr[sl]
    xnb[sl] = pp * xe[1] + (1.0 - pp) * xnb[sl]
    target[sl] = np.maximum(target[sl], phi)


def _centres(rng, n, extent, radius, width_cells):
    """n seeded centres inside `extent`, at least two radii plus three
    interface widths apart so that no two particles overlap (a cell inside
    both a delta and a laves particle has p_gamma < 0, which the model does
    not describe).  Returns fewer centres if the domain is too crowded."""
    extent = np.asarray(extent, dtype=np.float64)
    dmin = 2.0 * radius + 3.0 * width_cells
    out = []
    tries = 0
    while len(out) < n and tries < 200 * max(n, 1):
        tries += 1
        c = rng.uniform(0.0, 1.0, len(extent)) * (extent - 1)
        if all(np.sqrt(np.sum((c - o) ** 2)) >= dmin for o in out):
            out.append(c)
    return np.array(out).reshape(len(out), len(extent))


def grid2d(nx, ny, seed, matrix=MATRIX, enrich=ENRICH, noise=0.002, stripes=None,
           stripe_width=64, n_particles=4, radius=8.0, dx=5e-9, width=10e-9):
    """2D initial condition (interior nx x ny cells), returned with its halo.

    stripes: list of stripe start columns (interior coordinates), or None for
    one stripe centred in x.  Stripes run along y.  Particles alternate
    delta / laves and sit at seeded positions.
    """
    rng = np.random.default_rng(seed)
    shape = (ny, nx)
    xcr = np.full(shape, matrix[0]) + rng.uniform(-noise, noise, shape)
    xnb = np.full(shape, matrix[1]) + rng.uniform(-noise, noise, shape)
    if stripes is None:
        stripes = [nx // 2 - stripe_width // 2]
    for s in stripes:
        lo, hi = max(0, s), min(nx, s + stripe_width)
        xcr[:, lo:hi] += enrich[0] - matrix[0]
        xnb[:, lo:hi] += enrich[1] - matrix[1]
    phd = np.zeros(shape)
    phl = np.zeros(shape)
    centres = _centres(rng, n_particles, (ny, nx), radius, width / dx)
    for k in range(len(centres)):
        _embed((xcr, xnb, phd, phl), centres[k], radius, k % 2, dx, width, shape)
    out = []
    for a in (xcr, xnb, phd, phl):
        h = np.empty((ny + 2, nx + 2))
        h[1:-1, 1:-1] = a
        out.append(mirror_halo(h))
    return out


def grid3d(nx, ny, nz, seed, matrix=MATRIX, enrich=ENRICH, noise=0.002, slab=64,
           n_particles=32, radius=6.0, dx=5e-9, width=10e-9, dtype=np.float64):
    """3D initial condition: matrix + noise, one seeded enriched slab (normal
    to x) and seeded spherical particles alternating delta / laves."""
    rng = np.random.default_rng(seed)
    shape = (nz, ny, nx)
    xcr = np.full(shape, matrix[0]) + rng.uniform(-noise, noise, shape)
    xnb = np.full(shape, matrix[1]) + rng.uniform(-noise, noise, shape)
    s = int(rng.integers(0, max(1, nx - slab)))
    xcr[:, :, s:s + slab] += enrich[0] - matrix[0]
    xnb[:, :, s:s + slab] += enrich[1] - matrix[1]
    phd = np.zeros(shape)
    phl = np.zeros(shape)
    centres = _centres(rng, n_particles, (nz, ny, nx), radius, width / dx)
    for k in range(len(centres)):
        _embed((xcr, xnb, phd, phl), centres[k], radius, k % 2, dx, width, shape)
    out = []
    for a in (xcr, xnb, phd, phl):
        h = np.empty((nz + 2, ny + 2, nx + 2), dtype=dtype)
        h[1:-1, 1:-1, 1:-1] = a
        out.append(mirror_halo(h))
    return out


def config1(seed=1):
    """256 x 256, one central stripe 64 wide, 4 particles R = 8."""
    return grid2d(256, 256, seed)


def config2(seed=2, n=4096, n_particles=4):
    """4096 x 4096 with config1's recipe (4 particles R = 8) and 16 stripes
    64 wide at seeded columns; n_particles=64 gives the denser variant."""
    rng = np.random.default_rng(seed + 1000)
    stripes = sorted(int(v) for v in rng.integers(0, n - 64, 16))
    return grid2d(n, n, seed, stripes=stripes, n_particles=n_particles)


def batch_sides(count=64, seed=3, lo=128, hi=2048):
    """Side lengths log-uniform in [lo, hi] (seeded)."""
    rng = np.random.default_rng(seed)
    return [int(round(float(np.exp(v)))) for v in rng.uniform(np.log(lo), np.log(hi), count)]


def batch_grid(side, seed):
    """One batched-workload grid: compositions drawn from the matrix and
    enrichment ranges, a central stripe a quarter of the width, 4 particles."""
    rng = np.random.default_rng(seed)
    m = (rng.uniform(*MATRIX_RANGE[0]), rng.uniform(*MATRIX_RANGE[1]))
    e = (rng.uniform(*ENRICH_RANGE[0]), rng.uniform(*ENRICH_RANGE[1]))
    return grid2d(side, side, seed + 7, matrix=m, enrich=e,
                  stripe_width=max(4, min(64, side // 4)), n_particles=4)


# ---- recipes: the same kinds of grid, built on the device (pfa_ic_recipe) ----

def recipe2d(nx, ny, seed, matrix=MATRIX, enrich=ENRICH, noise=0.002, stripes=None,
             stripe_width=64, n_particles=4, radius=8.0, dx=5e-9, width=10e-9):
    """Recipe of a 2D grid like grid2d's: noise from the device's Philox
    stream (keyed by seed), stripes along y, particles at seeded centres
    alternating delta / laves."""
    rng = np.random.default_rng(seed)
    if stripes is None:
        stripes = [nx // 2 - stripe_width // 2]
    bands = [(max(0, s), min(nx, s + stripe_width)) for s in stripes]
    centres = _centres(rng, n_particles, (ny, nx), radius, width / dx)
    parts = [(float(c[1]), float(c[0]), 0.0, float(radius), k % 2) for k, c in enumerate(centres)]
    return {"nx": nx, "ny": ny, "nz": 0, "matrix": tuple(matrix), "enrich": tuple(enrich),
            "noise": noise, "seed": int(seed), "bands": bands, "particles": parts,
            "dx": dx, "width": width}


def recipe3d(nx, ny, nz, seed, matrix=MATRIX, enrich=ENRICH, noise=0.002, slab=64,
             n_particles=32, radius=6.0, dx=5e-9, width=10e-9):
    """Recipe of a 3D grid like grid3d's: one seeded enriched slab normal to
    x, seeded spheres alternating delta / laves."""
    rng = np.random.default_rng(seed)
    s = int(rng.integers(0, max(1, nx - slab)))
    centres = _centres(rng, n_particles, (nz, ny, nx), radius, width / dx)
    parts = [(float(c[2]), float(c[1]), float(c[0]), float(radius), k % 2)
             for k, c in enumerate(centres)]
    return {"nx": nx, "ny": ny, "nz": nz, "matrix": tuple(matrix), "enrich": tuple(enrich),
            "noise": noise, "seed": int(seed), "bands": [(s, min(nx, s + slab))],
            "particles": parts, "dx": dx, "width": width}


def reference_recipe2d(nx, ny, seed, radius=8.0, matrix=None, enrich=None, dx=5e-9,
                       width=10e-9):
    """The reference's default 2D initial condition as a recipe
    (src/alloy625.cpp:520-600): matrix and enrichment compositions drawn from
    the alloy ranges (here with numpy's generator, seeded), the bell-curve
    enrichment of init_gaussian_enrichment along x (widths bell = 150, 50 nm,
    src/parameters.h:32; mean over the middle two thirds = the matrix), no
    noise, and one delta seed embedded at the centre with embed_OPC's box and
    overwrite (seed_solitaire_delta).  The reference sizes the seed from the
    critical radius (2 x R* / dx) and blends toward the curvature-shifted
    delta composition; here the radius in cells is an argument and the blend
    goes to the flat equilibrium composition (as seed_pair's does)."""
    rng = np.random.default_rng(seed)
    m = matrix or (rng.uniform(*MATRIX_RANGE[0]), rng.uniform(*MATRIX_RANGE[1]))
    e = enrich or (rng.uniform(*ENRICH_RANGE[0]), rng.uniform(*ENRICH_RANGE[1]))
    return {"nx": nx, "ny": ny, "nz": 0, "matrix": tuple(m), "enrich": tuple(e), "noise": 0.0,
            "seed": int(seed), "bands": [], "dx": dx, "width": width,
            "particles": [(float(nx // 2), float(ny // 2), 0.0, float(radius), 0)],
            "profile": 1, "bell_sigma": (150e-9, 50e-9),
            "bell_range": (-nx * dx / 3.0, nx * dx / 3.0), "bell_x0": float(nx // 2),
            "particle_mode": 1}


# request sizes of the serving workload: (dimension, side)
SERVE_SIZES = ((2, 256), (2, 1024), (2, 4096), (3, 128), (3, 256))


def serve_trace(count=24, seed=5, rate=20.0, steps=(2000, 20000)):
    """Seeded request trace: Poisson arrivals at `rate` per second, sizes
    uniform over SERVE_SIZES, step counts uniform in `steps` (inclusive)."""
    rng = np.random.default_rng(seed)
    arrivals = np.cumsum(rng.exponential(1.0 / rate, count))
    out = []
    for k in range(count):
        dim, side = SERVE_SIZES[int(rng.integers(len(SERVE_SIZES)))]
        out.append({"rid": k, "dim": dim, "side": side, "arrival": float(arrivals[k]),
                    "steps": int(rng.integers(steps[0], steps[1] + 1)),
                    "seed": seed * 1000 + k})
    return out


def serve_fields(item):
    """Initial condition of one trace request: compositions drawn from the
    matrix and enrichment ranges, a stripe (2D) or slab (3D), particles."""
    rng = np.random.default_rng(item["seed"])
    m = (rng.uniform(*MATRIX_RANGE[0]), rng.uniform(*MATRIX_RANGE[1]))
    e = (rng.uniform(*ENRICH_RANGE[0]), rng.uniform(*ENRICH_RANGE[1]))
    s = item["side"]
    if item["dim"] == 2:
        return grid2d(s, s, item["seed"] + 7, matrix=m, enrich=e,
                      stripe_width=max(4, min(64, s // 4)), n_particles=4)
    return grid3d(s, s, s, item["seed"] + 7, matrix=m, enrich=e, slab=max(4, s // 8),
                  n_particles=8, radius=6.0)


def serve_recipe(item):
    """serve_fields' request as a recipe the device builds (same composition
    draws, stripe / slab and particle counts)."""
    rng = np.random.default_rng(item["seed"])
    m = (rng.uniform(*MATRIX_RANGE[0]), rng.uniform(*MATRIX_RANGE[1]))
    e = (rng.uniform(*ENRICH_RANGE[0]), rng.uniform(*ENRICH_RANGE[1]))
    s = item["side"]
    if item["dim"] == 2:
        return recipe2d(s, s, item["seed"] + 7, matrix=m, enrich=e,
                        stripe_width=max(4, min(64, s // 4)), n_particles=4)
    return recipe3d(s, s, s, item["seed"] + 7, matrix=m, enrich=e, slab=max(4, s // 8),
                    n_particles=8, radius=6.0)
