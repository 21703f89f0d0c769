"""Initial conditions built on the device from a recipe, against the
oracle's evaluation of the same recipe: exact where no particle reaches
(noise stream, bands, ghost ring), within FP64 rounding of tanh inside the
particles; through the raw entry point, a batch slot and a 3D handle; and a
served request built on the device equals the same request uploaded."""
import numpy as np
import pytest

from pfa_gb300 import ic

pytestmark = pytest.mark.gpu
TANH_TOL = 1e-14  # device tanh and p(phi) against the host's, values O(1)


def _outside(rec, shape):
    """Mask (with the ghost ring) of the cells no particle box reaches."""
    m = np.ones(shape, dtype=bool)
    is3d = len(shape) == 3
    for (x, y, z, R, _) in rec["particles"]:
        pad = int(np.ceil(R + 6 * (rec["width"] / 2) / rec["dx"])) + 1
        c = [x, y, z] if is3d else [x, y]
        sl = []
        for d, n in zip(c, reversed(shape)):
            f = int(np.floor(d))
            sl.append(slice(max(0, f - pad), min(n, f + pad + 3)))  # +1 ghost offset, +1 mirror
        m[tuple(reversed(sl))] = False
    return m


def _compare(got, want, rec, tol=TANH_TOL, exact=True):
    out = _outside(rec, want[0].shape)
    for g, w in zip(got, want):
        if exact:
            assert np.array_equal(g[out], w[out])
        assert np.max(np.abs(g - w)) <= tol


@pytest.mark.parametrize("dims", [2, 3])
def test_generate_into_device_arrays(pfa, dims):
    import torch
    import oracle as O
    rec = (ic.recipe2d(150, 97, seed=11, stripes=[3, 60, 140], stripe_width=16, n_particles=6,
                       radius=5.0) if dims == 2 else
           ic.recipe3d(45, 38, 29, seed=12, slab=9, n_particles=5, radius=4.0))
    want = O.ic_fields(rec)
    dev = [torch.full(want[0].shape, -1.0, dtype=torch.float64, device="cuda") for _ in range(4)]
    for call in range(2):  # the same recipe twice gives the same bits
        pfa.ic_generate(rec, [t.data_ptr() for t in dev])
        torch.cuda.synchronize()
        got = [t.cpu().numpy() for t in dev]
        _compare(got, want, rec)


@pytest.mark.parametrize("dims", [(1, 1, 0), (3, 2, 0), (1, 7, 0), (2, 1, 3), (1, 1, 2)])
def test_generate_tiny_grids(pfa, dims):
    """One-cell-wide grids: every interior cell writes several ghost cells."""
    import torch
    import oracle as O
    nx, ny, nz = dims
    rec = {"nx": nx, "ny": ny, "nz": nz, "matrix": (0.30, 0.02), "enrich": (0.27, 0.17),
           "noise": 0.002, "seed": 77, "bands": [(0, 1)],
           "particles": [(0.2, 0.4, 0.3, 1.5, 1)], "dx": 5e-9, "width": 10e-9}
    want = O.ic_fields(rec)
    dev = [torch.full(want[0].shape, -1.0, dtype=torch.float64, device="cuda") for _ in range(4)]
    pfa.ic_generate(rec, [t.data_ptr() for t in dev])
    torch.cuda.synchronize()
    for g, w in zip([t.cpu().numpy() for t in dev], want):
        assert np.max(np.abs(g - w)) <= TANH_TOL


@pytest.mark.parametrize("dims", [2, 3])
def test_reference_profile_and_embedding_on_device(pfa, dims):
    """The bell-curve profile and embed_OPC's box on the device against the
    oracle (exp and tanh to rounding; the amplitude comes from the host)."""
    import torch
    import oracle as O
    if dims == 2:
        rec = ic.reference_recipe2d(300, 50, seed=8, radius=5.0)
    else:
        rec = ic.recipe3d(40, 30, 24, seed=9, slab=6, n_particles=3, radius=3.0)
        rec.update(profile=1, bell_sigma=(60e-9, 30e-9), bell_range=(-40 * 5e-9 / 3, 40 * 5e-9 / 3),
                   bell_x0=20.0, particle_mode=1, bands=[])
    want = O.ic_fields(rec)
    dev = [torch.full(want[0].shape, -1.0, dtype=torch.float64, device="cuda") for _ in range(4)]
    pfa.ic_generate(rec, [t.data_ptr() for t in dev])
    torch.cuda.synchronize()
    for g, w in zip([t.cpu().numpy() for t in dev], want):
        assert np.max(np.abs(g - w)) <= TANH_TOL


def test_batch_slot_from_recipe(pfa):
    import oracle as O
    recs = [ic.recipe2d(n, m, seed=20 + n, stripe_width=8, n_particles=3, radius=4.0)
            for n, m in ((70, 50), (33, 129), (256, 40))]
    b = pfa.Batch(pfa.model_params(), 1 << 28)
    slots = [b.add_recipe(r) for r in recs]
    for r, s in zip(recs, slots):
        want = O.ic_fields(r)
        # the FP32 form keeps each value as hi - c with c a multiple of 2^-40
        # (compositions) or 2^-39 (phases)
        _compare(b.read(s), want, r, tol=2.0 ** -39 + TANH_TOL, exact=False)
    # stepping the device-built grids equals stepping the uploaded ones
    b2 = pfa.Batch(pfa.model_params(), 1 << 28)
    up = [b2.add(O.ic_fields(r)) for r in recs]
    b.run(60)
    b2.run(60)
    for s, u in zip(slots, up):
        for x, y in zip(b.read(s), b2.read(u)):
            assert np.max(np.abs(x - y)) <= 1e-12
    b.close()
    b2.close()


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_grid3d_from_recipe(pfa, precision):
    import oracle as O
    rec = ic.recipe3d(36, 30, 26, seed=31, slab=7, n_particles=4, radius=4.0)
    want = O.ic_fields(rec)
    g = pfa.Grid3D(None, pfa.model_params(dim=3), precision=precision, recipe=rec)
    tol = TANH_TOL if precision == "fp64" else 2.0 ** -39 + TANH_TOL
    got = g.read()
    inner = (slice(1, -1),) * 3
    for x, y in zip(got, want):
        assert np.max(np.abs(x[inner] - y[inner])) <= tol
    g.run(20)
    h = pfa.Grid3D(want, pfa.model_params(dim=3), precision=precision)
    h.run(20)
    for x, y in zip(g.read(), h.read()):
        assert np.max(np.abs(x[inner] - y[inner])) <= 1e-12
    g.close()
    h.close()


def test_served_recipe_equals_served_fields(pfa):
    import oracle as O
    from pfa_gb300.serve import GpuBackend, Request, Server
    recs = [ic.recipe2d(62, 40, seed=1, stripe_width=12, n_particles=2, radius=4.0),
            ic.recipe3d(20, 14, 12, seed=2, slab=6, n_particles=2, radius=3.0),
            ic.recipe2d(100, 33, seed=3, stripe_width=20, n_particles=2, radius=4.0)]
    steps = [120, 90, 75]

    def serve(reqs):
        be = GpuBackend(pfa, pfa.model_params(), pfa.model_params(dim=3), 1 << 28, 1 << 28)
        done = Server(be, tick_steps=50).run_trace(reqs, realtime=False)
        be.close()
        return {r.req.rid: r.result for r in done}

    a = serve([Request(k, None, n, recipe=r) for k, (r, n) in enumerate(zip(recs, steps))])
    b = serve([Request(k, O.ic_fields(r), n) for k, (r, n) in enumerate(zip(recs, steps))])
    for k in a:
        for x, y in zip(a[k], b[k]):
            assert np.max(np.abs(x - y)) <= 1e-12, k


def test_device_embedding_matches_reference_code(pfa):
    """The device's particles in embed_OPC's mode against embed_OPC's loop run
    with the reference's compiled tanh_interp, p and equilibrium compositions
    (tests/golden/ic_embed.npz): within device tanh / p rounding."""
    import torch
    from conftest import golden
    from golden.make_golden import IC_RECIPES
    g = golden("ic_embed.npz")
    for n, rec in enumerate(IC_RECIPES):
        shape = g[f"r{n}_cr"].shape
        dev = [torch.full(shape, -1.0, dtype=torch.float64, device="cuda") for _ in range(4)]
        pfa.ic_generate(rec, [t.data_ptr() for t in dev])
        torch.cuda.synchronize()
        for t, name in zip(dev, ("cr", "nb", "pd", "pl")):
            assert np.max(np.abs(t.cpu().numpy() - g[f"r{n}_{name}"])) <= TANH_TOL, (n, name)
