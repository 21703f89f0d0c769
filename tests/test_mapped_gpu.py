"""Page-locked host buffers (the fast path of the copy engines, read
asynchronously): uploads and read-outs give the same bits as pageable
buffers; a caller may overwrite its buffer as soon as an upload returns
(batch members: after pfa_batch_sync); the asynchronous upload and
read-out keep stream order on a handle and across two alternating handles.
Also the FP64-free split of the layout conversion against the FP64
expression it replaces."""
import numpy as np
import pytest

from pfa_gb300 import ic

pytestmark = pytest.mark.gpu


def _pinned_like(arrays):
    import torch
    out = []
    for a in arrays:
        h = torch.empty(a.shape, dtype=torch.float64, pin_memory=True).numpy()
        h[...] = a
        out.append(h)
    return out


def _same(a, b):
    return all(np.array_equal(x, y) for x, y in zip(a, b))


@pytest.mark.parametrize("precision", ["fp32", "fp32k"])
def test_grid2d_mapped_upload_and_read(pfa, precision):
    f = ic.grid2d(130, 77, seed=4, stripe_width=16, n_particles=2, radius=5.0)
    g = ic.grid2d(130, 77, seed=5, stripe_width=16, n_particles=2, radius=5.0)
    p = pfa.model_params()
    runs = []
    for pin in (False, True):
        grid = pfa.Grid2D(f, p, precision=precision)
        grid.run(30)
        src = _pinned_like(g) if pin else [a.copy() for a in g]
        grid.upload(src)
        for a in src:
            a[...] = -1.0  # the upload has finished reading
        grid.run(40)
        out = _pinned_like(g) if pin else [np.empty_like(a) for a in g]
        grid.read(out)
        runs.append([np.array(a) for a in out])
        grid.close()
    assert _same(runs[0], runs[1])
    # an upload (row bands, conversion overlapped with the copies) leaves the
    # same state as creating the grid from those fields
    fresh = pfa.Grid2D(g, p, precision=precision)
    fresh.run(40)
    assert _same(fresh.read(), runs[0])
    fresh.close()


def test_batch_mapped_add_and_read(pfa):
    fields = [ic.grid2d(n, m, seed=n, stripe_width=8, n_particles=2, radius=4.0)
              for n, m in ((64, 40), (33, 90))]
    runs = []
    for pin in (False, True):
        b = pfa.Batch(pfa.model_params(), 1 << 26)
        slots = []
        for f in fields:
            src = _pinned_like(f) if pin else [a.copy() for a in f]
            slots.append(b.add(src))
            b.sync()  # page-locked sources are read asynchronously until then
            for a in src:
                a[...] = -1.0
        b.run(25)
        res = []
        for s, f in zip(slots, fields):
            out = _pinned_like(f) if pin else [np.empty_like(a) for a in f]
            b.read(s, out)
            res.append([np.array(a) for a in out])
        runs.append(res)
        b.close()
    for x, y in zip(*runs):
        assert _same(x, y)


def test_grid3d_mapped_upload_and_read(pfa):
    f = ic.grid3d(22, 18, 14, seed=6, slab=5, n_particles=2, radius=3.0)
    p = pfa.model_params(dim=3)
    runs = []
    for pin in (False, True):
        g = pfa.Grid3D(f, p, precision="fp32")
        g.run(5)
        src = _pinned_like(f) if pin else [a.copy() for a in f]
        g.upload(src)
        for a in src:
            a[...] = -1.0
        g.run(12)
        out = _pinned_like(f) if pin else [np.empty_like(a) for a in f]
        g.read(out)
        runs.append([np.array(a) for a in out])
        g.close()
    assert _same(runs[0], runs[1])


def test_split_matches_the_fp64_expression(pfa):
    """The import kernels' FP64-free split equals hi = float(v),
    c = float(double(hi) - v) bit-for-bit: random values over the whole
    double range, both signs, and the rounding ties and edges."""
    rng = np.random.default_rng(7)
    bits = rng.integers(0, 1 << 63, 200000, dtype=np.int64).view(np.float64)
    typical = np.concatenate([rng.uniform(-1.5, 1.5, 100000), rng.uniform(0, 1e-3, 50000)])
    ties = []
    for e in (950, 951, 1000, 1022, 1023, 1148, 1149, 1150, 949):
        for low in (0, 1, (1 << 28) - 1, 1 << 28, (1 << 28) + 1, (1 << 29) - 1):
            for top in (0, 1, (1 << 23) - 1):
                ties.append((e << 52) | (top << 29) | low)
    ties = np.array(ties, dtype=np.int64).view(np.float64)
    special = np.array([0.0, -0.0, 5e-324, -5e-324, 1e-300, 1e300, np.inf, -np.inf,
                        3.4028234663852886e38, 1.1754943508222875e-38, 1e-22, 2.0 ** -74])
    v = np.concatenate([bits, typical, ties, -ties, special])
    v = v[~np.isnan(v)]
    hi, c = pfa.split_device(v)
    with np.errstate(over="ignore", invalid="ignore"):
        want_hi = v.astype(np.float32)
        want_c = (want_hi.astype(np.float64) - v).astype(np.float32)
    assert np.array_equal(hi.view(np.uint32), want_hi.view(np.uint32))
    ok = np.isfinite(want_c)
    assert np.array_equal(c[ok].view(np.uint32), want_c[ok].view(np.uint32))


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_async_read_then_upload_keeps_order(pfa, precision):
    """A read-out enqueued without waiting, then an upload and steps on the
    same handle: the read-out still returns the state before the upload
    (the upload waits for its copies), and the steps run on the uploaded
    fields."""
    f = ic.grid2d(150, 97, seed=6, stripe_width=20, n_particles=2, radius=5.0)
    g = ic.grid2d(150, 97, seed=7, stripe_width=20, n_particles=2, radius=5.0)
    p = pfa.model_params()
    ref = pfa.Grid2D(f, p, precision=precision)
    ref.run(20)
    want_read = ref.read()
    ref.upload(g)
    ref.run(15)
    want_end = ref.read()
    ref.close()
    grid = pfa.Grid2D(f, p, precision=precision)
    grid.run(20)
    out = _pinned_like([np.zeros_like(a) for a in f])
    src = _pinned_like(g)
    grid.read(out, wait=False)
    grid.upload(src, wait=False)
    grid.run(15)
    grid.sync()
    assert _same(out, want_read)
    assert _same(grid.read(), want_end)
    grid.close()


def test_two_handles_pipelined_jobs_match_serial(pfa):
    """Independent jobs on two alternating handles with asynchronous
    transfers (job k+1's upload and job k-1's read-out overlap job k's
    steps): every job's result is the one a serial upload / run / read gives."""
    p = pfa.model_params()
    jobs = [ic.grid2d(256, 192, seed=s, stripes=[40, 150], stripe_width=24, n_particles=3,
                      radius=6.0) for s in range(5)]
    want = []
    g = pfa.Grid2D(jobs[0], p, precision="fp32")
    for f in jobs:
        g.upload(f)
        g.run(40)
        want.append(g.read())
    g.close()
    host_in = [_pinned_like(f) for f in jobs]
    host_out = [_pinned_like([np.zeros_like(a) for a in f]) for f in jobs]
    h = [pfa.Grid2D(jobs[0], p, precision="fp32"), pfa.Grid2D(jobs[0], p, precision="fp32")]
    h[0].upload(host_in[0], wait=False)
    for k in range(len(jobs)):
        d, o = h[k % 2], h[(k + 1) % 2]
        if k + 1 < len(jobs):
            o.upload(host_in[k + 1], wait=False)
        d.run(40)
        d.read(host_out[k], wait=False)
    for x in h:
        x.sync()
        x.close()
    for k in range(len(jobs)):
        assert _same(host_out[k], want[k]), k
