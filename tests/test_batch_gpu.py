"""Batches of 2D grids (one launch per step over all members).

A member of a batch must advance bit-for-bit as the same grid does alone in
a single-grid FP32 handle, whatever the other members, the launch shape and
the joins / leaves between runs; the arena refuses grids it has no room for.
"""
import numpy as np
import pytest

from pfa_gb300 import ic

pytestmark = pytest.mark.gpu

SHAPES = [(3, 3), (5, 7), (34, 66), (102, 39), (130, 130), (257, 64)]  # (ny, nx) with ring
GIB = 1 << 30


def _grids(seed0=0):
    out = []
    for k, (ny, nx) in enumerate(SHAPES):
        out.append(ic.grid2d(nx - 2, ny - 2, seed=seed0 + k, stripe_width=max(2, (nx - 2) // 4),
                             n_particles=2 if min(nx, ny) > 40 else 0, radius=4.0))
    return out


def _alone(pfa, f, p, steps):
    g = pfa.Grid2D(f, p, precision="fp32")
    g.run(steps)
    out = g.read()
    s = g.summarize()
    g.close()
    return out, s


def _eq(a, b):
    return all(np.array_equal(x[1:-1, 1:-1], y[1:-1, 1:-1]) for x, y in zip(a, b))


def test_batch_members_equal_single_grid_runs(pfa):
    p = pfa.model_params()
    grids = _grids()
    b = pfa.Batch(p, GIB)
    slots = [b.add(f) for f in grids]
    b.run(37)
    for s, f in zip(slots, grids):
        want, wsum = _alone(pfa, f, p, 37)
        got = b.read(s)
        assert _eq(got, want), s
        np.testing.assert_array_equal(b.summarize(s), wsum)
        # the ghost ring of the read-out mirrors the interior
        for a in got:
            assert np.array_equal(a[0, 1:-1], a[1, 1:-1])
            assert np.array_equal(a[1:-1, -1], a[1:-1, -2])
    b.close()


@pytest.mark.parametrize("rows,persistent", [(16, True), (48, False), (1 << 30, True),
                                             (1, False)])
def test_launch_shapes_give_identical_results(pfa, rows, persistent):
    p = pfa.model_params()
    grids = _grids(seed0=10)
    ref = pfa.Batch(p, GIB)
    rs = [ref.add(f) for f in grids]
    ref.set_launch(64, True)
    ref.run(20)
    b = pfa.Batch(p, GIB)
    bs = [b.add(f) for f in grids]
    b.set_launch(rows, persistent)
    b.run(20)
    for x, y in zip(rs, bs):
        assert _eq(ref.read(x), b.read(y))
    info = b.launch()
    assert info["persistent"] == persistent and info["units"] > 0
    ref.close()
    b.close()


def test_continuous_batching_joins_and_leaves(pfa):
    """Grid A runs 50 steps while others join and leave between runs: same
    bits as A alone for 50 steps; the others likewise for their own steps."""
    p = pfa.model_params()
    fa, fb, fc, fd = _grids(seed0=20)[2:6]
    b = pfa.Batch(p, GIB)
    a = b.add(fa)
    b.run(10)
    sb = b.add(fb)              # B joins at step 10 of A
    b.run(15)
    sc = b.add(fc)              # C joins at 25
    b.run(5)
    got_b = b.read(sb)
    b.remove(sb)                # B leaves after 20 of its own steps
    sd = b.add(fd)              # D takes the freed space
    b.run(1)                    # an odd run flips the shared parity
    b.run(19)
    assert _eq(b.read(a), _alone(pfa, fa, p, 50)[0])
    assert _eq(got_b, _alone(pfa, fb, p, 20)[0])
    assert _eq(b.read(sc), _alone(pfa, fc, p, 25)[0])
    assert _eq(b.read(sd), _alone(pfa, fd, p, 20)[0])
    b.close()


def test_tune_keeps_state_and_results(pfa):
    p = pfa.model_params()
    grids = _grids(seed0=30)
    b = pfa.Batch(p, GIB)
    slots = [b.add(f) for f in grids]
    b.run(6)
    before = [b.read(s) for s in slots]
    ms = b.tune(reps=3)
    assert ms > 0
    for s, x in zip(slots, before):
        assert _eq(b.read(s), x)       # tuning does not advance the members
    b.run(14)
    for s, f in zip(slots, grids):
        assert _eq(b.read(s), _alone(pfa, f, p, 20)[0])
    b.close()


def test_arena_admission(pfa):
    p = pfa.model_params()
    f = ic.grid2d(100, 60, seed=5, stripe_width=20, n_particles=0)
    need = pfa.Batch.footprint(f[0].shape)
    assert need == ((100 + 31) // 32 * 32) * 60 * 48  # 256-byte multiple here
    b = pfa.Batch(p, 2 * need + 256)
    s0 = b.add(f)
    s1 = b.add(f)
    assert b.add(f) is None                     # refused: no room
    assert b.info()["used_bytes"] == 2 * need
    b.remove(s0)
    s2 = b.add(f)                               # the freed block is reused
    assert s2 == s0 and b.info()["grids"] == 2
    b.remove(s1)
    b.remove(s2)
    big = ic.grid2d(160, 60, seed=6, stripe_width=20, n_particles=0)
    assert pfa.Batch.footprint(big[0].shape) <= 2 * need + 256
    s3 = b.add(big)                             # needs the two blocks coalesced
    assert s3 is not None
    b.run(4)
    assert _eq(b.read(s3), _alone(pfa, big, p, 4)[0])
    b.close()


def test_fp32_batch_error_against_fp64(pfa):
    p = pfa.model_params()
    fields = [ic.batch_grid(s, seed=100 + k) for k, s in enumerate((96, 150, 200))]
    b = pfa.Batch(p, GIB)
    slots = [b.add(f) for f in fields]
    b.run(300)
    for s, f in zip(slots, fields):
        g = pfa.Grid2D(f, p, precision="fp64")
        g.run(300)
        err = [float(np.max(np.abs(x[1:-1, 1:-1] - y[1:-1, 1:-1])))
               for x, y in zip(b.read(s), g.read())]
        g.close()
        assert max(err) <= 5e-7, err  # stated bound 1e-5; the form holds far less
    b.close()


def test_batch_errors(pfa):
    p = pfa.model_params()
    b = pfa.Batch(p, GIB)
    with pytest.raises(pfa.PfaError):
        b.remove(3)
    with pytest.raises(pfa.PfaError):
        b.summarize(0)
    b.run(5)  # an empty batch runs nothing
    b.close()


def _pinned(shape):
    import torch
    return torch.empty(shape, dtype=torch.float64, pin_memory=True).numpy()


def test_async_reads_equal_sync_reads(pfa):
    """pfa_batch_read_async into page-locked arrays, no wait until one sync:
    the same fields as pfa_batch_read and as each grid run alone."""
    p = pfa.model_params()
    grids = _grids(seed0=40)
    b = pfa.Batch(p, GIB)
    slots = [b.add(f) for f in grids]
    b.run(25)
    outs = [[_pinned(f[0].shape) for _ in range(4)] for f in grids]
    for s, o in zip(slots, outs):
        b.read_async(s, o)
    b.run(10)  # enqueued behind the reads: the reads keep the 25-step state
    b.sync()
    for s, f, o in zip(slots, grids, outs):
        want, _ = _alone(pfa, f, p, 25)
        assert _eq(o, want), s
        assert _eq(b.read(s), _alone(pfa, f, p, 35)[0]), s
    b.close()


def test_staging_ring_wraps_without_host_waits(pfa):
    """Many add / run / read / remove cycles enqueued without a wait, through
    a staging ring far smaller than their traffic (16 MiB for ~80 MiB): every
    cycle's read-out equals the grid run alone."""
    p = pfa.model_params()
    f = ic.grid2d(178, 178, seed=7, stripe_width=40, n_particles=2, radius=5.0)  # 1 MiB FP64
    want, _ = _alone(pfa, f, p, 6)
    b = pfa.Batch(p, 8 * pfa.Batch.footprint(f[0].shape))
    host = [_pinned(f[0].shape) for _ in range(4)]
    for x, a in zip(host, f):
        x[...] = a
    outs = []
    for cycle in range(40):
        s1, s2 = b.add(host), b.add(host)
        b.run(6)
        o = [[_pinned(f[0].shape) for _ in range(4)] for _ in range(2)]
        b.read_async(s1, o[0])
        b.read_async(s2, o[1])
        b.remove(s1)
        b.remove(s2)
        outs += o
    b.sync()
    for k, o in enumerate(outs):
        assert _eq(o, want), k
    b.close()


def test_removed_block_reused_at_once(pfa):
    """A grid removed while its steps are still enqueued and another added
    into the freed block right away: the new grid's import waits for those
    steps, and it advances as it would alone."""
    p = pfa.model_params()
    fa = ic.grid2d(200, 150, seed=8, stripe_width=40, n_particles=3, radius=5.0)
    fb = ic.grid2d(200, 150, seed=9, stripe_width=30, n_particles=2, radius=4.0)
    b = pfa.Batch(p, pfa.Batch.footprint(fa[0].shape))  # room for one grid only
    sa = b.add(fa)
    b.run(200)
    b.remove(sa)
    sb = b.add(fb)
    assert sb is not None
    b.run(30)
    assert _eq(b.read(sb), _alone(pfa, fb, p, 30)[0])
    b.close()


def test_grid_larger_than_the_staging_ring(pfa):
    """A member whose FP64 fields exceed the ring grows it: one interior row
    of 200 000 cells holds 19.2 MB of FP64 fields (ghost ring included) but
    only 9.6 MB of FP32 records, so the ring (the arena's size, at least
    16 MiB) is too small for it."""
    p = pfa.model_params()
    f = ic.grid2d(200000, 1, seed=10, stripe_width=5000, n_particles=0)
    assert 4 * f[0].size * 8 > (16 << 20) > pfa.Batch.footprint(f[0].shape)
    b = pfa.Batch(p, pfa.Batch.footprint(f[0].shape))
    s = b.add(f)
    b.run(12)
    assert _eq(b.read(s), _alone(pfa, f, p, 12)[0])
    b.close()
