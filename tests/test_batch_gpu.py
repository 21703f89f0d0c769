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
