"""Serving on the GPU: a request's result is the same bits whether it is
served alone or mixed with other 2D and 3D requests, and equals a direct
FP32 run of the same grid; admission under a small budget still serves
everything."""
import numpy as np
import pytest

from pfa_gb300 import ic
from pfa_gb300.serve import GpuBackend, Request, Server

pytestmark = pytest.mark.gpu
GIB = 1 << 30


def _requests():
    return [
        Request(0, ic.grid2d(62, 40, seed=1, stripe_width=12, n_particles=2, radius=4.0), 230),
        Request(1, ic.grid3d(20, 14, 12, seed=2, slab=6, n_particles=2, radius=3.0), 150),
        Request(2, ic.grid2d(100, 33, seed=3, stripe_width=20, n_particles=2, radius=4.0), 75),
        Request(3, ic.grid2d(5, 9, seed=4, stripe_width=2, n_particles=0), 301),
        Request(4, ic.grid3d(9, 9, 9, seed=5, slab=3, n_particles=0), 64),
    ]


def _serve(pfa, reqs, arena=GIB, budget3=GIB, tick=100):
    be = GpuBackend(pfa, pfa.model_params(), pfa.model_params(dim=3), arena, budget3)
    srv = Server(be, tick_steps=tick)
    done = srv.run_trace(reqs, realtime=False)
    be.close()
    return {r.req.rid: r for r in done}, srv


def _same(a, b):
    return all(np.array_equal(x, y) for x, y in zip(a, b))


def test_alone_equals_mixed(pfa):
    reqs = _requests()
    mixed, srv = _serve(pfa, reqs, tick=40)
    assert srv.ticks > 1
    for r in reqs:
        alone, _ = _serve(pfa, [r], tick=100)
        assert _same(mixed[r.rid].result, alone[r.rid].result), r.rid


def test_served_equals_direct_fp32_runs(pfa):
    reqs = _requests()
    done, _ = _serve(pfa, reqs, tick=64)
    for r in reqs:
        if r.dim == 2:
            g = pfa.Grid2D(r.fields, pfa.model_params(), precision="fp32")
        else:
            g = pfa.Grid3D(r.fields, pfa.model_params(dim=3), precision="fp32")
        g.run(r.steps)
        want = g.read()
        g.close()
        got = done[r.rid].result
        inner = (slice(1, -1),) * r.dim
        assert all(np.array_equal(x[inner], y[inner]) for x, y in zip(got, want)), r.rid


def test_small_budget_serves_everything(pfa):
    """A 2D arena that holds one of the larger grids at a time and a 3D
    budget for one grid: requests wait their turn and still finish exact."""
    reqs = _requests()
    arena = max(pfa.Batch.footprint(r.fields[0].shape) for r in reqs if r.dim == 2)
    budget3 = max(pfa.Grid3D.footprint(r.fields[0].shape) for r in reqs if r.dim == 3)
    tight, srv = _serve(pfa, reqs, arena=arena, budget3=budget3, tick=50)
    roomy, _ = _serve(pfa, reqs)
    for r in reqs:
        assert _same(tight[r.rid].result, roomy[r.rid].result), r.rid
    # the 2D requests could not all be resident at once
    order = sorted((tight[k] for k in (0, 2, 3)), key=lambda x: x.admitted)
    assert order[1].admitted >= order[0].finished
