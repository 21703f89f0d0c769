"""Scheduling logic of the serving layer, on the CPU with a stand-in backend:
every request gets exactly its steps, admission is first-in first-out under
the footprint budgets, latencies are measured from arrival."""
import numpy as np
import pytest

from pfa_gb300.serve import Request, Server, fifo_latencies, latency_stats


class FakeBackend:
    """Budgets in bytes = cells; a handle's 'result' counts the steps it ran."""

    def __init__(self, budget_2d, budget_3d):
        self.budget = {2: budget_2d, 3: budget_3d}
        self.used = {2: 0, 3: 0}
        self.calls = []

    def footprint(self, req):
        return req.cells

    def admit(self, req):
        need = self.footprint(req)
        if self.used[req.dim] + need > self.budget[req.dim]:
            return None
        self.used[req.dim] += need
        return {"req": req, "steps": 0}

    def advance(self, steps_2d, handles_2d, items_3d):
        self.calls.append((steps_2d, [n for _, n in items_3d]))
        for h in handles_2d:
            h["steps"] += steps_2d
        for h, n in items_3d:
            h["steps"] += n

    def retire(self, handle):
        self.used[handle["req"].dim] -= self.footprint(handle["req"])
        return [np.full(handle["req"].fields[0].shape, float(handle["steps"]))]


class Clock:
    def __init__(self):
        self.t = 0.0

    def __call__(self):
        self.t += 0.001
        return self.t


def _req(rid, shape, steps, arrival=0.0):
    return Request(rid, [np.zeros(shape)] * 4, steps, arrival)


def _server(b2, b3, tick=100):
    be = FakeBackend(b2, b3)
    return Server(be, tick_steps=tick, clock=Clock()), be


def test_each_request_runs_exactly_its_steps():
    reqs = [_req(0, (12, 12), 250), _req(1, (20, 9), 1000), _req(2, (6, 6, 6), 130),
            _req(3, (5, 40), 7), _req(4, (7, 7, 9), 301)]
    srv, be = _server(10 ** 6, 10 ** 6, tick=64)
    done = srv.run_trace(reqs, realtime=False)
    assert [r.req.rid for r in done] == [0, 1, 2, 3, 4]
    for r in done:
        assert r.result[0].flat[0] == r.req.steps
        assert r.latency is not None and r.latency > 0
    # batched 2D steps never pass the end of any member
    assert all(n2 <= 64 and all(n <= 64 for n in n3) for n2, n3 in be.calls)
    assert srv.cell_updates == sum(r.steps * r.cells for r in reqs)


def test_admission_is_fifo_under_the_budget():
    # budget 2D: 300 cells; the 2nd request (10 x 25 = 250 cells) waits for the 1st
    reqs = [_req(0, (12, 12), 250), _req(1, (12, 27), 10), _req(2, (4, 4), 10)]
    srv, be = _server(300, 10)
    srv.submit(reqs[0])
    srv.submit(reqs[1])
    srv.submit(reqs[2])
    srv.tick()
    assert [r.req.rid for r in srv.active] == [0]         # 1 does not fit; 2 may not overtake
    assert [r.req.rid for r in srv.queue] == [1, 2]
    while srv.queue or srv.active:
        srv.tick()
    done = {r.req.rid: r for r in srv.done}
    assert done[1].admitted >= done[0].finished
    assert done[2].admitted >= done[1].admitted
    assert all(done[k].result[0].flat[0] == reqs[k].steps for k in range(3))
    assert be.used == {2: 0, 3: 0}


def test_request_larger_than_budget_is_reported():
    srv, _ = _server(50, 50)
    with pytest.raises(RuntimeError, match="does not fit"):
        srv.run_trace([_req(0, (12, 12), 5)], realtime=False)


def test_latency_statistics_and_fifo_model():
    lat = fifo_latencies([0.0, 0.5, 0.6, 10.0], [1.0, 1.0, 1.0, 2.0])
    np.testing.assert_allclose(lat, [1.0, 1.5, 2.4, 2.0])

    class R:
        def __init__(self, x):
            self.latency = x

    s = latency_stats([R(x) for x in range(1, 101)])
    assert s["p50_s"] == pytest.approx(50.5) and s["max_s"] == 100 and s["n"] == 100
