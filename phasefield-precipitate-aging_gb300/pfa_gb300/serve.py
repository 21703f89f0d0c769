"""Serving many phase-field runs on one GPU: continuous batching with
HBM-footprint admission.

A request is one initial condition (four fields in the reference layout, 2D
(ny, nx) or 3D (nz, ny, nx) with the ghost ring, or a recipe the device
builds them from, pfa_ic_recipe) and a number of explicit steps.  Requests are admitted first-in first-out while their device
footprint fits the budget; 2D requests join one ``Batch`` (all advance with
one launch per time step), 3D requests get their own ``Grid3D`` handle on
their own stream, so 2D and 3D work overlap on the GPU.  Every tick advances
each admitted request by up to ``tick_steps`` steps -- never past its own
end -- then reads back and retires the finished ones and admits new ones.
A request's result does not depend on what else is being served: the batch
steps every member exactly as it would run alone.

The scheduling logic talks to a backend object (``GpuBackend`` here), so it
can be exercised without a GPU by a stand-in with the same methods.
"""
import time
from dataclasses import dataclass, field
from typing import List, Optional

import numpy as np


@dataclass
class Request:
    rid: int
    fields: Optional[list]    # four float64 arrays with the ghost ring (or None: recipe)
    steps: int
    arrival: float = 0.0      # seconds after the start of the trace
    recipe: Optional[dict] = None  # initial condition the device builds (pfa_ic_recipe)

    @property
    def shape(self):
        """Field shape with the ghost ring."""
        if self.fields is not None:
            return self.fields[0].shape
        r = self.recipe
        if int(r.get("nz", 0)) > 1:
            return (r["nz"] + 2, r["ny"] + 2, r["nx"] + 2)
        return (r["ny"] + 2, r["nx"] + 2)

    @property
    def dim(self):
        return len(self.shape)

    @property
    def cells(self):
        return int(np.prod([n - 2 for n in self.shape]))


@dataclass
class Record:
    """What the server keeps about one request."""
    req: Request
    handle: object = None
    nbytes: int = 0
    done_steps: int = 0
    admitted: Optional[float] = None
    finished: Optional[float] = None
    result: Optional[list] = None

    @property
    def remaining(self):
        return self.req.steps - self.done_steps

    @property
    def latency(self):
        return None if self.finished is None else self.finished - self.req.arrival


class GpuBackend:
    """2D requests in one Batch (its arena is the 2D budget), 3D requests in
    FP32 Grid3D handles (their summed footprint is the 3D budget)."""

    def __init__(self, lib, params2d, params3d, arena_2d, budget_3d):
        self.lib = lib
        self.batch = lib.Batch(params2d, arena_2d)
        self.params3d = params3d
        self.budget_3d = budget_3d
        self.used_3d = 0

    def footprint(self, req):
        if req.dim == 2:
            return self.lib.Batch.footprint(req.shape)
        return self.lib.Grid3D.footprint(req.shape, "fp32")

    def admit(self, req):
        """Place the request on the device (its fields uploaded, or built
        there from its recipe); None when its budget has no room."""
        if req.dim == 2:
            if req.fields is None:
                slot = self.batch.add_recipe(req.recipe)
            else:
                slot = self.batch.add(req.fields)
            return None if slot is None else ("2d", slot)
        need = self.footprint(req)
        if self.used_3d + need > self.budget_3d:
            return None
        g = self.lib.Grid3D(req.fields, self.params3d, precision="fp32", recipe=req.recipe)
        self.used_3d += need
        return ("3d", g, need)

    def advance(self, steps_2d, handles_2d, items_3d):
        """Enqueue steps_2d steps of the batch (whose members are handles_2d)
        and each (handle, steps) 3D run, then wait for all of them."""
        for h, n in items_3d:
            if n > 0:
                h[1].run(n)
        if steps_2d > 0:
            self.batch.run(steps_2d)
        self.batch.sync()
        for h, _ in items_3d:
            h[1].sync()

    def retire(self, handle):
        """Read the result back and free the request's device memory."""
        if handle[0] == "2d":
            out = self.batch.read(handle[1])
            self.batch.remove(handle[1])
            return out
        out = handle[1].read()
        handle[1].close()
        self.used_3d -= handle[2]
        return out

    def close(self):
        self.batch.close()


class Server:
    def __init__(self, backend, tick_steps=100, clock=time.perf_counter):
        self.backend = backend
        self.tick_steps = tick_steps
        self.clock = clock
        self.t0 = None
        self.queue: List[Record] = []     # submitted, not admitted (FIFO)
        self.active: List[Record] = []
        self.done: List[Record] = []
        self.ticks = 0
        self.cell_updates = 0
        self.step_launches = 0  # step kernels enqueued: one per batch step, one per 3D step

    def now(self):
        if self.t0 is None:
            self.t0 = self.clock()
        return self.clock() - self.t0

    def submit(self, req):
        self.queue.append(Record(req))

    def _admit(self):
        """First in, first out: stop at the first request that does not fit,
        so a large request is not overtaken indefinitely."""
        while self.queue:
            rec = self.queue[0]
            h = self.backend.admit(rec.req)
            if h is None:
                break
            rec.handle = h
            rec.nbytes = self.backend.footprint(rec.req)
            rec.admitted = self.now()
            self.active.append(self.queue.pop(0))

    def tick(self):
        """Admit, advance every active request, retire the finished ones.
        Returns the records finished in this tick."""
        self._admit()
        if not self.active:
            return []
        two = [r for r in self.active if r.req.dim == 2]
        three = [r for r in self.active if r.req.dim == 3]
        # the batch advances its members together: stop at the first end
        n2 = min([self.tick_steps] + [r.remaining for r in two]) if two else 0
        items3 = [(r.handle, min(self.tick_steps, r.remaining)) for r in three]
        self.backend.advance(n2, [r.handle for r in two], items3)
        self.step_launches += n2 + sum(n for _, n in items3)
        for r in two:
            r.done_steps += n2
            self.cell_updates += n2 * r.req.cells
        for r, (_, n) in zip(three, items3):
            r.done_steps += n
            self.cell_updates += n * r.req.cells
        finished = [r for r in self.active if r.remaining == 0]
        for r in finished:
            r.result = self.backend.retire(r.handle)
            r.handle = None
            r.finished = self.now()
            self.active.remove(r)
            self.done.append(r)
        self.ticks += 1
        return finished

    def run_trace(self, requests, realtime=True):
        """Serve requests arriving at their .arrival times (seconds after the
        first call); returns the finished records in request order."""
        pending = sorted(requests, key=lambda r: (r.arrival, r.rid))
        self.now()
        k = 0
        while k < len(pending) or self.queue or self.active:
            t = self.now()
            while k < len(pending) and (pending[k].arrival <= t or not realtime):
                self.submit(pending[k])
                k += 1
            if not self.queue and not self.active:
                if k < len(pending):  # idle until the next arrival
                    time.sleep(max(0.0, min(0.01, pending[k].arrival - t)))
                continue
            before = len(self.done)
            self.tick()
            if not self.active and self.queue and len(self.done) == before:
                raise RuntimeError(
                    f"request {self.queue[0].req.rid} does not fit the device budget")
        return sorted(self.done, key=lambda r: r.req.rid)


def latency_stats(records):
    lat = np.array([r.latency for r in records])
    return {"p50_s": float(np.percentile(lat, 50)), "p99_s": float(np.percentile(lat, 99)),
            "mean_s": float(lat.mean()), "max_s": float(lat.max()), "n": int(lat.size)}


def fifo_latencies(arrivals, service):
    """Completion latencies of a one-at-a-time FIFO server with the given
    service times (seconds)."""
    t = 0.0
    out = []
    for a, s in zip(arrivals, service):
        t = max(t, a) + s
        out.append(t - a)
    return np.array(out)
