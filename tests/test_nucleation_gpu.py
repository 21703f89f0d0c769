"""GPU nucleation: Philox known answers, bit-exact event sets against the CPU
replica, the reference-generated golden events, and the event rate against
the reference's nucleation probability and its own nucleation kernel's
event counts."""
import numpy as np
import pytest

import oracle as O
from conftest import fields_of, golden

pytestmark = pytest.mark.gpu


def _nuc_kwargs(p):
    return dict(sigma=p["sigma"], unit_a=p["unit_a"], d=p["d"], dt_nuc=p["dt"])


def _nucleate_once(pfa, fields, nuc, seed=42, calls=1, precision="fp64"):
    """Put `fields` into the *_new slot, run device_nucleation `calls` times,
    swap back and read (the reference applies nucleation to *_new before the
    caller's swap, src/main.cpp:307-321)."""
    grid = pfa.Grid2D(fields, pfa.model_params(), precision=precision)
    grid.set_nucleation(seed=seed, geometry=pfa.NUC_FIXED_GEOMETRY)
    if precision == "fp64":
        grid.swap()
    events = []
    for _ in range(calls):
        grid.nucleate(**_nuc_kwargs(nuc))
        events.append(grid.events())
    if precision == "fp64":
        grid.swap()
    out = grid.read()
    grid.close()
    return out, events


def test_philox_device_known_answers(pfa):
    ctr = np.array([[0, 0, 0, 0], [0xffffffff] * 4], dtype=np.uint32)
    out = pfa.philox_device(ctr[:1], 0)
    assert list(out[0]) == [0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8]
    out = pfa.philox_device(ctr[1:], 0xffffffffffffffff)
    assert list(out[0]) == [0x408f276d, 0x41c83b0e, 0xa20bc7c6, 0x6d5451fd]
    out = pfa.philox_device(np.array([[0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344]],
                                     dtype=np.uint32), (0x299f31d0 << 32) | 0xa4093822)
    assert list(out[0]) == [0xd16cfe09, 0x94fdcceb, 0x5001e420, 0x24126ea1]
    rng = np.random.default_rng(1)
    c = rng.integers(0, 2 ** 32, (257, 4), dtype=np.uint64).astype(np.uint32)
    key = int(rng.integers(0, 2 ** 63))
    dev = pfa.philox_device(c, key)
    for k in range(0, 257, 17):
        assert list(dev[k]) == O.philox(list(map(int, c[k])), [key & 0xffffffff, key >> 32])


@pytest.mark.parametrize("tag", ["a", "b"])
def test_events_match_reference_golden(pfa, tag):
    from golden.make_golden import NUC_A, NUC_B
    nuc = NUC_A if tag == "a" else NUC_B
    g = golden("nucleation.npz")
    out, events = _nucleate_once(pfa, fields_of(g, f"{tag}_ic"), nuc)
    ev = events[0]
    assert [e[0] for e in ev] == list(g[f"{tag}_cells"])
    assert [e[1] for e in ev] == list(g[f"{tag}_phases"])
    for a, b in zip(out, fields_of(g, f"{tag}_out")):
        assert np.array_equal(a, b)


@pytest.mark.parametrize("seed", [1, 7, 2026])
def test_event_sets_bit_exact_against_cpu_replica(pfa, orc, seed):
    # nearly every cell of this enriched grid needs the FP64 decision: the
    # first quarter of them is listed for the FP64 pass, the rest is decided
    # in place, so both routes are checked against the replica
    from golden.make_golden import NUC_A, nuc_struct
    from pfa_gb300 import ic
    f = ic.grid2d(96, 80, seed=seed, matrix=(0.2600, 0.1680), enrich=(0.2720, 0.1692),
                  stripes=[30], stripe_width=20, n_particles=2, radius=5.0)
    out, events = _nucleate_once(pfa, f, NUC_A, seed=seed, calls=2)
    want = f
    total = 0
    for call in range(2):
        # the second call mostly finds cells inside the first call's scan radius
        want, ev, n = orc.nucleation2d(want, nuc_struct(NUC_A), seed, call)
        total += n
        assert [(e[0], e[1]) for e in ev] == events[call], call
    assert total > 0
    for a, b in zip(out, want):
        assert np.array_equal(a, b)


def test_physical_parameters_give_no_events(pfa):
    """With the reference's sigma = 0.13 J/m^2 and its wrapper geometry the
    probability underflows to 0 at the workload compositions."""
    from pfa_gb300 import ic
    f = ic.config1()
    grid = pfa.Grid2D(f, pfa.model_params())
    grid.set_nucleation(seed=42, geometry=pfa.NUC_REFERENCE_GEOMETRY)
    grid.swap()
    grid.nucleate(sigma=(0.13, 0.13), unit_a=0.352e-9, d=(5e-9,) * 3,
                  dt_nuc=100 * grid.params["dt"])
    assert grid.events() == []
    grid.swap()
    assert all(np.array_equal(a, b) for a, b in zip(grid.read(), f))
    grid.close()


def test_event_rate_matches_reference_probability(pfa, orc):
    """Uniform grid, all cells eligible: delta and laves event counts are
    binomial with the reference's P_nuc (oracle pinned to the reference's
    nucleation_probability_sphere by the golden vectors)."""
    from pfa_gb300 import ic
    n = 384
    comp = (0.2720, 0.1692)
    f = ic.grid2d(n, n, seed=5, matrix=comp, enrich=comp, noise=0.0, stripes=[], n_particles=0)
    nuc = dict(sigma=(0.05, 0.06), unit_a=0.352e-9, d=(2e-10, 2e-10, 1.0), dt=1e6)
    Va = 0.25 * nuc["unit_a"] ** 3
    dV = nuc["d"][0] * nuc["d"][1] * nuc["d"][2]
    dG = orc.g(0, [comp[0]], [comp[1]])[0]
    dcc, dnn = orc.D(0, 0, [comp[0]], [comp[1]])[0], orc.D(1, 1, [comp[0]], [comp[1]])[0]
    P = [orc.nucleation_probability_sphere(comp[0], comp[1], dG, dcc, dnn, s, Va, dV / Va, dV,
                                           nuc["dt"])[1] for s in nuc["sigma"]]
    _, events = _nucleate_once(pfa, f, nuc, seed=99)
    N = n * n
    for ph in range(2):
        k = sum(1 for e in events[0] if e[1] == ph)
        mean, sd = N * P[ph], np.sqrt(N * P[ph] * (1 - P[ph]))
        assert abs(k - mean) < 5 * sd, (ph, k, mean, sd)


def test_event_rate_matches_reference_nucleation_kernel(pfa, orc):
    """The same case the reference's own nucleation kernel ran on a GB300
    (tests/golden/ref_gpu_nucleation.npz: uniform enriched grid, single-cell
    nuclei): the event rate per phase is binomial with the oracle's P_nuc and
    agrees with the reference kernel's rate over its four calls, within 5
    sigma.  The reference also decides its ghost ring (514^2 cells); this
    library decides interior cells only (512^2)."""
    from pfa_gb300 import ic
    from test_oracle import _ref_nuc_probabilities
    g = golden("ref_gpu_nucleation.npz")
    comp = tuple(float(v) for v in g["comp"])
    side = int(round(np.sqrt(int(g["cells"][0])))) - 2
    f = ic.grid2d(side, side, seed=5, matrix=comp, enrich=comp, noise=0.0, stripes=[],
                  n_particles=0)
    nuc = dict(sigma=tuple(float(v) for v in g["sigma"]), unit_a=float(g["unit_a"][0]),
               d=tuple(float(v) for v in g["d"]), dt=float(g["dt"][0]))
    P = _ref_nuc_probabilities(orc, g)
    n_ours, n_ref = side * side, int(g["cells"][0])
    calls = g["counts"].shape[0]
    for seed in (3, 4):
        _, events = _nucleate_once(pfa, f, nuc, seed=seed)
        for ph in range(2):
            k = sum(1 for e in events[0] if e[1] == ph)
            m = n_ours * P[ph]
            assert abs(k - m) < 5 * np.sqrt(m * (1 - P[ph])), (ph, k, m)
            ref_rate = g["counts"][:, ph].sum() / (calls * n_ref)
            sd = np.sqrt(P[ph] * (1 - P[ph]) * (1 / n_ours + 1 / (calls * n_ref)))
            assert abs(k / n_ours - ref_rate) < 5 * sd, (ph, k / n_ours, ref_rate)


def test_nucleation_in_the_step_loop(pfa):
    """pfa_run with a nucleation interval equals the reference's loop order:
    evolution, nucleation when k % interval == 0, swap."""
    from pfa_gb300 import ic
    from golden.make_golden import NUC_A
    f = ic.grid2d(64, 48, seed=3, matrix=(0.2600, 0.1680), enrich=(0.2720, 0.1692),
                  stripes=[20], stripe_width=16, n_particles=1, radius=5.0)
    p = pfa.model_params()
    a = pfa.Grid2D(f, p)
    a.set_nucleation(seed=5, geometry=pfa.NUC_FIXED_GEOMETRY, interval=10, sigma=NUC_A["sigma"],
                     unit_a=NUC_A["unit_a"], d=NUC_A["d"], dt_nuc=NUC_A["dt"])
    a.run(35)
    b = pfa.Grid2D(f, p)
    b.set_nucleation(seed=5, geometry=pfa.NUC_FIXED_GEOMETRY)
    for k in range(35):
        b.L.pfa_device_evolution(b.ref, b.nx, b.ny, 3, 13, 13, p["alpha"], p["dt"])
        if k % 10 == 0:
            b.nucleate(**_nuc_kwargs(NUC_A))
        b.swap()
    # a cell that nucleates both phases has p_gamma < 0 and diverges, as in the
    # reference; both loops must still agree bit for bit
    for x, y in zip(a.read(), b.read()):
        assert np.array_equal(x, y, equal_nan=True)
    a.close()
    b.close()


@pytest.mark.parametrize("precision", ["fp32", "fp32k"])
def test_fp32_events_match_replica_on_the_same_state(pfa, orc, precision):
    """The FP32 forms decide on their exact stored values (hi - c): the CPU
    replica run on the state they hold gives the same events and painted
    fields (painted values keep a compensation: 16-bit counts of 2^-39 at
    most, or FP32)."""
    from golden.make_golden import NUC_A, nuc_struct
    from pfa_gb300 import ic
    f = ic.grid2d(96, 80, seed=7, matrix=(0.2600, 0.1680), enrich=(0.2720, 0.1692),
                  stripes=[30], stripe_width=20, n_particles=2, radius=5.0)
    g = pfa.Grid2D(f, pfa.model_params(), precision=precision)
    state = g.read()
    g.close()
    want, ev, n = orc.nucleation2d(state, nuc_struct(NUC_A), 11, 0)
    assert n > 0
    out, events = _nucleate_once(pfa, f, NUC_A, seed=11, precision=precision)
    assert events[0] == [(e[0], e[1]) for e in ev]
    tol = 2.0 ** -39 if precision == "fp32" else 1e-15
    for a, b in zip(out, want):
        assert np.max(np.abs(a[1:-1, 1:-1] - b[1:-1, 1:-1])) <= tol


def test_fp32_nucleation_runs_and_paints(pfa):
    from golden.make_golden import NUC_A
    g = golden("nucleation.npz")
    out, events = _nucleate_once(pfa, fields_of(g, "a_ic"), NUC_A, precision="fp32")
    assert len(events[0]) > 0
    for cell, ph in events[0]:
        y, x = divmod(cell, out[0].shape[1])
        assert abs(out[2 + ph][y, x] - 1.0) < 1e-7


# NUC_A's probabilities at a spacing where the neighbourhood scan covers each
# cell alone (1.75 nm / dx <= 1, the decision kernel's one-load path): dx = dy
# = 2 nm, dz scaled so that dV = dx dy dz is NUC_A's.  The nuclei are then
# narrower than a cell, so the paint takes its parallel path as well.
NUC_F = dict(sigma=(0.05, 0.05), unit_a=0.352e-9, d=(2e-9, 2e-9, 0.01), dt=1e6)


def _enriched(nx, ny, seed):
    from pfa_gb300 import ic
    return ic.grid2d(nx, ny, seed=seed, matrix=(0.2720, 0.1692), enrich=(0.2720, 0.1692),
                     stripes=[], n_particles=0)


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
@pytest.mark.parametrize("shape", [(48, 64), (131, 97)])
def test_one_cell_scan_matches_replica(pfa, orc, shape, precision):
    """A nucleation call after a step (pfa_run with a nucleation interval)
    whose neighbourhood scan covers each cell alone: the same events as the
    step followed by device_nucleation, bit-identical fields, and the events
    and painted fields of the CPU replica run on the state after the step.
    On these enriched grids most cells need the FP64 decision, more than the
    list holds, so cells are also decided in place."""
    from golden.make_golden import nuc_struct
    ny, nx = shape
    f = _enriched(nx, ny, seed=nx + ny)
    p = pfa.model_params()
    a = pfa.Grid2D(f, p, precision=precision)
    a.set_nucleation(seed=9, geometry=pfa.NUC_FIXED_GEOMETRY, interval=1, **_nuc_kwargs(NUC_F))
    a.run(1)
    ev_a, out_a = a.events(), a.read()
    a.close()
    b = pfa.Grid2D(f, p, precision=precision)
    b.set_nucleation(seed=9, geometry=pfa.NUC_FIXED_GEOMETRY)
    pfa.check(b.L.pfa_device_evolution(b.ref, b.nx, b.ny, 3, 13, 13, p["alpha"], p["dt"]),
              "device_evolution")
    b.nucleate(**_nuc_kwargs(NUC_F))  # FP64: on *_new, before the caller's swap
    if precision == "fp64":
        b.swap()
    ev_b, out_b = b.events(), b.read()
    b.close()
    assert len(ev_a) > nx * ny // 100
    assert ev_a == ev_b
    for x, y in zip(out_a, out_b):
        assert np.array_equal(x, y)
    c = pfa.Grid2D(f, p, precision=precision)
    c.run(1)
    state = c.read()
    c.close()
    want, ev, n = orc.nucleation2d(state, nuc_struct(NUC_F), 9, 0)
    assert ev_a == [(e[0], e[1]) for e in ev]
    tol = 2.0 ** -39 if precision == "fp32" else 0.0  # FP32: a 16-bit compensation count
    for x, y in zip(out_a, want):
        assert np.max(np.abs(x[1:-1, 1:-1] - y[1:-1, 1:-1])) <= tol


def test_one_cell_scan_in_the_step_loop(pfa):
    """pfa_run with a nucleation interval (replayed from a graph) equals the
    per-step loop with device_nucleation calls, bit for bit, over 35 steps
    and 4 calls, in the FP32 form."""
    from pfa_gb300 import ic
    f = ic.grid2d(96, 64, seed=5, matrix=(0.2600, 0.1680), enrich=(0.2720, 0.1692),
                  stripes=[30], stripe_width=24, n_particles=1, radius=5.0)
    p = pfa.model_params()
    a = pfa.Grid2D(f, p, precision="fp32")
    a.set_nucleation(seed=5, geometry=pfa.NUC_FIXED_GEOMETRY, interval=10, **_nuc_kwargs(NUC_F))
    a.run(35)
    b = pfa.Grid2D(f, p, precision="fp32")
    b.set_nucleation(seed=5, geometry=pfa.NUC_FIXED_GEOMETRY)
    calls = 0
    for k in range(35):
        pfa.check(b.L.pfa_device_evolution(b.ref, b.nx, b.ny, 3, 13, 13, p["alpha"], p["dt"]),
                  "device_evolution")
        if k % 10 == 0:
            b.nucleate(**_nuc_kwargs(NUC_F))
            calls += len(b.events())
    assert calls > 0
    for x, y in zip(a.read(), b.read()):
        assert np.array_equal(x, y, equal_nan=True)
    a.close()
    b.close()
