"""3D nucleation on the GPU against the oracle's 3D replica (spheres; no
counterpart in the reference, which is 2D only): bit-exact event sets and
painted fields, FP64 and FP32 forms, graph replay equal to single steps."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _fields(seed=3, particles=1):
    from pfa_gb300 import ic
    # a uniformly enriched grid (events everywhere), with or without a seeded
    # particle; with the coarse kernel spacing of NUC_B (scan radius 17.5
    # cells) a particle would veto every cell of this small grid
    return ic.grid3d(20, 16, 12, seed=seed, matrix=(0.2720, 0.1692), enrich=(0.2720, 0.1692),
                     slab=0, n_particles=particles, radius=3.0)


def _inner(a):
    return a[1:-1, 1:-1, 1:-1]


@pytest.mark.parametrize("tag", ["a", "b"])
def test_fp64_events_and_fields_match_oracle(pfa, orc, tag):
    import oracle as O
    from golden.make_golden import NUC_A, NUC_B, nuc_struct
    nuc = NUC_A if tag == "a" else NUC_B
    f = _fields(particles=1 if tag == "a" else 0)
    p = pfa.model_params(dim=3)
    # the oracle: one step, then the first nucleation call (call index 0)
    stepped = orc.run3d(f, O.model_params(dim=3), 1)
    want, ev, n = orc.nucleation3d(stepped, nuc_struct(nuc), 42, 0)
    assert n > 3
    g = pfa.Grid3D(f, p)
    g.set_nucleation(seed=42, interval=1, sigma=nuc["sigma"], unit_a=nuc["unit_a"], d=nuc["d"],
                     dt_nuc=nuc["dt"])
    g.run(1)
    got_ev = g.events()
    got = g.read()
    g.close()
    assert got_ev == [(e[0], e[1]) for e in ev]
    for x, y in zip(got, want):
        d = np.max(np.abs(_inner(x) - _inner(y))) / max(np.max(np.abs(_inner(y))), 1.0e-300)
        assert d <= 1e-12, d


def test_fp32_events_match_oracle_on_the_same_state(pfa, orc):
    """The FP32 form decides on its exact stored values (hi - c): the
    oracle's replica on the exported state gives the same events and fields."""
    from golden.make_golden import NUC_B, nuc_struct
    f = _fields(seed=5, particles=0)
    p = pfa.model_params(dim=3)
    plain = pfa.Grid3D(f, p, precision="fp32")
    plain.run(1)
    state = plain.read()
    plain.close()
    want, ev, n = orc.nucleation3d(state, nuc_struct(NUC_B), 7, 0)
    assert n > 3
    g = pfa.Grid3D(f, p, precision="fp32")
    g.set_nucleation(seed=7, interval=1, sigma=NUC_B["sigma"], unit_a=NUC_B["unit_a"],
                     d=NUC_B["d"], dt_nuc=NUC_B["dt"])
    g.run(1)
    assert g.events() == [(e[0], e[1]) for e in ev]
    got = g.read()
    g.close()
    for x, y in zip(got, want):
        # painted values carry their 16-bit compensation (2^-40); the rest round-trips
        assert np.max(np.abs(_inner(x) - _inner(y))) <= 1e-12


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_nucleation_graph_replay_equals_single_steps(pfa, precision):
    from golden.make_golden import NUC_A
    # calls after steps 0, 3 and 6; (dozens of nuclei painted into a grid this
    # small make the state degenerate after a few more steps)
    f = _fields(seed=6, particles=1)
    p = pfa.model_params(dim=3)
    kw = dict(seed=11, interval=3, sigma=NUC_A["sigma"], unit_a=NUC_A["unit_a"], d=NUC_A["d"],
              dt_nuc=NUC_A["dt"])
    a = pfa.Grid3D(f, p, precision=precision)
    a.set_nucleation(**kw)
    a.run(7)
    b = pfa.Grid3D(f, p, precision=precision)
    b.set_nucleation(**kw)
    for _ in range(7):
        b.run(1)
    for x, y in zip(a.read(), b.read()):
        assert np.isfinite(x).all()
        assert np.array_equal(x, y)
    assert a.events() == b.events()
    a.close()
    b.close()


def test_physical_parameters_nucleate_nothing(pfa):
    from pfa_gb300 import ic
    f = ic.grid3d(24, 20, 16, seed=8, slab=8, n_particles=2, radius=3.0)
    p = pfa.model_params(dim=3)
    g = pfa.Grid3D(f, p, precision="fp32")
    g.set_nucleation(seed=42, interval=5)
    g.run(20)
    assert g.events() == []
    g.close()
