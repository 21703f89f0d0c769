"""Checkpoint / resume (Grid2D / Grid3D .checkpoint and .resume over
pfa_get_counters / pfa3d_get_counters, the matching setters and the FP32
forms' records): a run split at a checkpoint and resumed in a new handle
gives, bit for bit, the fields of the same run uninterrupted, with nucleation
events on both sides of the split (the phase of the nucleation interval and
the Philox counter of the next call are part of the state)."""
import ctypes

import numpy as np
import pytest

from pfa_gb300 import ic

pytestmark = pytest.mark.gpu

# sparse single-cell nuclei on an enriched grid, about 1e-3 per cell, phase
# and call (the parameters of the reference-kernel nucleation golden, so
# that nuclei rarely meet and the fields stay finite)
NUC = dict(seed=11, interval=10, sigma=(0.05, 0.06), unit_a=0.352e-9, d=(2e-9, 2e-9, 1e-3),
           dt_nuc=1e7)


def _grid():
    return ic.grid2d(90, 70, seed=3, matrix=(0.2720, 0.1692), enrich=(0.2720, 0.1692),
                     stripes=[], n_particles=0)


@pytest.mark.parametrize("precision", ["fp64", "fp32", "fp32k"])
def test_resumed_run_is_bit_identical(pfa, tmp_path, precision):
    p = pfa.model_params()
    a = pfa.Grid2D(_grid(), p, precision=precision)
    a.set_nucleation(geometry=pfa.NUC_FIXED_GEOMETRY, **NUC)
    a.run(35)  # nucleation after steps 0, 10, 20, 30
    plain = pfa.Grid2D(_grid(), p, precision=precision)
    plain.run(35)
    assert any(not np.array_equal(x, y) for x, y in zip(a.read(), plain.read())), "no event"
    plain.close()
    path = str(tmp_path / "state.npz")
    a.checkpoint(path)
    a.run(45)
    want = a.read()
    assert all(np.isfinite(x).all() for x in want)
    a.close()
    b = pfa.Grid2D.resume(path)
    b.run(45)
    for x, y in zip(b.read(), want):
        assert np.array_equal(x, y), precision
    b.close()
    # the counters are part of the state: resumed without them, the next
    # nucleation calls draw other numbers at other steps
    c = pfa.Grid2D.resume(path)
    pfa.check(c.L.pfa_set_counters(c.ref, 0, 0), "pfa_set_counters")
    c.run(45)
    assert any(not np.array_equal(x, y) for x, y in zip(c.read(), want))
    c.close()


def test_fp32_state_buffer_size_is_checked(pfa):
    g = pfa.Grid2D(_grid(), pfa.model_params(), precision="fp32")
    n = int(g.L.pfa_f32_state_bytes(g.ref))
    assert n == ((90 + 31) // 32) * 32 * 70 * 24  # A (16 B) + packed B (8 B) per record
    raw = np.zeros(n - 8, dtype=np.uint8)
    assert g.L.pfa_read_f32_state(g.ref, raw.ctypes.data, raw.size) == 1  # PFA_EINVAL
    g.L.pfa_clear_error()
    g.set_precision("fp64")
    assert int(g.L.pfa_f32_state_bytes(g.ref)) == 0
    g.close()


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_resumed_3d_run_is_bit_identical(pfa, tmp_path, precision):
    """The same for a 3D grid: nucleation after steps 0, 3 and 6 of 7 on the
    3D nucleation tests' uniformly enriched grid (finite that long),
    checkpoint after step 1.  The first call's nuclei deplete this small grid,
    so the later calls paint nothing and cannot show the counters' effect on
    the fields (the 2D test does); here the counters are checked as numbers:
    restored, then advanced by the resumed run."""
    from golden.make_golden import NUC_A
    f = ic.grid3d(20, 16, 12, seed=6, matrix=(0.2720, 0.1692), enrich=(0.2720, 0.1692),
                  slab=0, n_particles=1, radius=3.0)
    p = pfa.model_params(dim=3)
    kw = dict(seed=11, interval=3, sigma=NUC_A["sigma"], unit_a=NUC_A["unit_a"], d=NUC_A["d"],
              dt_nuc=NUC_A["dt"])
    a = pfa.Grid3D(f, p, precision=precision)
    a.set_nucleation(**kw)
    a.run(1)
    assert len(a.events()) > 0
    path = str(tmp_path / "state3d.npz")
    a.checkpoint(path)
    a.run(6)
    want = a.read()
    assert all(np.isfinite(x).all() for x in want)
    a.close()
    b = pfa.Grid3D.resume(path)
    steps, calls = ctypes.c_uint64(), ctypes.c_uint64()
    pfa.check(b.L.pfa3d_get_counters(b.h, ctypes.byref(steps), ctypes.byref(calls)), "counters")
    assert (steps.value, calls.value) == (1, 1)
    b.run(6)
    pfa.check(b.L.pfa3d_get_counters(b.h, ctypes.byref(steps), ctypes.byref(calls)), "counters")
    assert (steps.value, calls.value) == (7, 3)  # calls after steps 3 and 6
    for x, y in zip(b.read(), want):
        assert np.array_equal(x, y), precision
    b.close()


def test_resumed_fp32_variable_mobility_run_is_bit_identical(pfa, tmp_path):
    """The FP32 variable-mobility step with nucleation, split at a checkpoint
    (resume restores the precision, then the mobility, then the records)."""
    p = pfa.model_params()
    a = pfa.Grid2D(_grid(), p, precision="fp32", mobility="variable")
    a.set_nucleation(geometry=pfa.NUC_FIXED_GEOMETRY, **NUC)
    a.run(35)
    path = str(tmp_path / "vm.npz")
    a.checkpoint(path)
    a.run(45)
    want = a.read()
    assert all(np.isfinite(x).all() for x in want)
    a.close()
    b = pfa.Grid2D.resume(path)
    assert (b.precision, b.mobility) == ("fp32", "variable")
    b.run(45)
    for x, y in zip(b.read(), want):
        assert np.array_equal(x, y)
    b.close()
