"""The variable-mobility Cahn-Hilliard (pfa_set_mobility) on the GPU.

The reference wrote this form and left it disabled: its mobility kernels are
commented out (src/discretization.cu:175-358) and its
chemical_convolution_Cr/Nb kernels (:618-778) are compiled but never launched.
Parity anchors:
  * the reference's own chemical_convolution kernels, run on a GB300 on two
    states with the oracle's coefficients (tests/golden/ref_gpu_varmob.npz,
    tests/golden/make_ref_gpu_golden.py): the divergences the library's
    compat stages produce;
  * the oracle's restatement built on the reference's compiled energy,
    diffusivity and curvature functions (tests/golden/step2d_varmob.npz):
    1, 10 and 60 steps of the fused and the stage-by-stage forms;
  * the oracle itself on odd sizes.
Tolerance: 1e-12 per field (max|a - b| / max|b| over interior and ghost
edges), as for the plain FP64 step.  The FP32 forms of the step are held to
the FP64 one: max |FP32 - FP64| per field 1e-7 after one step, 1e-5 after
the 1000 steps of C1, 1e-6 after 60 steps on ragged sizes.
"""
import numpy as np
import pytest

import oracle as O
from conftest import field_err, fields_of, golden

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-12
NAMES = ("cr", "nb", "pd", "pl")


def _grid(pfa, f, mode="fused"):
    return pfa.Grid2D(f, pfa.model_params(), mode=mode, mobility="variable")


@pytest.mark.parametrize("mode", ["fused", "compat"])
def test_steps_match_reference_built_oracle(pfa, mode):
    g = golden("step2d_varmob.npz")
    for k in range(2):
        grid = _grid(pfa, fields_of(g, f"g{k}_ic"), mode)
        done = 0
        for s in (1, 10, 60):
            if mode == "fused":
                grid.run(s - done)
            else:
                for _ in range(s - done):
                    grid.step_stages()
            done = s
            err = field_err(grid.read(), fields_of(g, f"g{k}_s{s}"))
            assert max(err) <= FP64_TOL, (mode, k, s, err)
        grid.close()


def test_divergence_matches_reference_kernels(pfa):
    """The compat stages up to device_laplacian leave the divergences of Cr
    and Nb in the *_new arrays: against the reference's compiled
    chemical_convolution kernels on the same states (interior cells)."""
    r = golden("ref_gpu_varmob.npz")
    dx, dy = r["dxy"]
    for k in range(2):
        f = [r[f"s{k}_{n}"] for n in NAMES]
        grid = _grid(pfa, f, mode="compat")
        a = (grid.ref, grid.nx, grid.ny, 3, 13, 13)
        L = grid.L
        for fn in (L.pfa_device_boundaries, L.pfa_device_fictitious, L.pfa_fictitious_boundaries,
                   L.pfa_device_mobilities, L.pfa_mobility_boundaries):
            pfa.check(fn(*a), "stage")
        pfa.check(L.pfa_device_laplacian(*a, dx, dy), "device_laplacian")
        grid.swap()  # the *_new arrays become readable
        out = grid.read()
        grid.close()
        for got, n in zip(out[:2], ("cr", "nb")):
            want = r[f"s{k}_div_{n}"]
            d = np.max(np.abs(got[1:-1, 1:-1] - want[1:-1, 1:-1]))
            assert d <= FP64_TOL * np.max(np.abs(want[1:-1, 1:-1])), (k, n, d)


@pytest.mark.parametrize("shape", [(1, 1), (5, 7), (17, 13), (33, 65), (100, 3)])
def test_fused_and_stages_match_oracle_on_odd_sizes(pfa, orc, shape):
    from pfa_gb300 import ic
    ny, nx = shape
    f = ic.grid2d(nx, ny, seed=nx * 13 + ny, stripe_width=max(1, nx // 3),
                  n_particles=1 if min(nx, ny) > 12 else 0, radius=3.0)
    want = orc.run2d_varmob(f, O.model_params(), 30)
    fused = _grid(pfa, f)
    fused.run(30)
    assert max(field_err(fused.read(), want)) <= FP64_TOL
    fused.close()
    stages = _grid(pfa, f, mode="compat")
    for _ in range(30):
        stages.step_stages()
    assert max(field_err(stages.read(), want)) <= FP64_TOL
    stages.close()


def test_variable_mobility_is_not_the_constant_form(pfa):
    """The two Cahn-Hilliard forms differ (the divergence does act), and the
    constant form is restored by PFA_MOBILITY_CONSTANT."""
    g = golden("step2d_varmob.npz")
    f = fields_of(g, "g0_ic")
    p = pfa.model_params()
    a = pfa.Grid2D(f, p, mobility="variable")
    b = pfa.Grid2D(f, p)
    c = pfa.Grid2D(f, p, mobility="variable")
    pfa.check(c.L.pfa_set_mobility(c.ref, pfa.MOBILITY_CONSTANT), "pfa_set_mobility")
    for x in (a, b, c):
        x.run(20)
    ra, rb, rc = a.read(), b.read(), c.read()
    assert max(float(np.max(np.abs(u - v))) for u, v in zip(ra[:2], rb[:2])) > 1e-6
    for u, v in zip(rb, rc):
        assert np.array_equal(u, v)
    for x in (a, b, c):
        x.close()


def test_fp32_variable_mobility_needs_the_five_point_mask(pfa):
    """The FP32 forms take the variable mobility with the 5-point mask, in
    either order of the two settings, and refuse it with the 9-point mask."""
    g = golden("step2d_varmob.npz")
    f = fields_of(g, "g0_ic")
    p = pfa.model_params()
    L = pfa.load()
    grid = pfa.Grid2D(f, p, precision="fp32")
    pfa.check(L.pfa_set_mobility(grid.ref, pfa.MOBILITY_VARIABLE), "pfa_set_mobility")
    grid.close()
    grid = pfa.Grid2D(f, p, mobility="variable")
    pfa.check(L.pfa_set_precision(grid.ref, pfa.FP32), "pfa_set_precision")
    grid.close()
    m9 = pfa.nine_point_mask(p["dx"], p["dx"])
    grid = pfa.Grid2D(f, p, mask=m9, precision="fp32")
    assert L.pfa_set_mobility(grid.ref, pfa.MOBILITY_VARIABLE) == 1  # PFA_EINVAL
    L.pfa_clear_error()
    grid.close()
    grid = pfa.Grid2D(f, p, mask=m9, mode="compat", mobility="variable")
    assert L.pfa_set_precision(grid.ref, pfa.FP32) == 1  # compat mode is FP64 only
    L.pfa_clear_error()
    grid.close()


# The FP32 variable-mobility step against the FP64 one (itself pinned above).
# The FP32 form evaluates the flux as div (D(X, Y) grad x^gamma): with
# paraboloid energies the fictitious compositions share their diffusion
# potentials, so x^phase = T_phase x^gamma + const with T_phase = H_phase^-1
# H_gamma, each phase's coefficients compose to p_phase D, and the phase
# gradient terms vanish -- the same discrete face sums as the 16-coefficient
# FP64 form, up to rounding.  Tolerance: max |FP32 - FP64| per field over the
# interior, 1e-7 after one step, 1e-5 after the 1000 steps of C1.
FP32_VM_ONE_STEP = 1e-7
FP32_VM_TOL = 1e-5


def _vm_err(pfa, f, steps, precision):
    p = pfa.model_params()
    a = pfa.Grid2D(f, p, mobility="variable")
    b = pfa.Grid2D(f, p, mobility="variable", precision=precision)
    a.run(steps)
    b.run(steps)
    ra, rb = a.read(), b.read()
    a.close()
    b.close()
    return [float(np.max(np.abs(x[1:-1, 1:-1] - y[1:-1, 1:-1]))) for x, y in zip(ra, rb)], ra, rb


@pytest.mark.parametrize("precision", ["fp32", "fp32k"])
def test_fp32_variable_mobility_matches_fp64(pfa, precision):
    from pfa_gb300 import ic
    f = ic.config1()
    err, _, _ = _vm_err(pfa, f, 1, precision)
    assert max(err) <= FP32_VM_ONE_STEP, err
    err, ra, rb = _vm_err(pfa, f, 1000, precision)
    assert max(err) <= FP32_VM_TOL, err
    # the divergence acts: the constant-mobility FP32 step ends elsewhere
    c = pfa.Grid2D(f, pfa.model_params(), precision=precision)
    c.run(1000)
    rc = c.read()
    c.close()
    assert max(float(np.max(np.abs(x - y))) for x, y in zip(rb[:2], rc[:2])) > 100 * FP32_VM_TOL


@pytest.mark.parametrize("shape", [(1, 1), (5, 7), (17, 13), (33, 65), (100, 3), (31, 61)])
def test_fp32_variable_mobility_on_odd_sizes(pfa, shape):
    """Ragged strips (widths that are not multiples of 30) and short row
    segments, 60 steps, against the FP64 variable-mobility step."""
    from pfa_gb300 import ic
    ny, nx = shape
    f = ic.grid2d(nx, ny, seed=nx * 7 + ny, stripe_width=max(1, nx // 3),
                  n_particles=1 if min(nx, ny) > 12 else 0, radius=3.0)
    err, _, _ = _vm_err(pfa, f, 60, "fp32")
    assert max(err) <= 1e-6, (shape, err)
