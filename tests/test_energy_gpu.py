"""On-device free energy (summarize_energy, src/alloy625.cpp:865-919) against
the golden vectors made from the reference's compiled energies."""
import numpy as np
import pytest

from conftest import fields_of, golden
from pfa_gb300 import ic

pytestmark = pytest.mark.gpu


def test_energy_matches_reference_golden(pfa):
    g = golden("energy.npz")
    dx, dy, k0, k1, w0, w1, Om = g["params"]
    p = dict(pfa.model_params(), dx=dx, dy=dy, kappa=[k0, k1], omega=[w0, w1])
    grid = pfa.Grid2D(fields_of(g, "ic"), p)
    e, chem, grad = grid.energy(alpha=Om, maps=True)
    grid.close()
    np.testing.assert_allclose(e, g["energy"][0], rtol=1e-12)
    inner = (slice(1, -1), slice(1, -1))
    np.testing.assert_allclose(chem[inner], g["chem"][inner], rtol=0,
                               atol=1e-12 * np.abs(g["chem"]).max())
    np.testing.assert_allclose(grad[inner], g["grad"][inner], rtol=0,
                               atol=1e-12 * np.abs(g["grad"]).max())
    assert not chem[0].any() and not grad[:, -1].any()  # ghost ring untouched


def test_energy_matches_oracle_after_steps(pfa, orc):
    p = pfa.model_params()
    f = ic.grid2d(70, 45, seed=8, stripe_width=14, n_particles=2, radius=5.0)
    g = pfa.Grid2D(f, p)
    g.run(60)
    e = g.energy()
    want = orc.energy2d(g.read(), p["dx"], p["dx"], p["kappa"], p["omega"], p["alpha"])
    np.testing.assert_allclose(e, want, rtol=1e-12)
    # the FP32 form's energy is that of its exported fields
    g32 = pfa.Grid2D(f, p, precision="fp32")
    g32.run(60)
    e32 = g32.energy()
    want32 = orc.energy2d(g32.read(), p["dx"], p["dx"], p["kappa"], p["omega"], p["alpha"])
    np.testing.assert_allclose(e32, want32, rtol=1e-12)
    assert abs(e32 - e) <= 1e-5 * abs(e)
    g.close()
    g32.close()


def test_energy_3d_uniform_in_z(pfa):
    p2 = pfa.model_params()
    p3 = pfa.model_params(dim=3)
    f2 = ic.grid2d(33, 21, seed=9, stripe_width=8, n_particles=2, radius=4.0)
    nz = 5
    f3 = [np.repeat(a[None], nz + 2, axis=0) for a in f2]
    e2 = pfa.Grid2D(f2, p2).energy(alpha=p3["alpha"])
    g3 = pfa.Grid3D(f3, p3)
    e3 = g3.energy()
    g3.close()
    np.testing.assert_allclose(e3, nz * p3["dz"] * e2, rtol=1e-12)
