"""3D grids (7-point Laplacian) on the GPU against the oracle's 3D step.

The reference is 2D only; the oracle extends its equations unchanged to
three dimensions (oracle/step_impl.h, step3d), and the 3D kernels are held
to the same tolerances as the 2D ones: FP64 within 1e-12 of the oracle,
the FP32 form within 1e-5 absolute of FP64.
"""
import numpy as np
import pytest

import oracle as O
from conftest import field_err

pytestmark = pytest.mark.gpu


def _params(pfa):
    return pfa.model_params(dim=3)


@pytest.mark.parametrize("shape", [(1, 1, 1), (7, 3, 5), (12, 14, 20), (40, 9, 33)])
def test_fp64_3d_matches_oracle(pfa, orc, shape):
    from pfa_gb300 import ic
    nz, ny, nx = shape
    f = ic.grid3d(nx, ny, nz, seed=nx + 7 * ny + 31 * nz, slab=max(1, nx // 3),
                  n_particles=2 if min(shape) >= 9 else 0, radius=3.0)
    p = _params(pfa)
    want = orc.run3d(f, O.model_params(dim=3), 30)
    g = pfa.Grid3D(f, p)
    g.run(30)
    got = g.read()
    g.close()
    # compare interior + faces (edges/corners of the ghost ring are not read)
    # relative to the field's magnitude (fields that are zero everywhere: absolute)
    err = [np.max(np.abs(a[1:-1, 1:-1, 1:-1] - b[1:-1, 1:-1, 1:-1])) /
           max(np.max(np.abs(b[1:-1, 1:-1, 1:-1])), 1.0e-300)
           for a, b in zip(got, want)]
    assert max(err) <= 1e-12, err
    for a in got:  # zero-flux faces mirror the interior
        assert np.array_equal(a[0, 1:-1, 1:-1], a[1, 1:-1, 1:-1])
        assert np.array_equal(a[1:-1, 1:-1, -1], a[1:-1, 1:-1, -2])


@pytest.mark.parametrize("shape", [(1, 1, 1), (2, 5, 6), (3, 17, 31), (7, 3, 5), (12, 14, 20),
                                   (40, 9, 33), (41, 30, 61)])
def test_fp32_3d_matches_oracle_on_odd_sizes(pfa, orc, shape):
    """The FP32 form's plane pipeline (two planes per barrier, a one-plane
    tail for odd plane counts, clamped planes at the faces) on sizes that
    hit every branch, against the FP64 oracle within the stated bound."""
    from pfa_gb300 import ic
    nz, ny, nx = shape
    f = ic.grid3d(nx, ny, nz, seed=nx + 5 * ny + 17 * nz, slab=max(1, nx // 3),
                  n_particles=2 if min(shape) >= 9 else 0, radius=3.0)
    want = orc.run3d(f, O.model_params(dim=3), 25)
    g = pfa.Grid3D(f, _params(pfa), precision="fp32")
    g.run(25)
    got = g.read()
    g.close()
    for a, b in zip(got, want):
        assert np.max(np.abs(a[1:-1, 1:-1, 1:-1] - b[1:-1, 1:-1, 1:-1])) <= 1e-5


def test_3d_uniform_in_z_equals_2d(pfa):
    from pfa_gb300 import ic
    f2 = ic.grid2d(45, 37, seed=4, stripe_width=9, n_particles=2, radius=4.0)
    f3 = [np.repeat(a[None, :, :], 6, axis=0) for a in f2]
    p = _params(pfa)
    g2 = pfa.Grid2D(f2, p)
    g2.run(40)
    g3 = pfa.Grid3D(f3, p)
    g3.run(40)
    a2, a3 = g2.read(), g3.read()
    for x, y in zip(a3, a2):
        for z in range(1, x.shape[0] - 1):
            assert np.max(np.abs(x[z, 1:-1, 1:-1] - y[1:-1, 1:-1])) <= 1e-12 * np.max(np.abs(y))
    g2.close()
    g3.close()


def test_c4_recipe_64_cube_against_oracle(pfa, orc):
    """The 512^3 workload's recipe (matrix + noise, an enriched slab,
    spheres R = 6) on a 64^3 crop: the FP64 step against the oracle's 3D
    restatement after 100 steps (1e-12), and the FP32 form against FP64 at
    the workload's 2000 steps within the stated bound (measured at 512^3:
    4.1e-8)."""
    from pfa_gb300 import ic
    f = ic.grid3d(64, 64, 64, seed=4, slab=16, n_particles=4, radius=6.0)
    p = _params(pfa)
    want = orc.run3d(f, O.model_params(dim=3), 100)
    b = pfa.Grid3D(f, p)
    b.run(100)
    got = b.read()
    err = [np.max(np.abs(x[1:-1, 1:-1, 1:-1] - y[1:-1, 1:-1, 1:-1])) /
           np.max(np.abs(y[1:-1, 1:-1, 1:-1])) for x, y in zip(got, want)]
    assert max(err) <= 1e-12, err
    a = pfa.Grid3D(f, p, precision="fp32")
    a.run(2000)
    b.run(1900)
    err = [float(np.max(np.abs(x[1:-1, 1:-1, 1:-1] - y[1:-1, 1:-1, 1:-1])))
           for x, y in zip(a.read(), b.read())]
    print("64^3 crop of the 512^3 recipe, fp32 max field error after 2000 steps", err)
    assert max(err) <= 2e-7, err
    a.close()
    b.close()


def test_fp32_3d_error_against_fp64(pfa):
    from pfa_gb300 import ic
    f = ic.grid3d(64, 48, 40, seed=9, slab=16, n_particles=4, radius=5.0)
    p = _params(pfa)
    a = pfa.Grid3D(f, p, precision="fp32")
    b = pfa.Grid3D(f, p)
    a.run(300)
    b.run(300)
    fa, fb = a.read(), b.read()
    err = [float(np.max(np.abs(x[1:-1, 1:-1, 1:-1] - y[1:-1, 1:-1, 1:-1]))) for x, y in zip(fa, fb)]
    print("3D fp32 max field error after 300 steps", err)
    assert max(err) <= 5e-7, err  # stated bound 1e-5; the form holds far less
    sa, sb = a.summarize(), b.summarize()
    np.testing.assert_allclose(sa[:2], sb[:2], rtol=0, atol=1e-9)
    a.close()
    b.close()


def test_3d_summary_matches_oracle(pfa, orc):
    from pfa_gb300 import ic
    f = ic.grid3d(30, 20, 10, seed=10, slab=8, n_particles=2, radius=3.0)
    g = pfa.Grid3D(f, _params(pfa))
    np.testing.assert_allclose(g.summarize(), orc.summarize(f), rtol=1e-13)
    g.run(5)
    np.testing.assert_allclose(g.summarize(), orc.summarize(g.read()), rtol=1e-13)
    g.close()


def test_3d_graph_replay_equals_single_steps(pfa):
    from pfa_gb300 import ic
    f = ic.grid3d(33, 18, 12, seed=11, slab=8, n_particles=2, radius=3.0)
    p = _params(pfa)
    for prec in ("fp64", "fp32"):
        a = pfa.Grid3D(f, p, precision=prec)
        a.run(23)
        b = pfa.Grid3D(f, p, precision=prec)
        for _ in range(23):
            b.run(1)
        for x, y in zip(a.read(), b.read()):
            assert np.array_equal(x, y), prec
        a.close()
        b.close()


def test_3d_async_transfers_keep_order(pfa):
    """pfa3d_read_async then pfa3d_upload_async and steps on one handle, and
    jobs alternating over two handles: each read-out returns the state of its
    own job, as the waiting calls give it."""
    import torch
    from pfa_gb300 import ic
    p = _params(pfa)
    jobs = [ic.grid3d(40, 33, 21, seed=s, slab=10, n_particles=2, radius=4.0) for s in range(4)]

    def pinned(arrays):
        out = []
        for a in arrays:
            h = torch.empty(a.shape, dtype=torch.float64, pin_memory=True).numpy()
            h[...] = a
            out.append(h)
        return out

    want = []
    g = pfa.Grid3D(jobs[0], p, precision="fp32")
    for f in jobs:
        g.upload(f)
        g.run(12)
        want.append(g.read())
    g.close()
    host_in = [pinned(f) for f in jobs]
    host_out = [pinned([np.zeros_like(a) for a in f]) for f in jobs]
    h = [pfa.Grid3D(jobs[0], p, precision="fp32") for _ in range(2)]
    h[0].upload(host_in[0], wait=False)
    for k in range(len(jobs)):
        d, o = h[k % 2], h[(k + 1) % 2]
        if k + 1 < len(jobs):
            o.upload(host_in[k + 1], wait=False)
        d.run(12)
        d.read(host_out[k], wait=False)
    for x in h:
        x.sync()
        x.close()
    for k in range(len(jobs)):
        assert all(np.array_equal(a, b) for a, b in zip(host_out[k], want[k])), k


def test_staging_wait_that_runs_out_is_reported(pfa):
    """The bounded wait of the FP32 3D step's TMA ring: with one plane's copy
    withheld (pfa3d_test_skip_plane: the first CTA neither arms nor issues
    it), that CTA's wait runs out after about a second, the CTA stops and
    drains its other copies, and the handle reports PFA_ECUDA once (a TMA
    staging wait gave up).  The context stays usable: the same handle, given
    its fields again, then runs bit for bit like a fresh one."""
    from pfa_gb300 import ic
    f = ic.grid3d(64, 48, 40, seed=21, slab=12, n_particles=2, radius=4.0)
    p = pfa.model_params(dim=3)
    L = pfa.load()
    g = pfa.Grid3D(f, p, precision="fp32")
    pfa.check(L.pfa3d_test_skip_plane(g.h, 1), "pfa3d_test_skip_plane")
    g.run(1)
    with pytest.raises(pfa.PfaError, match="gave up"):
        g.sync()
    L.pfa_clear_error()
    g.sync()  # reported once
    g.upload(f)
    g.run(6)
    ref = pfa.Grid3D(f, p, precision="fp32")
    ref.run(6)
    for a, b in zip(g.read(), ref.read()):
        assert np.array_equal(a, b)
    g.close()
    ref.close()
