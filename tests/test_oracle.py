"""The CPU oracle against the reference's own compiled code (golden vectors).

tests/golden/*.npz were produced by tests/golden/make_golden.py from the
reference's thermo/parabola625.c and thermo/nucleation.c; these tests pin
the oracle's restated energy tables and step semantics to them.
"""
import numpy as np

import oracle as O
from conftest import field_err, fields_of, golden


def test_energies_match_reference(orc):
    g = golden("energies.npz")
    x, y, pd, pg, pl = g["xcr"], g["xnb"], g["pd"], g["pg"], g["pl"]
    np.testing.assert_allclose(orc.p(g["phi"]), g["p"], rtol=0, atol=1e-15)
    np.testing.assert_allclose(orc.pprime(g["phi"]), g["pprime"], rtol=0, atol=1e-14)
    for ph in range(3):
        for c in range(2):
            ref = g[f"fict_{ph}_{c}"]
            got = orc.fict(ph, c, x, y, pd, pg, pl)
            assert np.max(np.abs(got - ref)) <= 1e-14 * np.max(np.abs(ref)), (ph, c)
        ref = g[f"g_{ph}"]
        assert np.max(np.abs(orc.g(ph, x, y) - ref)) <= 1e-14 * np.max(np.abs(ref))
    for r in range(2):
        for c in range(2):
            ref = g[f"D_{r}_{c}"]
            got = orc.D(r, c, g["dx_cr"], g["dx_nb"])
            assert np.max(np.abs(got - ref)) <= 1e-14 * np.max(np.abs(ref)), (r, c)


def test_nucleation_probability_matches_reference(orc):
    g = golden("energies.npz")
    Va = 0.25 * 0.352e-9 ** 3
    dV = (2e-10) ** 2 * 1.0
    for a, b, s, R, P in zip(g["nuc_x"], g["nuc_y"], g["nuc_sigma"], g["nuc_R"], g["nuc_P"]):
        dG = orc.g(0, [a], [b])[0]
        r_, p_ = orc.nucleation_probability_sphere(a, b, dG, orc.D(0, 0, [a], [b])[0],
                                                   orc.D(1, 1, [a], [b])[0], s, Va, dV / Va, dV, 1e6)
        assert abs(r_ - R) <= 1e-14 * abs(R)
        assert abs(p_ - P) <= 1e-12 * max(abs(P), 1e-3)


def test_step_matches_reference(orc):
    g = golden("step2d.npz")
    prm = O.model_params()
    assert prm.dt == g["params"][0] and prm.dx == g["params"][1]
    cur = fields_of(g, "ic")
    done = 0
    for k in (1, 10, 100, 400):
        cur = orc.run2d(cur, prm, k - done)
        done = k
        err = field_err(cur, fields_of(g, f"s{k}"))
        assert max(err) <= 1e-13, (k, err)


def test_step_reference_dt_rule(orc):
    g = golden("step2d_refdt.npz")
    prm = O.model_params(dt_rule=0)
    assert prm.dt == g["params"][0]
    out = orc.run2d(fields_of(g, "ic"), prm, 50)
    assert max(field_err(out, fields_of(g, "s50"))) <= 1e-13


def test_nucleation_replica_matches_reference(orc):
    from golden.make_golden import NUC_A, NUC_B, nuc_struct
    g = golden("nucleation.npz")
    for tag, p in (("a", NUC_A), ("b", NUC_B)):
        res, events, n = orc.nucleation2d(fields_of(g, f"{tag}_ic"), nuc_struct(p), 42, 0)
        assert n == len(g[f"{tag}_cells"]) and n > 10
        assert [e[0] for e in events] == list(g[f"{tag}_cells"])
        assert [e[1] for e in events] == list(g[f"{tag}_phases"])
        for a, b in zip(res, fields_of(g, f"{tag}_out")):
            assert np.array_equal(a, b)


def test_summary_matches_reference(orc):
    g = golden("summary.npz")
    s = orc.summarize(fields_of(g, "ic"))
    np.testing.assert_allclose(s, g["summary"], rtol=1e-14, atol=0)


def test_free_energy_matches_reference(orc):
    g = golden("energy.npz")
    dx, dy, k0, k1, w0, w1, Om = g["params"]
    e, chem, grad = orc.energy2d(fields_of(g, "ic"), dx, dy, [k0, k1], [w0, w1], Om, maps=True)
    np.testing.assert_allclose(e, g["energy"][0], rtol=1e-13, atol=0)
    np.testing.assert_allclose(chem, g["chem"], rtol=1e-13, atol=1e-13 * np.abs(g["chem"]).max())
    np.testing.assert_allclose(grad, g["grad"], rtol=1e-13, atol=1e-13 * np.abs(g["grad"]).max())
    # both terms are present where the particles are
    assert np.abs(g["grad"]).max() > 0.01 * np.abs(g["chem"]).max()


def test_philox_known_answers():
    # Known-answer vectors of Philox4x32-10 published with the Random123
    # library (Salmon et al., SC'11).
    kat = [
        ([0, 0, 0, 0], [0, 0], [0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8]),
        ([0xffffffff] * 4, [0xffffffff] * 2, [0x408f276d, 0x41c83b0e, 0xa20bc7c6, 0x6d5451fd]),
        ([0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344], [0xa4093822, 0x299f31d0],
         [0xd16cfe09, 0x94fdcceb, 0x5001e420, 0x24126ea1]),
    ]
    for c, k, want in kat:
        assert O.philox(c, k) == want


def test_oracle_conserves_mass(orc):
    from pfa_gb300 import ic
    prm = O.model_params()
    f = ic.grid2d(40, 30, seed=3, stripe_width=10, n_particles=3, radius=4.0)
    s0 = orc.summarize(f)
    out = orc.run2d(f, prm, 200)
    s1 = orc.summarize(out)
    assert abs(s1[0] - s0[0]) < 1e-13 and abs(s1[1] - s0[1]) < 1e-13


def test_oracle_variable_mobility_conserves_mass(orc):
    """The variable-mobility Cahn-Hilliard is a divergence with zero flux
    through the mirrored edges: the mean compositions stay put."""
    from pfa_gb300 import ic
    prm = O.model_params()
    f = ic.grid2d(40, 30, seed=5, stripe_width=10, n_particles=3, radius=4.0)
    s0 = orc.summarize(f)
    out = orc.run2d_varmob(f, prm, 200)
    s1 = orc.summarize(out)
    assert abs(s1[0] - s0[0]) < 1e-13 and abs(s1[1] - s0[1]) < 1e-13
    assert max(float(np.max(np.abs(a - b))) for a, b in zip(out[:2], f[:2])) > 1e-6  # it moved


def test_oracle_3d_reduces_to_2d(orc):
    """A 3D grid uniform along z evolves like the 2D grid (7-point stencil with
    zero z-flux)."""
    from pfa_gb300 import ic
    prm = O.model_params()
    f2 = ic.grid2d(12, 10, seed=4, stripe_width=4, n_particles=2, radius=3.0)
    f3 = [np.repeat(a[None, :, :], 5, axis=0) for a in f2]
    o2 = orc.run2d(f2, prm, 20)
    o3 = orc.run3d(f3, prm, 20)
    for a, b in zip(o3, o2):
        assert np.max(np.abs(a[2, 1:-1, 1:-1] - b[1:-1, 1:-1])) <= 1e-12 * np.max(np.abs(b))


def test_nine_point_step_matches_reference_cuda_kernels(orc):
    """The oracle with the reference's 9-point mask (convolved as given, like
    its convolution_kernel) against the reference's own CUDA step run with
    that mask (tests/golden/ref_gpu_nine.npz): dx = dy after 1, 10, 100, 500
    steps and dy = 1.25 dx after 100, whole arrays (the 260-cell side makes
    the reference's ghost corners deterministic) within 1e-12 of each
    field's magnitude; measured <= 2.4e-15."""
    from ref_gpu import nine_point_mask
    r = golden("ref_gpu_nine.npz")
    prm = O.model_params()
    assert prm.dt == r["dt"][0]
    for tag in ("iso", "aniso"):
        q = prm.with_mask(nine_point_mask(*r[f"{tag}_dxy"]))
        cur, done = fields_of(r, "ic"), 0
        counts = sorted(int(k.split("_s")[1].split("_")[0]) for k in r.files
                        if k.startswith(f"{tag}_s") and k.endswith("_cr"))
        for k in counts:
            cur = orc.run2d(cur, q, k - done)
            done = k
            want = fields_of(r, f"{tag}_s{k}")
            err = [float(np.max(np.abs(a - b)) / np.max(np.abs(b))) for a, b in zip(cur, want)]
            assert max(err) <= 1e-12, (tag, k, err)
    # the default (5-point) step is untouched by the mask fields
    assert O.model_params().mask3 == 0


def test_step_matches_reference_cuda_kernels(orc):
    """The oracle's step against the reference's own CUDA step kernels
    (src/discretization.cu, compiled here for sm_103a and run on a GB300 by
    tests/golden/make_ref_gpu_golden.py, nucleation off): within 1e-12 of
    each field's magnitude on the golden grid (1, 10, 100, 400 steps), with
    the reference's dt rule (50 steps) and on the 256 x 256 workload (1000
    steps); measured <= 3.2e-15."""
    r = golden("ref_gpu_step2d.npz")
    g = golden("step2d.npz")
    prm = O.model_params()
    cur, done = fields_of(g, "ic"), 0
    for k in (1, 10, 100, 400):
        cur = orc.run2d(cur, prm, k - done)
        done = k
        assert max(field_err(cur, fields_of(r, f"step_s{k}"))) <= 1e-12, k
    g = golden("step2d_refdt.npz")
    got = orc.run2d(fields_of(g, "ic"), O.model_params(dt_rule=0), 50)
    assert max(field_err(got, fields_of(r, "refdt_s50"))) <= 1e-12
    got = orc.run2d(fields_of(r, "config1_ic"), prm, 1000)
    assert max(field_err(got, fields_of(r, "config1_s1000"))) <= 1e-12


def _ref_nuc_probabilities(orc, g):
    """The oracle's P_nuc (pinned to the reference's
    nucleation_probability_sphere) for the reference-kernel nucleation case."""
    x, y = (float(v) for v in g["comp"])
    dx, dy, dz = (float(v) for v in g["d"])
    dV = dx * dy * dz
    va = 0.25 * float(g["unit_a"][0]) ** 3
    dG = orc.g(0, [x], [y])[0]
    dcc, dnn = orc.D(0, 0, [x], [y])[0], orc.D(1, 1, [x], [y])[0]
    return [orc.nucleation_probability_sphere(x, y, dG, dcc, dnn, float(s), va, dV / va, dV,
                                              float(g["dt"][0]))[1] for s in g["sigma"]]


def test_reference_nucleation_kernel_rate_matches_oracle_probability(orc):
    """Event counts of the reference's own nucleation kernel (clock-seeded
    curand, run on a GB300 by tests/golden/make_ref_gpu_golden.py: uniform
    enriched grid, single-cell nuclei, four calls) are binomial with the
    oracle's P_nuc: each call and their sum within 5 sigma."""
    g = golden("ref_gpu_nucleation.npz")
    n = int(g["cells"][0])
    P = _ref_nuc_probabilities(orc, g)
    counts = g["counts"]
    for ph in range(2):
        assert 1e-4 < P[ph] < 1e-2, P
        for k in list(counts[:, ph]) + [int(counts[:, ph].sum())]:
            m = n * P[ph] * (len(counts) if k == counts[:, ph].sum() else 1)
            assert abs(k - m) < 5 * np.sqrt(m * (1 - P[ph])), (ph, k, m)


def test_variable_mobility_matches_reference(orc):
    """The variable-mobility restatement (step2d_varmob: the reference's
    disabled mobility and chemical_convolution kernels,
    src/discretization.cu:175-358, 618-778) against the same semantics built
    on the reference's compiled functions (tests/golden/step2d_varmob.npz):
    chemical-potential derivatives and curvatures of all three phases, the
    divergences, and 1, 10, 60 steps on two grids."""
    g = golden("step2d_varmob.npz")
    x, y = g["x"], g["y"]
    for ph in range(3):
        for c in range(2):
            want = g[f"dg_{ph}_{c}"]
            assert np.max(np.abs(orc.dg(ph, c, x, y) - want)) <= 1e-14 * np.max(np.abs(want))
        for i in range(2):
            for j in range(2):
                assert orc.d2g(ph, i, j) == g[f"d2g_{ph}"][i, j]
    p = O.model_params()
    assert p.dt == g["params"][0] and p.dx == g["params"][1]
    for k in range(2):
        f0 = [g[f"g{k}_ic_{n}"] for n in ("cr", "nb", "pd", "pl")]
        div = orc.chem_div2d(f0, p.dx, p.dy)
        for a, n in zip(div, ("cr", "nb")):
            want = g[f"g{k}_div_{n}"]
            assert np.max(np.abs(a - want)) <= 1e-12 * np.max(np.abs(want)), (k, n)
        done, f = 0, f0
        for s in (1, 10, 60):
            f = orc.run2d_varmob(f, p, s - done)
            done = s
            err = field_err(f, [g[f"g{k}_s{s}_{n}"] for n in ("cr", "nb", "pd", "pl")])
            assert max(err) <= 1e-12, (k, s, err)


def test_variable_mobility_flux_reduces_to_d_grad_gamma(orc):
    """The identity the FP32 variable-mobility form rests on, on the oracle's
    restatement: (1) the three phases' fictitious compositions share their
    diffusion potentials (dg_phase(x^phase) = dg_gam(x^gam)); (2) hence the
    16-coefficient divergence of the reference's mobility / chemical
    convolution kernels equals the sum over the four faces of
    (D_n + D_c)(x^gam_n - x^gam_c) / (2 d^2), D(X, Y) the diffusivity matrix
    at each cell."""
    from pfa_gb300 import ic
    f = ic.grid2d(24, 20, seed=9, stripe_width=8, n_particles=2, radius=3.0)
    fict, _ = orc.mobility2d(f)
    gam, phases = fict[0:2], (fict[0:2], fict[2:4], fict[4:6])
    for c in range(2):
        mu = orc.dg(0, c, gam[0], gam[1])
        for ph in (1, 2):
            other = orc.dg(ph, c, phases[ph][0], phases[ph][1])
            # rounding: a few ulps of the potential's terms (slopes up to
            # 2e11 times compositions near 0.25), 1e-12 of the potential
            assert np.max(np.abs(other - mu)) <= 1e-12 * np.max(np.abs(mu)), (ph, c)
    dx = dy = 5e-9
    want = orc.chem_div2d(f, dx, dy)
    X, Y = f[0], f[1]
    ny, nx = X.shape
    D = [[orc.D(r, k, X.ravel(), Y.ravel()).reshape(ny, nx) for k in range(2)] for r in range(2)]
    r2 = (0.5 / dx**2, 0.5 / dy**2)
    for row in range(2):
        got = np.zeros((ny - 2, nx - 2))
        c = (slice(1, -1), slice(1, -1))
        for (sy, sx), r in (((slice(1, -1), slice(2, None)), r2[0]),
                            ((slice(1, -1), slice(0, -2)), r2[0]),
                            ((slice(2, None), slice(1, -1)), r2[1]),
                            ((slice(0, -2), slice(1, -1)), r2[1])):
            for k in range(2):
                got += r * (D[row][k][sy, sx] + D[row][k][c]) * (gam[k][sy, sx] - gam[k][c])
        ref = want[row][1:-1, 1:-1]
        assert np.max(np.abs(got - ref)) <= 1e-12 * np.max(np.abs(ref)), row  # 2e-14 seen
