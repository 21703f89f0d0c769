"""Initial-condition recipes without a GPU: the recipe struct's C layout
against both ctypes mirrors, argument validation of the entry points, and
the oracle's recipe semantics (the documented noise stream, bands, particles,
ghost ring)."""
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

LAYOUT_C = r"""
#include <stddef.h>
#include <stdio.h>
#include "pfa_gb300.h"
#define F(m) printf("%s %zu\n", #m, offsetof(pfa_ic_recipe, m));
int main(void) {
  printf("size %zu\n", sizeof(pfa_ic_recipe));
  F(nx) F(ny) F(nz) F(matrix) F(enrich) F(noise) F(seed) F(n_bands) F(band)
  F(n_particles) F(centre) F(radius) F(phase) F(dx) F(width) F(profile) F(bell_sigma)
  F(bell_range) F(bell_x0) F(particle_mode)
  return 0;
}
"""


def test_recipe_layout_matches_the_header(tmp_path):
    from pfa_gb300 import lib
    import oracle as O
    src = tmp_path / "layout.c"
    src.write_text(LAYOUT_C)
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c99", "-I", os.path.join(ROOT, "include"), str(src), "-o",
                    str(exe)], check=True)
    got = dict(line.split() for line in subprocess.run([str(exe)], capture_output=True,
                                                       text=True, check=True).stdout.splitlines())
    for cls in (lib.IcRecipe, O.OrcIcRecipe):
        import ctypes
        assert int(got["size"]) == ctypes.sizeof(cls)
        for name, _ in cls._fields_:
            assert int(got[name]) == getattr(cls, name).offset, (cls.__name__, name)


def _rec(**kw):
    from pfa_gb300 import ic
    r = ic.recipe2d(48, 40, seed=9, stripes=[6, 30], stripe_width=8, n_particles=3, radius=4.0)
    r.update(kw)
    return r


def test_entry_points_reject_bad_recipes(pfa):
    import ctypes
    lib = pfa
    L = lib.load()
    bad = [dict(nx=0), dict(particles=[(1.0, 1.0, 0.0, 2.0, 0)] * 65),
           dict(bands=[(0, 1)] * 17), dict(dx=0.0), dict(width=float("nan")),
           dict(particles=[(1.0, float("inf"), 0.0, 2.0, 0)])]
    for kw in bad:
        rec = _rec(**kw)
        if len(rec["particles"]) > lib.IC_MAX_PARTICLES or len(rec["bands"]) > lib.IC_MAX_BANDS:
            with pytest.raises(ValueError):
                lib.ic_recipe(rec)
            continue
        r = lib.ic_recipe(rec)
        rc = L.pfa_ic_generate(ctypes.byref(r), *[ctypes.c_void_p(8)] * 4, None)
        assert rc == 1, kw  # PFA_EINVAL, before any device work
    # a 2D recipe is not a 3D grid; a null recipe is refused
    h = ctypes.c_void_p()
    pv = np.zeros(12)
    d = np.ones(3)
    r = lib.ic_recipe(_rec())
    assert L.pfa3d_create_ic(ctypes.byref(h), ctypes.byref(r), lib._ptr(pv), lib._ptr(d), 1) == 1
    assert L.pfa_ic_generate(None, *[ctypes.c_void_p(8)] * 4, None) == 1


def test_oracle_recipe_semantics(orc):
    import oracle as O
    from pfa_gb300 import ic
    rec = _rec()
    f = O.ic_fields(rec)
    ny, nx = rec["ny"], rec["nx"]
    # ghost ring = mirror of the interior
    for a in f:
        assert np.array_equal(a[0, 1:-1], a[1, 1:-1]) and np.array_equal(a[-1, 1:-1], a[-2, 1:-1])
        assert np.array_equal(a[:, 0], a[:, 1]) and np.array_equal(a[:, -1], a[:, -2])
    # the documented noise stream, exactly, where no particle box reaches
    pad = int(np.ceil(4.0 + 6 * (rec["width"] / 2) / rec["dx"])) + 1
    key = (rec["seed"] & 0xffffffff, rec["seed"] >> 32)
    checked = 0
    for (y, x) in [(0, 0), (5, 7), (17, 31), (39, 47), (20, 3)]:
        if any(abs(x - int(np.floor(p[0]))) <= pad and abs(y - int(np.floor(p[1]))) <= pad
               for p in rec["particles"]):
            continue
        c = y * nx + x
        w = O.philox([c & 0xffffffff, c >> 32, 0, 0x49430000], key)
        u = [(((w[0] << 32) | w[1]) >> 11) + 1, (((w[2] << 32) | w[3]) >> 11) + 1]
        u = [v * (1.0 / 9007199254740992.0) for v in u]
        want = [rec["matrix"][k] + rec["noise"] * (2.0 * u[k] - 1.0) for k in range(2)]
        for lo, hi in rec["bands"]:
            if lo <= x < hi:
                want = [want[k] + (rec["enrich"][k] - rec["matrix"][k]) for k in range(2)]
        assert f[0][y + 1, x + 1] == want[0] and f[1][y + 1, x + 1] == want[1]
        assert f[2][y + 1, x + 1] == 0.0 and f[3][y + 1, x + 1] == 0.0
        checked += 1
    assert checked >= 2
    # particle centres: phi near 1, composition near the phase's equilibrium
    for (x, y, _, R, ph) in rec["particles"]:
        xi, yi = int(round(x)), int(round(y))
        assert f[2 + ph][yi + 1, xi + 1] > 0.99
        xe = ic.XE["del" if ph == 0 else "lav"]
        assert abs(f[0][yi + 1, xi + 1] - xe[0]) < 1e-2 and abs(f[1][yi + 1, xi + 1] - xe[1]) < 1e-2


def test_oracle_reference_profile_and_embedding(orc):
    """The reference's default 2D initial condition as a recipe: the bell
    curve's mean over its range is the matrix composition and its peak the
    enrichment (thermo/enrichment.py); embed_OPC's box overwrites the phase
    (a second, overlapping particle of the same phase replaces the first's
    values inside its box)."""
    import oracle as O
    from pfa_gb300 import ic
    r = ic.reference_recipe2d(600, 60, seed=3, radius=6.0)
    f = O.ic_fields(r)
    nx, dx = r["nx"], r["dx"]
    pos = dx * (np.arange(nx) - nx // 2)
    inside = (pos >= r["bell_range"][0]) & (pos <= r["bell_range"][1])
    for k in range(2):
        row = f[k][1 + 55, 1:-1]  # a row outside the seed's box (rows 16..44)
        # the midpoint sum of the bell curve over the range: its mean to 1e-3
        assert abs(row[inside].mean() - r["matrix"][k]) < 3e-3 * r["matrix"][k]
        assert row[nx // 2] == r["enrich"][k]  # the peak
    assert f[2][1 + 30, 1 + 300] > 0.999  # the seed
    # overwrite: a small second particle over the first one lowers phi there
    r2 = dict(r, particles=r["particles"] + [(300.0, 30.0, 0.0, 1.0, 0)])
    g = O.ic_fields(r2)
    assert g[2][1 + 30, 1 + 306] < f[2][1 + 30, 1 + 306]


def test_oracle_embedding_matches_reference_code(orc):
    """The oracle's particles in embed_OPC's mode against embed_OPC's loop
    (src/alloy625.cpp:262-294) run with the reference's own compiled
    tanh_interp (thermo/nucleation.c:12-16), p and equilibrium compositions
    (thermo/parabola625.c) on the same particle-free fields
    (tests/golden/ic_embed.npz, tests/golden/make_golden.py): overlapping
    boxes, two spacings.  The oracle evaluates p in another order of
    operations, hence a few ulps."""
    import oracle as O
    from conftest import golden
    from golden.make_golden import IC_RECIPES
    g = golden("ic_embed.npz")
    for n, rec in enumerate(IC_RECIPES):
        got = O.ic_fields(rec, orc)
        for j, name in enumerate(("cr", "nb", "pd", "pl")):
            want = g[f"r{n}_{name}"]
            assert np.max(np.abs(got[j] - want)) <= 1e-15, (n, name)
            assert np.array_equal(got[j] == 0.0, want == 0.0)
    # the profile itself: tanh_interp(r, w) = 0.5 - 0.5 tanh(r / w)
    prof = 0.5 - 0.5 * np.tanh(g["tanh_r"][None, :] / g["tanh_w"][:, None])
    assert np.max(np.abs(prof - g["tanh_v"])) <= 2.3e-16
