"""libpfa_gb300 without a GPU: it builds, loads, exports every declared
symbol, and its host-side model code agrees with the oracle."""
import os
import re
import subprocess

import numpy as np

import oracle as O
from conftest import GOLDEN, ROOT


def _declared_c_functions():
    src = open(os.path.join(ROOT, "include", "pfa_gb300.h")).read()
    return sorted(set(re.findall(r"\b(pfa[0-9a-z]*_[a-z0-9_]+)\s*\(", src)))


def _exported(path):
    out = subprocess.run(["nm", "-D", "--defined-only", path], capture_output=True, text=True,
                         check=True).stdout
    return {ln.split()[-1] for ln in out.splitlines() if ln.strip()}


def test_library_exports_c_abi(pfa):
    names = _declared_c_functions()
    assert len(names) > 50
    assert "pfa3d_create" in names and "pfa_batch_create" in names
    L = pfa.load()
    for n in names:
        assert hasattr(L, n), n


def test_library_exports_reference_cxx_abi(pfa):
    want = [s for s in open(os.path.join(GOLDEN, "reference_abi_symbols.txt")).read().split() if s]
    have = _exported(pfa.LIB_PATH)
    missing = [s for s in want if s not in have]
    assert not missing, missing
    assert len(want) == 14


def test_batch_footprint_host_side(pfa):
    """Arena bytes of one batched grid: records of 32-aligned rows, 48 bytes
    per cell over both parities, rounded to 256 bytes (no GPU needed)."""
    L = pfa.load()
    for nx, ny in [(3, 3), (34, 66), (130, 130), (2050, 2050), (4098, 17)]:
        pitch = (nx - 2 + 31) // 32 * 32
        want = (pitch * (ny - 2) * 48 + 255) // 256 * 256
        assert L.pfa_batch_footprint(nx, ny) == want
    assert L.pfa_batch_footprint(2, 10) == 0


def test_model_params_match_oracle(pfa):
    for dim in (2, 3):
        for rule in (0, 1):
            a = pfa.model_params(dim=dim, dt_rule=rule)
            b = O.model_params(dim=dim, dt_rule=rule).as_dict()
            for k in ("D_Cr", "D_Nb", "kappa", "omega", "Lmob"):
                np.testing.assert_allclose(a[k], b[k], rtol=1e-15)
            assert a["dt"] == b["dt"]
    # the KKS-aware rule halves the explicit limit; the reference rule exceeds it
    p = pfa.model_params()
    lim = p["dx"] ** 2 / (4 * p["rho"])
    assert p["dt"] <= 0.5 * lim
    assert pfa.model_params(dt_rule=0)["dt"] > lim


def test_fast_coefficients_match_oracle(pfa, orc):
    """The FP32 path's gamma solve and grand-potential polynomials, evaluated
    in float64 with their float32 coefficients, against the oracle."""
    k = pfa.fast_coef()
    rng = np.random.default_rng(7)
    n = 500
    X = rng.uniform(0.2, 0.35, n)
    Y = rng.uniform(0.01, 0.2, n)
    pd = rng.uniform(0, 1, n)
    pl = rng.uniform(0, 1, n) * (1 - pd)
    pg = 1 - pd - pl
    mono = [pd * pd, pd * pg, pd * pl, pg * pg, pg * pl, pl * pl]
    d = k["den"].astype(np.float64)
    den = sum(d[i] * mono[i] for i in range(6))
    gam = []
    for c in range(2):
        a = k["num"][c].astype(np.float64)
        num = (X * (a[0] * pd + a[1] * pg + a[2] * pl) + Y * (a[3] * pd + a[4] * pg + a[5] * pl)
               + sum(a[6 + i] * mono[i] for i in range(6)))
        ref = orc.fict(0, c, X, Y, pd, pg, pl)
        assert np.max(np.abs(num / den - ref)) < 1e-6 * np.max(np.abs(ref))
        gam.append(ref)
    dgc = 4534264425.5240498 * gam[0] + 15095482346.486225 * gam[1] - 2573067053.9739881
    dgn = 15095482346.486225 * gam[0] + 110386166481.37187 * gam[1] - 9347516202.3169327
    for ph in (1, 2):
        xc = orc.fict(ph, 0, X, Y, pd, pg, pl)
        xn = orc.fict(ph, 1, X, Y, pd, pg, pl)
        direct = orc.g(0, *gam) - orc.g(ph, xc, xn) - dgc * (gam[0] - xc) - dgn * (gam[1] - xn)
        c = k["dP"][ph - 1].astype(np.float64)
        u1, u2 = gam[0] - k["xe_gam"][0], gam[1] - k["xe_gam"][1]
        poly = c[0] + u1 * (c[1] + c[3] * u1 + c[4] * u2) + u2 * (c[2] + c[5] * u2)
        assert np.max(np.abs(poly - direct)) < 1e-6 * np.max(np.abs(direct))


def test_masks_match_reference_formulas(pfa):
    m5 = pfa.five_point_mask(5e-9, 5e-9)
    assert m5[1, 1] == -2. * (5e-9 * 5e-9 + 5e-9 * 5e-9) / (5e-9 * 5e-9 * 5e-9 * 5e-9)
    assert m5.sum() == 0 or abs(m5.sum()) < 1e-6 * abs(m5[1, 1])
    m9 = pfa.nine_point_mask(5e-9, 5e-9)
    assert abs(m9.sum()) < 1e-6 * abs(m9[1, 1])


def test_c_layout_of_cudadata(pfa):
    import ctypes
    # 1 generator pointer + 4 streams + 4 events + 16 field pointers (src/type.h:58-107)
    assert ctypes.sizeof(pfa.CudaData) == 25 * ctypes.sizeof(ctypes.c_void_p)
