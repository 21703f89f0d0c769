"""Size limits refused before any allocation: the FP32 form's kernels index a
grid's (2D) or a plane's (3D) records with 32-bit integers, so a grid (plane)
of 2^31 records or more is refused with PFA_EINVAL by batch admission and 3D
creation, which check the sizes before reading the host arrays."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SIDE = 46400  # ceil(46398 / 32) * 32 * 46398 records > 2^31


def test_batch_refuses_a_grid_above_the_record_limit(pfa):
    b = pfa.Batch(pfa.model_params(), 1 << 24)
    tiny = [np.zeros(4) for _ in range(4)]
    slot = ctypes.c_int(-1)
    rc = b.L.pfa_batch_add(b.h, SIDE, SIDE, *[pfa._ptr(a) for a in tiny], ctypes.byref(slot))
    assert rc == 1  # PFA_EINVAL
    assert b"2^31" in b.L.pfa_last_error_message()
    b.L.pfa_clear_error()
    b.close()


def test_3d_refuses_a_plane_above_the_record_limit(pfa):
    L = pfa.load()
    p = pfa.model_params(dim=3)
    pv = pfa.params_vector(p)
    d = np.array([p["dx"]] * 3)
    tiny = [np.zeros(4) for _ in range(4)]
    h = ctypes.c_void_p()
    rc = L.pfa3d_create(ctypes.byref(h), SIDE, SIDE, 3, pfa._ptr(pv), pfa._ptr(d),
                        *[pfa._ptr(a) for a in tiny], pfa.FP32)
    assert rc == 1 and not h.value
    assert b"2^31" in L.pfa_last_error_message()
    L.pfa_clear_error()
