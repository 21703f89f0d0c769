"""The allocation-free field summary, pfa_summarize_fields_noalloc.

It exists for callers that cannot let a library allocate device memory -- a
host that owns all device memory through its own pool or a fixed budget and
forbids allocation after start-up, or a step loop that must not pay the
implicit device synchronisation of cudaMalloc/cudaFree.  Such a caller passes
device-resident fields and a device output buffer; the library works in a
static scratch array.  Here it is checked, through the C ABI, against the
allocating pfa_summarize on two calls in a row (the second call reuses the
scratch the first one left behind).  This file is collected last on purpose.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _vp(t):
    return ctypes.c_void_p(t.data_ptr())


def test_noalloc_summary_matches_allocating_summary(pfa):
    import torch

    from pfa_gb300 import ic

    L = pfa.load()
    fields = ic.grid2d(300, 211, seed=77, stripe_width=40, n_particles=3, radius=6.0)
    ref = pfa.Grid2D(fields, pfa.model_params())
    want = ref.summarize()
    ref.close()

    dev = [torch.from_numpy(np.ascontiguousarray(a)).to("cuda") for a in fields]
    out = torch.zeros(5, dtype=torch.float64, device="cuda")
    ny, nx = fields[0].shape
    for _ in range(2):
        out.fill_(-1.0)
        torch.cuda.synchronize()
        rc = L.pfa_summarize_fields_noalloc(*[_vp(t) for t in dev], nx, ny, _vp(out), None)
        assert rc == 0, L.pfa_last_error_message()
        torch.cuda.synchronize()
        # same sums in a different (row-wise) order: equal to rounding
        np.testing.assert_allclose(out.cpu().numpy(), want, rtol=1e-13, atol=1e-15)


def test_noalloc_summary_rejects_grids_beyond_its_scratch(pfa):
    import torch

    L = pfa.load()
    buf = torch.zeros(8, dtype=torch.float64, device="cuda")
    # 16384 interior rows is the most the static scratch holds; the check runs
    # before anything is launched, so the small buffers are never read
    rc = L.pfa_summarize_fields_noalloc(*[_vp(buf)] * 4, 3, 16384 + 3, _vp(buf), None)
    assert rc == 1  # PFA_EINVAL
    assert b"16384" in L.pfa_last_error_message()
    L.pfa_clear_error()
