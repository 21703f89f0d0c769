"""Checkpoint files on the host: Grid2D.resume / Grid3D.resume refuse a file
that is not a checkpoint of their kind with ValueError before any device work
(so these run without a GPU), and the reader returns what the writer stored."""
import json

import numpy as np
import pytest

from pfa_gb300 import lib


def _write(path, meta, shape=(6, 5), mask=True, f32=None):
    fields = {k: np.full(shape, i + 0.5) for i, k in enumerate(("cr", "nb", "pd", "pl"))}
    extra = {}
    if mask:
        extra["mask"] = lib.five_point_mask(5e-9, 5e-9)
    if f32 is not None:
        extra["f32_state"] = f32
    np.savez(path, meta=np.array(json.dumps(meta)), **fields, **extra)


def _meta(dim=2, **kw):
    m = dict(format=lib.CHECKPOINT_FORMAT, dim=dim, params={}, precision="fp64", mode="fused",
             mobility="constant", nucleation=None, steps=7, nucleation_calls=3)
    m.update(kw)
    return m


def test_reader_returns_what_was_stored(tmp_path):
    p = str(tmp_path / "a.npz")
    raw = np.arange(48, dtype=np.uint8)
    _write(p, _meta(), f32=raw)
    meta, fields, mask, got = lib._load_checkpoint(p, dim=2)
    assert (meta["steps"], meta["nucleation_calls"]) == (7, 3)
    assert [float(f[0, 0]) for f in fields] == [0.5, 1.5, 2.5, 3.5]
    assert np.array_equal(mask, lib.five_point_mask(5e-9, 5e-9))
    assert np.array_equal(got, raw) and got.flags["C_CONTIGUOUS"]


@pytest.mark.parametrize("case", ["format", "dim", "no-meta", "shapes"])
def test_resume_refuses_other_files(tmp_path, case):
    p = str(tmp_path / "b.npz")
    if case == "format":
        _write(p, _meta(format="something-else"))
    elif case == "dim":
        _write(p, _meta(dim=3))
    elif case == "no-meta":
        np.savez(p, cr=np.zeros((4, 4)))
    else:
        _write(p, _meta(dim=3), shape=(6, 5))  # 2D arrays under a 3D record
    cls = lib.Grid3D if case == "shapes" else lib.Grid2D
    with pytest.raises(ValueError):
        cls.resume(p)
