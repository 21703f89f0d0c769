import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG_DIR = os.path.join(ROOT, "phasefield-precipitate-aging_gb300")
ORACLE_DIR = os.path.join(ROOT, "oracle")
GOLDEN = os.path.join(ROOT, "tests", "golden")
for p in (PKG_DIR, ORACLE_DIR):
    if p not in sys.path:
        sys.path.insert(0, p)

FIELDS = ("cr", "nb", "pd", "pl")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs on the GB300 box)")


@pytest.fixture(scope="session")
def orc():
    import oracle
    oracle.build(fast=False)
    return oracle.Oracle()


@pytest.fixture(scope="session")
def pfa():
    from pfa_gb300 import build, lib
    build.build()
    lib.load()
    return lib


def golden(name):
    return np.load(os.path.join(GOLDEN, name))


def fields_of(d, prefix):
    return [d[f"{prefix}_{n}"] for n in FIELDS]


def field_err(a, b, corners=False):
    """Per-field max|a - b| / max|b| over interior and ghost edges (the
    reference leaves its four corner cells unspecified)."""
    out = []
    for x, y in zip(a, b):
        m = np.ones(x.shape, dtype=bool)
        if not corners and x.ndim == 2:
            m[0, 0] = m[0, -1] = m[-1, 0] = m[-1, -1] = False
        d = np.max(np.abs(x - y)[m])
        s = np.max(np.abs(y[m]))
        out.append(d / s if s > 0 else d)
    return out


def interior(a):
    return a[(slice(1, -1),) * a.ndim]
