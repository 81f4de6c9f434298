"""Shared test set-up: the ``gpu`` marker, the package loader and the oracle.

``-m "not gpu"`` tests run on a machine without a GPU (oracle against the
reference's known answers, host logic, ABI exports); ``-m gpu`` tests call the
CUDA library through the C ABI and compare it with the oracle.
"""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import __graft_entry__ as graft  # noqa: E402


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a)")


@pytest.fixture(scope="session")
def oracle():
    import oracle as O  # the oracle (test infrastructure)
    O.build()
    return O


@pytest.fixture(scope="session")
def pyoracle():
    import pyoracle as PO
    return PO


@pytest.fixture(scope="session")
def pkg():
    graft.build_library()
    return graft.load_package()


@pytest.fixture(scope="session")
def gpu(pkg):
    """The package, after checking that a CUDA context can be made."""
    pkg.default_context(0)
    return pkg


def rel_linf(got, ref, floor_frac=1e-12):
    """Relative L-infinity error on pixels carrying non-negligible value
    (|ref| > floor_frac * max|ref|); on the remaining pixels the absolute
    error is taken relative to max|ref|.  Returns the larger of the two."""
    got = np.asarray(got, dtype=np.float64)
    ref = np.asarray(ref, dtype=np.float64)
    assert got.shape == ref.shape, (got.shape, ref.shape)
    if ref.size == 0:
        return 0.0
    a = np.abs(ref)
    top = float(a.max())
    d = np.abs(got - ref)
    if top == 0.0:
        return float(d.max())
    sel = a > floor_frac * top
    rel = float((d[sel] / a[sel]).max()) if sel.any() else 0.0
    rest = float(d[~sel].max()) / top if (~sel).any() else 0.0
    return max(rel, rest)
