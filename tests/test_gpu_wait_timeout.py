"""The tile deposit's bounded wait for a bulk copy.

Each warp of the deposit waits on an mbarrier for its staged pair records;
the wait polls a bounded number of times and, when the copy has not landed,
records a timeout that the host turns into SPHG_ERR_TIMEOUT instead of a
hang.  ``sphg_probe_wait_timeout`` runs that wait on a barrier that no copy
completes: it must give up (no fault, no hang) and leave the context usable.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_bounded_wait_gives_up_and_context_stays_usable(gpu):
    from sphtogrid_gb300 import _lib

    L = _lib.lib()
    ctx = gpu.default_context(0)
    t = C.c_int32(-1)
    _lib.check(L.sphg_probe_wait_timeout(ctx.handle, 4096, C.byref(t)), ctx.handle)
    assert t.value == 1
    assert L.sphg_probe_wait_timeout(ctx.handle, 0, C.byref(t)) != 0  # polls out of range

    rng = np.random.default_rng(7)
    n, P = 2000, 32
    pos = rng.uniform(0.0, 1.0, (3, n))
    hsml = rng.uniform(0.02, 0.08, n)
    m = np.full(n, 1e-3)
    rho = rng.uniform(0.5, 2.0, n)
    par = gpu.mappingParameters(x_lim=[0, 1], y_lim=[0, 1], z_lim=[0, 1], Npixels=P)
    img = gpu.sphMapping(pos.copy(), hsml, m, rho, rho, rho, param=par, kernel=gpu.Cubic(2),
                         precision="fp32c", dimensions=3)
    assert np.isfinite(img).all() and img.max() > 0
