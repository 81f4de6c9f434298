"""Device building blocks of the tile deposit, through its diagnostic entry
points.

- The bounded wait for a bulk copy: each warp of the deposit waits on an
  mbarrier for its staged pair records; the wait polls a bounded number of
  times and, when the copy has not landed, records a timeout that the host
  turns into SPHG_ERR_TIMEOUT instead of a hang.  ``sphg_probe_wait_timeout``
  runs that wait on a barrier that no copy completes: it must give up (no
  fault, no hang) and leave the context usable.
- The deterministic mode's fixed-point rounding as three 21-bit chunks
  (``sphg_probe_fixed_chunks``).
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


def test_fixed_chunks_round_like_the_64bit_conversion(gpu):
    """The deterministic mode sums a tile's values as three 21-bit chunks of
    their fixed-point rounding (tiles of at most 2047 pairs) or as two
    32-bit words with a carry (larger tiles): both must hold round(v), ties
    to even, for every |v| < 2^62, so the two accumulations give the same
    bits."""
    from sphtogrid_gb300 import _lib

    L = _lib.lib()
    ctx = gpu.default_context(0)
    rng = np.random.default_rng(11)
    mags = np.exp2(rng.uniform(-30.0, 61.9, 200000))
    v = (mags * rng.choice([-1.0, 1.0], mags.size)).astype(np.float32)
    ties = np.array([k + 0.5 for k in range(-8, 8)], dtype=np.float32)
    edges = []
    for e in (20, 21, 22, 23, 41, 42, 43, 44, 61):
        for s in (-1.0, 1.0):
            b = np.float32(s * 2.0 ** e)
            edges += [b, np.nextafter(b, np.float32(0)), np.nextafter(b, np.float32(s * np.inf))]
            edges += [np.float32(s * (2.0 ** e + 0.5)), np.float32(s * (2.0 ** e - 0.5))]
    edges += [np.float32(0.0), np.float32(-0.0), np.float32(1e-45), np.float32(-1e-45),
              np.nextafter(np.float32(2.0 ** 62), np.float32(0)), -np.nextafter(np.float32(2.0 ** 62), np.float32(0))]
    v = np.concatenate([v, ties, np.array(edges, dtype=np.float32)])
    v = v[np.abs(v.astype(np.float64)) < 2.0 ** 62]
    x = np.zeros(2 * v.size, dtype=np.int64)
    _lib.check(L.sphg_probe_fixed_chunks(ctx.handle, int(v.size), v.ctypes.data, x.ctypes.data), ctx.handle)
    want = np.rint(v.astype(np.float64)).astype(np.int64)
    np.testing.assert_array_equal(x[1::2], want)  # the 64-bit conversion
    np.testing.assert_array_equal(x[0::2], want)  # the three chunks
