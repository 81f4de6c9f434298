"""Integer work of the mapping, particle by particle, against the oracle.

``sph_footprints`` (C ABI ``sphg_footprints``) runs the device code every map
runs before it deposits: centring (filter_shift.jl:6-32), the inclusive
filter (filter_shift.jl:40-58), the quantity skip (cic_2D.jl:154-168) and
pix_index_min_max (cic_shared.jl:46-52).  Each particle's state and its
[iMin, iMax, jMin, jMax, kMin, kMax] must equal the oracle's bit for bit.
The oracle reports an empty range as it computes it (max may fall more than
one below min); the library reports max = min - 1, so empties are compared
as empties.
"""
import importlib.util
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _synth():
    spec = importlib.util.spec_from_file_location("synth", os.path.join(ROOT, "sphtogrid.jl_gb300", "synth.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def _check(gpu, oracle, pos, hsml, q, dims, P, calc_mean=False, **par_kw):
    import torch

    par = gpu.mappingParameters(Npixels=P, **par_kw)
    opar = oracle.mapping_parameters(Npixels=P, **par_kw)
    pos_o = np.array(pos, copy=True, order="F")
    cpar = oracle.center_particles(pos_o, opar)
    rng_o, st_o = oracle.footprints(dims, cpar, pos_o, hsml, q, calc_mean=calc_mean)
    dev = torch.device("cuda:0")
    pos_t = torch.from_numpy(np.ascontiguousarray(pos.T)).to(dev).T  # (3, N), xyz contiguous per particle
    rng_g, st_g = gpu.sph_footprints(pos_t, torch.from_numpy(hsml).to(dev), torch.from_numpy(q).to(dev),
                                     param=par, dimensions=dims, calc_mean=calc_mean)
    rng_g = rng_g.cpu().numpy()
    st_g = st_g.cpu().numpy().astype(np.int8)
    np.testing.assert_array_equal(st_g, st_o)
    mapped = st_o == 2
    lo_o, hi_o = rng_o[:, 0::2], rng_o[:, 1::2]
    hi_o = np.maximum(hi_o, lo_o - 1)  # an empty range as the library reports it
    np.testing.assert_array_equal(rng_g[mapped][:, 0::2], lo_o[mapped])
    np.testing.assert_array_equal(rng_g[mapped][:, 1::2], hi_o[mapped])
    assert not rng_g[~mapped].any()
    return int(mapped.sum())


def test_footprints_uniform_2d_full(gpu, oracle):
    """The 2D projection workload at full size: 2^18 particles, 256^2."""
    d = _synth().uniform_2d()
    n = _check(gpu, oracle, d["pos"], d["hsml"], d["bin_q"], 2, 256, x_lim=[0, 1], y_lim=[0, 1], z_lim=[0, 1])
    assert n > 0.99 * d["hsml"].size


@pytest.mark.parametrize("dims,P", [(2, 64), (3, 32)])
@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_footprints_edges(gpu, oracle, dims, P, dtype):
    """Particles on the image boundaries and pixel edges, far outside it,
    with tiny, zero and huge smoothing lengths, and with all quantities zero
    (skipped unless calc_mean).  Pixel-edge particles whose x -+ h falls on
    an integer pixel coordinate, or one rounding step beside it, and
    smoothing lengths beyond 2^22 pixels are the cases the FP32 range
    computation hands to FP64."""
    rng = np.random.default_rng(3)
    n = 6000
    pos = rng.uniform(-0.2, 1.2, (3, n))
    k = n // 6
    pos[:, :k] = rng.integers(0, P + 1, (3, k)) / P  # pixel edges, the limits included
    pos[0, k:2 * k] = 0.0
    pos[1, 2 * k:3 * k] = 1.0
    hsml = np.exp(rng.uniform(np.log(1e-4), np.log(2.0), n))
    h = k // 3
    hsml[:h] = rng.integers(0, 9, h) / P  # x -+ h on a pixel edge
    hsml[h:2 * h] = np.nextafter(hsml[:h].astype(dtype), np.array(np.inf, dtype)).astype(np.float64)
    hsml[2 * h:3 * h] = np.nextafter(hsml[:h].astype(dtype), np.array(-np.inf, dtype)).astype(np.float64)
    hsml[3 * k:3 * k + 50] = 0.0
    hsml[3 * k + 50:3 * k + 100] = 5.0
    hsml[3 * k + 100:3 * k + 120] = 1e7
    q = rng.uniform(0.5, 2.0, n)
    q[4 * k:4 * k + 300] = 0.0
    args = (np.asfortranarray(pos.astype(dtype)), hsml.astype(dtype), q.astype(dtype), dims, P)
    lim = dict(x_lim=[0, 1], y_lim=[0, 1], z_lim=[0, 1])
    _check(gpu, oracle, *args, **lim)
    if dims == 2:
        _check(gpu, oracle, *args, calc_mean=True, **lim)


def test_footprints_centred_periodic(gpu, oracle):
    """A centred, periodic parameter set: the boxsize/2 shift of
    center_particles (filter_shift.jl:18-21) applies to particles beyond half
    a box."""
    rng = np.random.default_rng(5)
    n = 20000
    pos = np.asfortranarray(rng.uniform(0.0, 1.0, (3, n)))
    hsml = np.exp(rng.uniform(np.log(1e-3), np.log(0.1), n))
    q = rng.uniform(0.5, 2.0, n)
    _check(gpu, oracle, pos, hsml, q, 2, 128, center=[0.3, 0.6, 0.5], x_size=0.5, y_size=0.5, z_size=0.5,
           boxsize=1.0)


def test_footprints_multi_quantity(gpu, oracle):
    """Nq x N quantities: a particle is skipped only when all are zero."""
    rng = np.random.default_rng(7)
    n = 5000
    pos = np.asfortranarray(rng.uniform(0.0, 1.0, (3, n)))
    hsml = np.exp(rng.uniform(np.log(1e-3), np.log(0.05), n))
    q = rng.uniform(0.5, 2.0, (3, n))
    q[:, :400] = 0.0
    q[1, 400:800] = 0.0
    _check(gpu, oracle, pos, hsml, np.ascontiguousarray(q), 2, 96, x_lim=[0, 1], y_lim=[0, 1], z_lim=[0, 1])


def test_footprints_large_hdr(gpu, oracle):
    """The large-particle projection's distribution (hsml over three
    decades, 0.1-200 px) at 2^20 particles on 1024^2, Float32."""
    d = _synth().large_hdr_2d(N=2 ** 20, npix=1024, seed_grid=128)
    n = _check(gpu, oracle, d["pos"], d["hsml"], d["bin_q"], 2, 1024, x_lim=[0, 1], y_lim=[0, 1], z_lim=[0, 1])
    assert n > 0


def test_footprints_clumps_3d(gpu, oracle):
    """The 3D clump workload's distribution at 2^18 particles on 256^3."""
    d = _synth().clumps_3d(N=2 ** 18)
    _check(gpu, oracle, d["pos"], d["hsml"], d["bin_q"], 3, 256, x_lim=[0, 1], y_lim=[0, 1], z_lim=[0, 1])
