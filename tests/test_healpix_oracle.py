"""The HEALPix oracle (of the all-sky path): the ring-scheme
pixel functions against the known pixel centres of Gorski et al. 2005 and
self-consistency, the disc query against a brute-force search over all pixel
centres, and healpix_map's conservation of the particles' weight."""
import math

import numpy as np
import pytest


def test_pixel_centres_nside1(oracle):
    # 12 base pixels: rings at z = 2/3, 0, -2/3; phi = pi/4 + k pi/2, k pi/2, pi/4 + k pi/2
    for k in range(12):
        v = oracle.hp_pix2vec(1, k)
        ring, j = divmod(k, 4)
        z = (2.0 / 3.0, 0.0, -2.0 / 3.0)[ring]
        phi = (math.pi / 4 if ring != 1 else 0.0) + j * math.pi / 2
        s = math.sqrt(1.0 - z * z)
        assert np.allclose(v, [s * math.cos(phi), s * math.sin(phi), z], atol=1e-15)


@pytest.mark.parametrize("nside", [1, 2, 4, 8, 16])
def test_pixel_roundtrip(oracle, nside):
    npix = 12 * nside * nside
    zs = []
    for p in range(npix):
        v = oracle.hp_pix2vec(nside, p)
        assert abs(np.linalg.norm(v) - 1.0) < 1e-14
        t, f = oracle.hp_vec2ang(*v)
        assert oracle.hp_ang2pix(nside, t, f) == p  # a pixel contains its centre
        zs.append(v[2])
    assert np.all(np.diff(zs) <= 1e-15)  # RING ordering: z non-increasing


@pytest.mark.parametrize("nside", [4, 8, 16])
def test_query_disc_brute_force(oracle, nside):
    rng = np.random.default_rng(nside)
    npix = 12 * nside * nside
    centres = np.array([oracle.hp_pix2vec(nside, p) for p in range(npix)])
    for _ in range(40):
        theta = math.acos(rng.uniform(-1, 1))
        phi = rng.uniform(0, 2 * math.pi)
        radius = rng.uniform(0.01, 1.2)
        got = oracle.hp_query_disc(nside, theta, phi, radius)
        assert len(set(got.tolist())) == len(got)
        d = np.array([math.sin(theta) * math.cos(phi), math.sin(theta) * math.sin(phi), math.cos(theta)])
        ang = np.arccos(np.clip(centres @ d, -1, 1))
        inside = set(np.nonzero(ang < radius - 1e-12)[0].tolist())
        outside = set(np.nonzero(ang > radius + 1e-12)[0].tolist())
        assert inside <= set(got.tolist())
        assert not (outside & set(got.tolist()))


def test_query_disc_poles(oracle):
    nside = 8
    npix = 12 * nside * nside
    for theta in (0.05, math.pi - 0.05):
        got = set(oracle.hp_query_disc(nside, theta, 1.0, 0.3).tolist())
        centres = np.array([oracle.hp_pix2vec(nside, p) for p in range(npix)])
        d = np.array([math.sin(theta) * math.cos(1.0), math.sin(theta) * math.sin(1.0), math.cos(theta)])
        ang = np.arccos(np.clip(centres @ d, -1, 1))
        assert got == set(np.nonzero(ang <= 0.3)[0].tolist())


def _shell_case(seed, n):
    rng = np.random.default_rng(seed)
    r = rng.uniform(2.0, 6.0, n)
    v = rng.standard_normal((3, n))
    v /= np.linalg.norm(v, axis=0)
    pos = np.asfortranarray(v * r + np.array([[0.5], [-0.3], [0.2]]))
    hsml = rng.uniform(0.05, 0.6, n)
    m = rng.uniform(0.5, 1.5, n)
    rho = rng.uniform(0.5, 2.0, n)
    q = rng.uniform(0.5, 2.0, n)
    return pos, hsml, m, rho, q, rho.copy()


def test_healpix_map_conserves_weight(oracle):
    """Each mapped particle adds w * area * dz over its pixels (the
    renormalisation), so the weight map sums to sum(w * m / rho /
    (ang_pix dx)^2) over the mapped particles."""
    pos, h, m, rho, q, w = _shell_case(3, 400)
    nside = 16
    allsky, wmap, info = oracle.healpix_map(pos, h, m, rho, q, w, center=[0.5, -0.3, 0.2],
                                            radius_limits=[0.0, np.inf], Nside=nside)
    assert info["mapped"] == 400  # every particle is farther than its hsml
    p = pos  # centred in place, as the reference does
    dx = np.sqrt(p[0] ** 2 + p[1] ** 2 + p[2] ** 2)
    ang_pix = math.sqrt(4 * math.pi / (12 * nside * nside))
    expect = np.sum(w * m / rho / (ang_pix * dx) ** 2)
    assert math.isclose(wmap.sum(), expect, rel_tol=1e-12)
    assert math.isclose(allsky.sum(), np.sum(q * w * m / rho / (ang_pix * dx) ** 2), rel_tol=1e-12)


def test_healpix_selection_quirk(oracle):
    """filter_sort_particles indexes the distance-sorted permutation with the
    input-order shell mask (filter_particles.jl:42-46)."""
    pos = np.asfortranarray(np.array([[1.0, 5.0, 3.0], [0.0, 0.0, 0.0], [0.0, 0.0, 0.0]]))
    one = np.ones(3)
    sel = oracle.filter_sort_particles(pos.copy(), one, one, one, one * np.array([1.0, 2.0, 3.0]), one,
                                       [0.0, 0.0, 0.0], [2.0, 4.0], True)
    # mask (input order) = [F, F, T]; sorted (descending r) = [1, 2, 0] -> picks particle 0
    assert sel[4].tolist() == [1.0]
