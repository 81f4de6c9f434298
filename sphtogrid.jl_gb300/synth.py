"""Seeded synthetic particle sets with the shapes, sizes and value
distributions of the benchmark workloads (no public dataset is involved).

Every generator returns a dict with ``pos`` (3, N) in the Julia memory layout
(x, y, z contiguous per particle), ``hsml``, ``mass``, ``rho``, ``bin_q``
((N,) or (Nq, N)), ``weights`` and the mapping settings (``limits``,
``npix``, ``kernel``, ``dims``).
"""
from __future__ import annotations

import math

import numpy as np


def _julia_pos(p: np.ndarray) -> np.ndarray:
    """(3, N) array whose memory is Julia's 3 x N column-major layout."""
    return np.asfortranarray(p)


def uniform_2d(N=2 ** 18, npix=256, kernel="cubic", seed=0, dtype=np.float64):
    """2D projection workload: positions uniform in the unit cube, hsml
    lognormal (median 0.01, sigma 0.5) clipped to [0.002, 0.1], mass 1/N,
    rho uniform in [0.5, 2], Bin_Quant = Weights = rho."""
    rng = np.random.default_rng(seed)
    pos = rng.random((3, N))
    hsml = np.clip(np.exp(np.log(0.01) + 0.5 * rng.standard_normal(N)), 0.002, 0.1)
    rho = rng.uniform(0.5, 2.0, N)
    d = {
        "pos": _julia_pos(pos.astype(dtype)),
        "hsml": hsml.astype(dtype),
        "mass": np.full(N, 1.0 / N, dtype=dtype),
        "rho": rho.astype(dtype),
    }
    d["bin_q"] = d["rho"]
    d["weights"] = d["rho"]
    d.update(limits=(0.0, 1.0), npix=npix, kernel=kernel, dims=2)
    return d


def _mixture_density(pos, cen, sig, counts, background):
    """Number density of the clump mixture at each position (torch's
    multithreaded elementwise ops on the host when available)."""
    try:
        import torch
    except ImportError:  # pragma: no cover
        torch = None
    amp = counts / (2.0 * math.pi * sig ** 2) ** 1.5
    if torch is not None:
        p = torch.from_numpy(np.ascontiguousarray(pos.T))
        out = torch.full((pos.shape[0],), background, dtype=torch.float64)
        for c in range(cen.shape[0]):
            r2 = (p[0] - cen[c, 0]) ** 2 + (p[1] - cen[c, 1]) ** 2 + (p[2] - cen[c, 2]) ** 2
            out += amp[c] * torch.exp(r2 * (-0.5 / sig[c] ** 2))
        return out.numpy()
    pt = np.ascontiguousarray(pos.T)
    out = np.full(pos.shape[0], background)
    for c in range(cen.shape[0]):
        r2 = (pt[0] - cen[c, 0]) ** 2 + (pt[1] - cen[c, 1]) ** 2 + (pt[2] - cen[c, 2]) ** 2
        out += amp[c] * np.exp(r2 * (-0.5 / sig[c] ** 2))
    return out


def clumps_3d(N=2 ** 22, npix=256, n_clumps=64, seed=0, dtype=np.float32):
    """3D gridding workload: 64 isotropic Gaussian clumps (sigma 0.02-0.08)
    plus a 20% uniform background in the unit cube; hsml = 1.2 (32 / (4 pi/3
    n_local))^(1/3) from the analytic local number density, mass 1/N, rho
    proportional to the local density, Bin_Quant = temperature lognormal
    (median 1e6, sigma 1), WendlandC6, Float32."""
    rng = np.random.default_rng(seed)
    nb = int(0.2 * N)
    nc = N - nb
    cen = rng.random((n_clumps, 3))
    sig = rng.uniform(0.02, 0.08, n_clumps)
    lab = rng.integers(0, n_clumps, nc)
    counts = np.bincount(lab, minlength=n_clumps).astype(np.float64)
    pc = cen[lab] + sig[lab, None] * rng.standard_normal((nc, 3))
    pos = np.concatenate([pc, rng.random((nb, 3))])
    perm = rng.permutation(N)
    pos = pos[perm]
    nloc = _mixture_density(pos, cen, sig, counts, float(nb))
    hsml = 1.2 * (32.0 / (4.0 * math.pi / 3.0 * nloc)) ** (1.0 / 3.0)
    rho = nloc / N  # mass 1/N times number density
    temp = np.exp(np.log(1e6) + rng.standard_normal(N))
    d = {
        "pos": _julia_pos(pos.T.astype(dtype)),
        "hsml": hsml.astype(dtype),
        "mass": np.full(N, 1.0 / N, dtype=dtype),
        "rho": rho.astype(dtype),
        "bin_q": temp.astype(dtype),
    }
    d["weights"] = d["rho"]
    d.update(limits=(0.0, 1.0), npix=npix, kernel="wendlandc6", dims=3)
    return d


def differentiable_2d(N=2 ** 20, npix=512, seed=0, dtype=np.float64):
    """Adjoint workload: as ``uniform_2d`` mapped to 512^2 with WendlandC4."""
    d = uniform_2d(N=N, npix=npix, kernel="wendlandc4", seed=seed, dtype=dtype)
    return d


def batched_2d(n_maps=96, seed=0, dtype=np.float32, n_min=10_000, n_max=2_000_000,
               sizes=(128, 256, 512, 1024)):
    """Batched workload: independent 2D maps with particle counts lognormal
    between n_min and n_max, Npixels drawn from `sizes`, 1-4 quantities (rho,
    temperature lognormal median 1e6, a velocity component Gaussian sigma 300,
    magnetic-field magnitude lognormal), Quintic and WendlandC4 mixed;
    positions and hsml as ``uniform_2d``.  Returns a list of map dicts."""
    rng = np.random.default_rng(seed)
    mu = 0.5 * (math.log(n_min) + math.log(n_max))
    sig = (math.log(n_max) - math.log(n_min)) / 4.0
    maps = []
    for _ in range(n_maps):
        N = int(np.clip(round(math.exp(rng.normal(mu, sig))), n_min, n_max))
        P = int(rng.choice(sizes))
        nq = int(rng.integers(1, 5))
        kernel = str(rng.choice(["quintic", "wendlandc4"]))
        pos = rng.random((3, N))
        hsml = np.clip(np.exp(np.log(0.01) + 0.5 * rng.standard_normal(N)), 0.002, 0.1)
        rho = rng.uniform(0.5, 2.0, N)
        rows = [rho, np.exp(np.log(1e6) + rng.standard_normal(N)), 300.0 * rng.standard_normal(N),
                np.exp(np.log(1e-6) + rng.standard_normal(N))]
        q = np.stack(rows[:nq]) if nq > 1 else rows[0]
        d = {"pos": _julia_pos(pos.astype(dtype)), "hsml": hsml.astype(dtype),
             "mass": np.full(N, 1.0 / N, dtype=dtype), "rho": rho.astype(dtype),
             "bin_q": np.ascontiguousarray(q.astype(dtype)), "weights": rho.astype(dtype),
             "limits": (0.0, 1.0), "npix": P, "kernel": kernel, "dims": 2}
        maps.append(d)
    return maps


def _lognormal_field(ng, sigma_ln, slope, rng):
    """Density field on an ng^3 periodic grid: exp of a Gaussian random field
    with power spectrum P(k) ∝ k^slope, scaled to a standard deviation of
    sigma_ln in ln rho, normalised to mean 1."""
    kx = np.fft.fftfreq(ng) * ng
    kz = np.fft.rfftfreq(ng) * ng
    k2 = kx[:, None, None] ** 2 + kx[None, :, None] ** 2 + kz[None, None, :] ** 2
    amp = np.zeros_like(k2)
    nz = k2 > 0
    amp[nz] = k2[nz] ** (slope / 4.0)  # sqrt(P(k)), P ∝ |k|^slope
    noise = rng.standard_normal((ng, ng, ng // 2 + 1)) + 1j * rng.standard_normal((ng, ng, ng // 2 + 1))
    delta = np.fft.irfftn(noise * amp, s=(ng, ng, ng))
    delta *= sigma_ln / delta.std()
    rho = np.exp(delta)
    return rho / rho.mean()


def large_hdr_2d(N=2 ** 27, npix=4096, seed=0, dtype=np.float32, seed_grid=512, sigma_ln=2.0,
                 slope=-3.0, h_min=1e-4, h_max=0.2, n_ngb=64):
    """Large high-dynamic-range projection: particles in the periodic unit box
    sampled ∝ a log-normal density field (sigma_ln 2, P(k) ∝ k^-3 on a
    seed_grid^3 grid; per-cell counts Poisson with mean N * mass fraction, so
    the total is N up to Poisson noise), positions uniform inside their cell,
    hsml = (3 n_ngb / (4 pi N rho))^(1/3) from the cell's density clipped to
    [h_min, h_max] (three decades), mass 1/N, Bin_Quant = Weights = rho,
    Cubic kernel, 2D map of npix^2 over the unit box."""
    rng = np.random.default_rng(seed)
    rho_c = _lognormal_field(seed_grid, sigma_ln, slope, rng).reshape(-1)
    counts = rng.poisson(N * rho_c / rho_c.sum())
    cell = np.repeat(np.arange(rho_c.size, dtype=np.int64), counts)
    n = cell.size
    g = seed_grid
    ijk = np.stack([cell // (g * g), (cell // g) % g, cell % g]).astype(np.float64)
    pos = (ijk + rng.random((3, n))) / g
    rho = rho_c[cell]
    hsml = np.clip((3.0 * n_ngb / (4.0 * math.pi * n * rho)) ** (1.0 / 3.0), h_min, h_max)
    d = {"pos": _julia_pos(pos.astype(dtype)), "hsml": hsml.astype(dtype),
         "mass": np.full(n, 1.0 / n, dtype=dtype), "rho": rho.astype(dtype)}
    d["bin_q"] = d["rho"]
    d["weights"] = d["rho"]
    d.update(limits=(0.0, 1.0), npix=npix, kernel="cubic", dims=2, boxsize=1.0)
    return d
