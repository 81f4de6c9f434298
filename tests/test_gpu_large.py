"""Large high-dynamic-range projection (the large-particle workload): a
log-normal density field, hsml over three decades up to 0.2 of the box, so
the largest particles cover ~10^5 pixels and take the two-phase
renormalisation spread over many CTAs.  Reduced here to N = 2^22 particles
on a 1024^2 map (the full workload is 2^27 particles on 4096^2); checked
against the FP64 oracle on the same inputs."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def workload(gpu):
    from sphtogrid_gb300 import synth
    return synth.large_hdr_2d(N=2 ** 22, npix=1024, seed_grid=128, seed=1)


@pytest.fixture(scope="module")
def reference(oracle, workload):
    d = workload
    par = oracle.mapping_parameters(x_lim=[0, 1], y_lim=[0, 1], z_lim=[0, 1], Npixels=d["npix"])
    raw, info = oracle.sph_mapping(d["pos"], d["hsml"], d["mass"], d["rho"], d["bin_q"], d["weights"],
                                   param=par, kernel="cubic", return_both_maps=True, copy_pos=True)
    return raw, info


def _map(gpu, d, **kw):
    par = gpu.mappingParameters(x_lim=[0, 1], y_lim=[0, 1], z_lim=[0, 1], Npixels=d["npix"])
    return gpu.sphMapping(d["pos"].copy(order="F"), d["hsml"], d["mass"], d["rho"], d["bin_q"],
                          d["weights"], param=par, kernel=gpu.Cubic(2), return_both_maps=True,
                          show_progress=False, return_stats=True, **kw)


def _err(got, raw):
    W = raw[:, -1]
    keep = W >= 1e-6 * W.max()
    return float((np.abs(got[keep] - raw[keep]) / np.abs(raw[keep])).max())


def test_large_particles_present(workload):
    h = workload["hsml"].astype(np.float64) * workload["npix"]
    assert h.max() > 150.0  # footprints of ~10^5 pixels: above every large_cells setting
    assert h.min() < 2.0


@pytest.mark.parametrize("precision,det", [("fp32c", False), ("fp32c", True), ("fp64", False)])
def test_large_hdr_matches_oracle(gpu, workload, reference, precision, det):
    raw, info = reference
    got, st = _map(gpu, workload, precision=precision, deterministic=det)
    assert st["deposits"] == info["deposits"]  # integer footprints bit-exact
    err = _err(np.asarray(got), raw)
    assert err <= (1e-11 if precision == "fp64" else 1e-5), err
