"""Golden fixtures (tests/golden/, made by make_golden.py): the oracle must
reproduce them bit for bit; the GPU paths must match them within their
tolerances (FP64 1e-11, FP32C 1e-5 on pixels carrying weight)."""
import glob
import math
import os

import numpy as np
import pytest

from conftest import rel_linf

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
MAPS = sorted(os.path.basename(f)[:-4] for f in glob.glob(os.path.join(HERE, "map*.npz")))


def _load(name):
    return dict(np.load(os.path.join(HERE, name + ".npz")))


def _par(mod, P):
    return mod(center=[0.0, 0.0, 0.0], x_size=1.0, y_size=1.0, z_size=1.0, Npixels=P)


def test_fixtures_present():
    assert len(MAPS) == 7
    assert os.path.exists(os.path.join(HERE, "kat_fallback_2d.npz"))


@pytest.mark.parametrize("name", MAPS)
def test_oracle_reproduces_fixture(oracle, name):
    d = _load(name)
    dims = 2 if name.startswith("map2d") else 3
    kernel = name.split("_")[1]
    P = int(d["P"])
    par = _par(oracle.mapping_parameters, P)
    raw, info = oracle.sph_mapping(d["pos"], d["hsml"], d["m"], d["rho"], d["q"], d["w"], param=par,
                                   kernel=kernel, dimensions=dims, return_both_maps=True, raw3d=True)
    assert np.array_equal(raw, d["raw"])
    assert info["deposits"] == int(d["deposits"])


def test_known_answers(oracle):
    img = _load("kat_fallback_2d")["image"]
    assert math.isclose(img.sum() * (20.0 / 4) ** 2, 1.0, rel_tol=1e-10)
    k = _load("kat_mass_3d")
    assert math.isclose(k["value"].sum() * (128.0 / 200) ** 3, 3.0, rel_tol=1.5e-8)


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "fp32c"])
@pytest.mark.parametrize("name", MAPS)
def test_gpu_matches_fixture(gpu, name, precision):
    d = _load(name)
    dims = 2 if name.startswith("map2d") else 3
    kernel = name.split("_")[1]
    P = int(d["P"])
    par = _par(gpu.mappingParameters, P)
    raw = gpu.sphMapping(d["pos"].copy(order="F"), d["hsml"], d["m"], d["rho"], d["q"], d["w"],
                         param=par, kernel=gpu.kernel_from_name(kernel, dims), dimensions=dims,
                         return_both_maps=True, precision=precision, show_progress=False) \
        if dims == 2 else None
    red = gpu.sphMapping(d["pos"].copy(order="F"), d["hsml"], d["m"], d["rho"], d["q"], d["w"],
                         param=par, kernel=gpu.kernel_from_name(kernel, dims), dimensions=dims,
                         precision=precision, show_progress=False)
    if precision == "fp64":
        if raw is not None:
            assert rel_linf(raw, d["raw"], 1e-9) <= 1e-11
        assert rel_linf(red, d["reduced"], 1e-9) <= 1e-11
        return
    # FP32C: on pixels carrying weight (W >= 1e-6 max W), the error relative
    # to the magnitude the pixel sums (the map of |q|), so that quantities of
    # both signs cancelling in a pixel are judged against their magnitudes
    W = d["raw"][:, -1]
    keep = W >= 1e-6 * W.max()
    absq = d["raw_absq"]
    Wa = absq[:, -1:]
    if raw is not None:
        assert _scaled_err(raw[keep], d["raw"][keep], absq[keep]) <= 1e-5
    if dims == 2:
        k2 = np.repeat(keep.reshape(P, P)[:, :, None], red.shape[2], axis=2)
        mean = absq[:, :-1] / np.where(Wa > 0, Wa, 1.0)
        scale = np.where(Wa > 0, mean, absq[:, :-1]).reshape(P, P, -1)
    else:
        k2 = keep.reshape(P, P, P).transpose(2, 1, 0)
        qa = absq[:, :1]
        scale = np.maximum(qa / np.where(Wa > 0, Wa, 1.0), qa)[:, 0].reshape(P, P, P).transpose(2, 1, 0)
    assert _scaled_err(red[k2], d["reduced"][k2], scale[k2]) <= 1e-5


def _scaled_err(got, ref, scale):
    den = np.maximum(np.abs(ref), scale)
    sel = den > 0
    return float((np.abs(got - ref)[sel] / den[sel]).max()) if sel.any() else 0.0
