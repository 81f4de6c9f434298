"""map_it's projections (cic_interpolation.jl:314-380, rotate_particles.jl,
rotate_parameters.jl): the device reads positions through the projection;
the test restates the reference's steps on the host (copy, permute or
rotate, permute the parameters) and maps the result with the oracle."""
import math
import os

import numpy as np
import pytest

from conftest import rel_linf


def _rot_ref(alpha, beta, gamma):
    """Rx(a) Ry(b) Rz(c) as three matrix products (the definition)."""
    a, b, c = (math.radians(x) for x in (alpha, beta, gamma))
    rx = np.array([[1, 0, 0], [0, math.cos(a), -math.sin(a)], [0, math.sin(a), math.cos(a)]])
    ry = np.array([[math.cos(b), 0, math.sin(b)], [0, 1, 0], [-math.sin(b), 0, math.cos(b)]])
    rz = np.array([[math.cos(c), -math.sin(c), 0], [math.sin(c), math.cos(c), 0], [0, 0, 1]])
    return rx @ ry @ rz


def test_rotation_matrix(pkg):
    for ang in [(0, 0, 0), (30, 45, 60), (-90, 12.5, 270), (180, 90, 0)]:
        R = pkg.rotation_matrix_xyz(*ang)
        assert np.allclose(R, _rot_ref(*ang), rtol=0, atol=4e-16)
        assert np.allclose(R @ R.T, np.eye(3), atol=1e-15)


def test_bad_projection(pkg):
    from sphtogrid_gb300 import mapping
    with pytest.raises(ValueError):
        mapping._projection("zx")
    with pytest.raises(ValueError):
        mapping._projection([1.0, 2.0])
    pr, name = mapping._projection([10, 20, 30])
    assert name == "alpha=10.00beta=20.00gamma=30.00" and pr.kind == 3


def _oracle_projected(oracle, pkg, d, par_kw, projection, calc_mean):
    """The reference's steps on the host: copy, rotate, rotate parameters."""
    pos = np.array(d["pos"], dtype=np.float64 if not isinstance(projection, str) else d["pos"].dtype,
                   order="F", copy=True)
    kw = dict(par_kw)
    cen = list(kw.pop("center"))
    lims = [kw.pop("x_lim"), kw.pop("y_lim"), kw.pop("z_lim")]
    if projection in ("xz", "yz"):
        perm = [0, 2, 1] if projection == "xz" else [1, 2, 0]
        pos = np.asfortranarray(pos[perm, :])
        cen = [cen[k] for k in perm]
        lims = [lims[k] for k in perm]
    elif not isinstance(projection, str):
        R = pkg.rotation_matrix_xyz(*projection)
        x = d["pos"].astype(np.float64)
        pos = np.asfortranarray(np.stack(
            [(R[k, 0] * x[0] + R[k, 1] * x[1]) + R[k, 2] * x[2] for k in range(3)]))
    opar = oracle.mapping_parameters(center=cen, x_lim=lims[0], y_lim=lims[1], z_lim=lims[2], **kw)
    img, info = oracle.sph_mapping(pos.copy(order="F"), d["hsml"], d["m"], d["rho"], d["q"], d["rho"],
                                   param=opar, kernel="wendlandc6", kernel_dim=2, calc_mean=calc_mean)
    raw, _ = oracle.sph_mapping(pos.copy(order="F"), d["hsml"], d["m"], d["rho"], d["q"], d["rho"],
                                param=opar, kernel="wendlandc6", kernel_dim=2, calc_mean=calc_mean,
                                return_both_maps=True)
    return img, raw[:, -1]


def _case(seed, n, dtype):
    rng = np.random.default_rng(seed)
    return {"pos": np.asfortranarray(rng.uniform(-0.6, 0.6, (3, n)).astype(dtype)),
            "hsml": rng.uniform(0.01, 0.1, n).astype(dtype),
            "m": np.full(n, 1.0 / n, dtype=dtype),
            "rho": rng.uniform(0.5, 2.0, n).astype(dtype),
            "q": rng.uniform(0.0, 2.0, n).astype(dtype)}


@pytest.mark.gpu
@pytest.mark.parametrize("projection", ["xy", "xz", "yz", (30.0, 45.0, 60.0)])
@pytest.mark.parametrize("dtype", [np.float32, np.float64])
@pytest.mark.parametrize("precision", ["fp64", "fp32c"])
def test_map_it_matches_oracle(gpu, oracle, tmp_path, projection, dtype, precision):
    d = _case(21, 4000, dtype)
    par_kw = dict(center=[0.05, -0.02, 0.1], x_lim=[-0.5, 0.6], y_lim=[-0.5, 0.6],
                  z_lim=[-0.4, 0.45], Npixels=96)
    ref, W = _oracle_projected(oracle, gpu, d, par_kw, projection, calc_mean=True)
    par = gpu.mappingParameters(**par_kw)
    pos0 = d["pos"].copy(order="F")
    prefix = str(tmp_path / "img")
    img = gpu.map_it(d["pos"], d["hsml"], d["m"], d["rho"], d["q"], d["rho"], param=par,
                     projection=list(projection) if isinstance(projection, tuple) else projection,
                     precision=precision, show_progress=False, image_prefix=prefix)
    assert np.array_equal(d["pos"], pos0)  # the caller's positions are untouched
    if precision == "fp64":
        assert rel_linf(img, ref, 1e-9) <= 1e-11
    else:  # pixels carrying weight (W >= 1e-6 max W), q >= 0
        keep = (W >= 1e-6 * W.max()).reshape(96, 96)  # raw row ix*P + iy -> [ix, iy]
        got = np.asarray(img)[:, :, 0]
        assert rel_linf(got[keep], ref[:, :, 0][keep], 1e-9) <= 1e-5
    name = projection if isinstance(projection, str) else "alpha=30.00beta=45.00gamma=60.00"
    fits = f"{prefix}.{name}.fits"
    assert os.path.exists(fits)
    from sphtogrid_gb300 import io
    got, fpar, _, _ = io.read_fits_image(fits)
    assert np.array_equal(got, np.asarray(img)[:, :, 0])
    # written with the caller's parameters; read_fits_image rebuilds them from
    # the limits alone (io.jl:132-138), so the centre comes back as
    # mappingParameters derives it from the limits (parameters.jl:83-87)
    assert fpar.x_lim == par.x_lim and fpar.y_lim == par.y_lim and fpar.z_lim == par.z_lim
    from_lims = gpu.mappingParameters(x_lim=par_kw["x_lim"], y_lim=par_kw["y_lim"],
                                      z_lim=par_kw["z_lim"], Npixels=par_kw["Npixels"])
    assert fpar.center == from_lims.center
