"""CUDA deposition against the FP64 oracle through the C ABI.

Tolerances (relative L-infinity):
  * precision "fp64": 1e-11 on pixels with |value| > 1e-9 of the map's
    maximum (absolute, relative to the maximum, elsewhere) -- per-pixel weights
    are bitwise those of the oracle, only the order of the FP64 atomic sums
    differs;
  * precision "fp32c": 1e-5 on pixels carrying non-negligible weight: the
    pixel's weight W is at least 1e-6 of the map's largest W (for reduced maps
    Q/W the weight, not the ratio, decides; a pixel reached only by kernel
    tails has FP32 weights whose (1 - u)^k factors carry cancellation).
Integer work (footprints, deposit and particle counts) must match exactly.
"""
import math

import numpy as np
import pytest

from conftest import rel_linf

pytestmark = pytest.mark.gpu

KERNELS = ["cubic", "quintic", "wendlandc4", "wendlandc6", "wendlandc8"]
TOL = {"fp64": 1e-11, "fp32c": 1e-5}
FLOOR = 1e-9


def _case(seed, n, nq=1, dtype=np.float64, spread=0.55, hmin=0.01, hmax=0.3, qneg=False,
          layout="julia"):
    rng = np.random.default_rng(seed)
    pos = rng.uniform(-spread, spread, (3, n)) + np.array([[0.2], [-0.1], [0.3]])
    hsml = np.exp(rng.uniform(np.log(hmin), np.log(hmax), n))
    m = rng.uniform(0.5, 1.5, n) / max(n, 1)
    rho = rng.uniform(0.5, 2.0, n)
    lo = -1.0 if qneg else 0.5
    q = rng.uniform(lo, 2.0, (nq, n)) if nq > 1 else rng.uniform(lo, 2.0, n)
    if n > 4:
        if nq > 1:
            q[:, :2] = 0.0
        else:
            q[:2] = 0.0
    w = rng.uniform(0.5, 2.0, n)
    pos = pos.astype(dtype)
    pos = np.asfortranarray(pos) if layout == "julia" else np.ascontiguousarray(pos)
    c = lambda a: a.astype(dtype)
    return pos, c(hsml), c(m), c(rho), c(q), c(w)


def _params(pkg, oracle, P, boxsize=-1.0):
    kw = dict(center=[0.2, -0.1, 0.3], x_size=1.0, y_size=1.0, z_size=1.0, Npixels=P,
              boxsize=boxsize)
    return pkg.mappingParameters(**kw), oracle.mapping_parameters(**kw)


def _compare(gpu, oracle, case, P, dims, kernel, kdim=None, precision="fp64", tol=None,
             **kw):
    pos, hsml, m, rho, q, w = case
    par, opar = _params(gpu, oracle, P)
    kdim = dims if kdim is None else kdim
    pos_g, pos_o = pos.copy(order="A"), pos.copy(order="A")
    img, st = gpu.sphMapping(pos_g, hsml, m, rho, q, w, param=par,
                             kernel=gpu.kernel_from_name(kernel, kdim), dimensions=dims,
                             precision=precision, show_progress=False, return_stats=True, **kw)
    okw = {k: v for k, v in kw.items() if k != "deterministic"}  # GPU-only option
    ref, info = oracle.sph_mapping(pos_o, hsml, m, rho, q, w, param=opar, kernel=kernel,
                                   kernel_dim=kdim, dimensions=dims, copy_pos=False, **okw)
    # in-place centring is bitwise the reference's (filter_shift.jl:15)
    assert np.array_equal(pos_g, pos_o)
    assert st["deposits"] == info["deposits"]
    limit = TOL[precision] if tol is None else tol
    if precision == "fp64" or img.size == 0:
        err = rel_linf(img, ref, FLOOR)
    else:
        err = _fp32c_error(oracle, case, opar, dims, kernel, kdim, img, ref, **okw)
    assert err <= limit, f"rel L-inf {err:.3e}"
    return img, ref, st, info


def _rows_to_out(rows, P, dims, shape):
    """(PD, k) array on raw rows -> the output layout `shape`."""
    if dims == 2 and len(shape) == 2:
        return rows
    if dims == 2:
        return rows.reshape(P, P, rows.shape[1])
    return rows[:, 0].reshape(P, P, P).transpose(2, 1, 0)


def _fp32c_error(oracle, case, opar, dims, kernel, kdim, img, ref, **kw):
    """Relative L-inf error on pixels carrying weight, each pixel scaled by
    the magnitude of what it sums: the map of |q| (so quantities of both signs
    that cancel in a pixel are judged against the sum of their magnitudes)."""
    pos, hsml, m, rho, q, w = case
    raw, _ = oracle.sph_mapping(pos.copy(order="A"), hsml, m, rho, np.abs(q), w, param=opar,
                                kernel=kernel, kernel_dim=kdim, dimensions=dims,
                                return_both_maps=True, raw3d=True,
                                calc_mean=kw.get("calc_mean", False))
    P = opar.Npixels[0]
    W = raw[:, -1:]
    qa = raw[:, :-1]
    reduce = kw.get("reduce_image", True)
    if dims == 2 and kw.get("return_both_maps"):
        scale = raw
    elif dims == 2:
        scale = np.where((W > 0) & reduce, qa / np.where(W > 0, W, 1.0), qa)
    else:
        scale = np.maximum(qa / np.where(W > 0, W, 1.0), qa) if reduce else qa
    scale = _rows_to_out(scale, P, dims, img.shape)
    keep = _weight_mask(oracle, case, opar, dims, kernel, kdim, img.shape, **kw)
    den = np.maximum(np.abs(ref), scale)
    sel = keep & (den > 0)
    if not sel.any():
        return 0.0
    return float((np.abs(img - ref)[sel] / den[sel]).max())


def _weight_mask(oracle, case, opar, dims, kernel, kdim, shape, floor=1e-6, **kw):
    """Output pixels whose weight W is at least `floor` of the largest W."""
    pos, hsml, m, rho, q, w = case
    raw, _ = oracle.sph_mapping(pos.copy(order="A"), hsml, m, rho, q, w, param=opar,
                                kernel=kernel, kernel_dim=kdim, dimensions=dims,
                                return_both_maps=True, raw3d=True,
                                calc_mean=kw.get("calc_mean", False))
    W = raw[:, -1]
    keep = W >= floor * W.max() if W.size and W.max() > 0 else np.zeros(W.shape, bool)
    P = opar.Npixels[0]
    if dims == 2 and kw.get("return_both_maps"):
        return np.repeat(keep[:, None], shape[1], axis=1)
    if dims == 2:
        k2 = keep.reshape(P, P)  # row ix*P + iy -> [ix, iy]
        return np.repeat(k2[:, :, None], shape[2], axis=2)
    return keep.reshape(P, P, P).transpose(2, 1, 0)  # row ix*P^2+iy*P+iz -> [iz, iy, ix]


@pytest.mark.parametrize("kernel", KERNELS)
@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_2d_kernels_dtypes(gpu, oracle, kernel, dtype):
    _compare(gpu, oracle, _case(1, 3000, dtype=dtype), 48, 2, kernel)


@pytest.mark.parametrize("kernel", KERNELS)
@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_3d_kernels_dtypes(gpu, oracle, kernel, dtype):
    _compare(gpu, oracle, _case(2, 600, dtype=dtype, hmax=0.2), 24, 3, kernel)


@pytest.mark.parametrize("reduce_image", [True, False])
@pytest.mark.parametrize("return_both_maps", [True, False])
@pytest.mark.parametrize("calc_mean", [True, False])
def test_2d_multi_quantity_options(gpu, oracle, reduce_image, return_both_maps, calc_mean):
    _compare(gpu, oracle, _case(3, 2500, nq=3, qneg=True), 40, 2, "wendlandc4",
             reduce_image=reduce_image, return_both_maps=return_both_maps, calc_mean=calc_mean)


@pytest.mark.parametrize("reduce_image", [True, False])
def test_3d_reduce_options(gpu, oracle, reduce_image):
    _compare(gpu, oracle, _case(4, 800, qneg=True), 20, 3, "cubic", reduce_image=reduce_image)


def test_kernel_dim_differs_from_map_dim(gpu, oracle):
    # the 2D bug-fix test of the reference maps with Cubic() (dim 3)
    _compare(gpu, oracle, _case(5, 1500), 32, 2, "cubic", kdim=3)


def test_soa_position_layout(gpu, oracle):
    _compare(gpu, oracle, _case(6, 2000, layout="soa"), 32, 2, "quintic")


def test_fallback_branch_tiny_particles(gpu, oracle):
    # hsml far below a pixel: many particles see no pixel centre (calculate_weights fallback)
    _compare(gpu, oracle, _case(7, 4000, hmin=1e-4, hmax=5e-3), 32, 2, "cubic",
             return_both_maps=True)
    _compare(gpu, oracle, _case(8, 2000, hmin=1e-4, hmax=5e-3), 16, 3, "wendlandc6")


def test_huge_particles_clipped_at_edges(gpu, oracle):
    _compare(gpu, oracle, _case(9, 50, hmin=0.5, hmax=3.0), 64, 2, "wendlandc8",
             return_both_maps=True)
    _compare(gpu, oracle, _case(10, 10, hmin=0.3, hmax=1.5), 24, 3, "cubic")


def test_boundary_particles_inclusive(gpu, oracle):
    # particles exactly on the image edges are inside (filter_shift.jl:50)
    P = 16
    xs = np.array([-0.5, 0.5, 0.5, -0.5, 0.0, 0.5]) + 0.2
    ys = np.array([-0.5, 0.5, -0.5, 0.5, 0.5, 0.0]) - 0.1
    zs = np.array([0.0, 0.5, -0.5, 0.0, 0.0, 0.5000001]) + 0.3
    pos = np.asfortranarray(np.stack([xs, ys, zs]))
    n = pos.shape[1]
    one = np.ones(n)
    _compare(gpu, oracle, (pos, np.full(n, 0.05), one / n, one, one, one), P, 2, "cubic",
             return_both_maps=True)


def test_empty_and_all_filtered(gpu, oracle):
    z = np.zeros(0)
    _compare(gpu, oracle, (np.zeros((3, 0), order="F"), z, z, z, z, z), 8, 2, "cubic")
    _compare(gpu, oracle, (np.zeros((3, 0), order="F"), z, z, z, z, z), 8, 3, "cubic")
    pos = np.asfortranarray(np.full((3, 5), 10.0))
    one = np.ones(5)
    img, _, st, _ = _compare(gpu, oracle, (pos, one, one, one, one, one), 8, 2, "cubic")
    assert st["n_mapped"] == 0 and not img.any()


def test_zero_quantity_skipped(gpu, oracle):
    pos, hsml, m, rho, q, w = _case(11, 500)
    q[:] = 0.0
    img, _, st, _ = _compare(gpu, oracle, (pos, hsml, m, rho, q, w), 16, 2, "cubic",
                             return_both_maps=True)
    assert st["n_mapped"] == 0
    img, _, st, _ = _compare(gpu, oracle, (pos, hsml, m, rho, q, w), 16, 2, "cubic",
                             return_both_maps=True, calc_mean=True)
    assert st["n_mapped"] > 0


def test_periodic_centring(gpu, oracle):
    pos, hsml, m, rho, q, w = _case(12, 1500, spread=1.4)
    P = 24
    kw = dict(center=[0.2, -0.1, 0.3], x_size=1.0, y_size=1.0, z_size=1.0, Npixels=P, boxsize=2.0)
    par, opar = gpu.mappingParameters(**kw), oracle.mapping_parameters(**kw)
    pg, po = pos.copy(order="F"), pos.copy(order="F")
    img = gpu.sphMapping(pg, hsml, m, rho, q, w, param=par, kernel=gpu.Cubic(2),
                         show_progress=False, return_both_maps=True)
    ref, _ = oracle.sph_mapping(po, hsml, m, rho, q, w, param=opar, kernel="cubic",
                                kernel_dim=2, return_both_maps=True, copy_pos=False)
    assert np.array_equal(pg, po)
    assert rel_linf(img, ref, FLOOR) <= TOL["fp64"]


def test_sort_z_selection(gpu, oracle):
    pos, hsml, m, rho, q, w = _case(13, 800, spread=0.6)
    par, opar = _params(gpu, oracle, 24)
    img = gpu.sphMapping(pos.copy(order="F"), hsml, m, rho, q, w, param=par, kernel=gpu.Cubic(2),
                         show_progress=False, sort_z=True, return_both_maps=True)
    ref, _ = oracle.sph_mapping(pos.copy(order="F"), hsml, m, rho, q, w, param=opar,
                                kernel="cubic", kernel_dim=2, sort_z=True, return_both_maps=True)
    assert rel_linf(img, ref, FLOOR) <= TOL["fp64"]


def test_nonfinite_hsml_is_an_error(gpu):
    par = gpu.mappingParameters(x_lim=[0, 1], y_lim=[0, 1], z_lim=[0, 1], Npixels=8)
    pos = np.asfortranarray(np.full((3, 2), 0.5))
    hsml = np.array([0.1, np.nan])
    one = np.ones(2)
    with pytest.raises(gpu.SPHtoGridError) as e:
        gpu.sphMapping(pos, hsml, one, one, one, param=par, kernel=gpu.Cubic(), show_progress=False)
    assert e.value.status == 4
    # a NaN particle with q == 0 is skipped before its range is taken
    pos = np.asfortranarray(np.full((3, 2), 0.5))
    out = gpu.sphMapping(pos, hsml, one, one, np.array([1.0, 0.0]), param=par, kernel=gpu.Cubic(),
                         show_progress=False)
    assert np.isfinite(out).all()


def test_zero_hsml_gives_nan_like_reference(gpu, oracle):
    # hsml = 0: area 0, dz = Inf, 0 * Inf = NaN deposited (cic_2D.jl:80-91,187-199)
    pos = np.asfortranarray(np.array([[0.21], [0.33], [0.5]]))
    one = np.ones(1)
    par, opar = gpu.mappingParameters(x_lim=[0, 1], y_lim=[0, 1], z_lim=[0, 1], Npixels=8), \
        oracle.mapping_parameters(x_lim=[0, 1], y_lim=[0, 1], z_lim=[0, 1], Npixels=8)
    img = gpu.sphMapping(pos.copy(), np.zeros(1), one, one, one, param=par, kernel=gpu.Cubic(),
                         show_progress=False, return_both_maps=True)
    ref, _ = oracle.sph_mapping(pos.copy(), np.zeros(1), one, one, one, param=opar,
                                kernel="cubic", return_both_maps=True)
    assert np.array_equal(np.isnan(img), np.isnan(ref)) and np.isnan(ref).any()


def test_stats_3d_mass_diagnostic(gpu, oracle):
    img, ref, st, info = _compare(gpu, oracle, _case(14, 700), 20, 3, "wendlandc6")
    assert math.isclose(st["grid_mass"], info["grid_mass"], rel_tol=1e-11)


def test_reference_mass_conservation_3d(gpu):
    # runtests.jl:324-342 through the GPU path
    npix, r = 200, 64
    par = gpu.mappingParameters(x_lim=[-r, r], y_lim=[-r, r], z_lim=[-r, r], Npixels=npix)
    pos = np.array([[0.0101], [-0.001], [0.001]])
    w = np.ones(1) * par.pixelSideLength
    img = gpu.sphMapping(pos, np.array([5.0]), np.array([3.0]), np.ones(1), np.ones(1), w,
                         param=par, dimensions=3, kernel=gpu.Cubic(), reduce_image=False,
                         show_progress=False)
    vpix = (par.x_lim[1] - par.x_lim[0]) ** 3 / npix ** 3
    assert math.isclose(vpix * img.sum(), 3.0, rel_tol=1.5e-8)


def test_reference_fallback_2d(gpu):
    # runtests.jl:718-738 through the GPU path
    npix, r = 4, 10
    par = gpu.mappingParameters(x_lim=[-r, r], y_lim=[-r, r], z_lim=[-r, r], Npixels=npix)
    w = np.ones(1) * par.pixelSideLength
    img = gpu.sphMapping(np.array([[0.5], [0.0], [0.0]]), np.ones(1), np.ones(1), np.ones(1),
                         np.ones(1), w, param=par, kernel=gpu.Cubic(), reduce_image=False,
                         show_progress=False)
    apix = (par.x_lim[1] - par.x_lim[0]) ** 2 / npix ** 2
    assert math.isclose(apix * img.sum(), 1.0, rel_tol=1e-10)


def test_device_tensors(gpu, oracle):
    torch = pytest.importorskip("torch")
    pos, hsml, m, rho, q, w = _case(15, 3000, nq=2)
    par, opar = _params(gpu, oracle, 32)
    t = lambda a: torch.as_tensor(np.ascontiguousarray(a), device="cuda")
    tpos = torch.as_tensor(np.ascontiguousarray(pos.T), device="cuda").T  # Julia layout
    img = gpu.sphMapping(tpos, t(hsml), t(m), t(rho), t(q), t(w), param=par,
                         kernel=gpu.WendlandC6(2), show_progress=False)
    pos_o = pos.copy(order="F")
    ref, _ = oracle.sph_mapping(pos_o, hsml, m, rho, q, w, param=opar, kernel="wendlandc6",
                                copy_pos=False)
    assert img.shape == ref.shape
    assert rel_linf(img.cpu().numpy(), ref, FLOOR) <= TOL["fp64"]
    assert np.array_equal(tpos.cpu().numpy(), pos_o)  # centred in place on the device


def test_uniform_2d_workload_full_size(gpu, oracle):
    """The 2D projection workload (N = 2^18, 256^2, Cubic) against the oracle."""
    from sphtogrid_gb300 import synth
    d = synth.uniform_2d()
    par = gpu.mappingParameters(x_lim=[0, 1], y_lim=[0, 1], z_lim=[0, 1], Npixels=256)
    opar = oracle.mapping_parameters(x_lim=[0, 1], y_lim=[0, 1], z_lim=[0, 1], Npixels=256)
    img, st = gpu.sphMapping(d["pos"].copy(order="F"), d["hsml"], d["mass"], d["rho"], d["bin_q"],
                             d["weights"], param=par, kernel=gpu.Cubic(2), show_progress=False,
                             return_stats=True)
    ref, info = oracle.sph_mapping(d["pos"].copy(order="F"), d["hsml"], d["mass"], d["rho"],
                                   d["bin_q"], d["weights"], param=opar, kernel="cubic",
                                   kernel_dim=2)
    assert st["deposits"] == info["deposits"]
    assert rel_linf(img, ref, FLOOR) <= TOL["fp64"]


def test_clumps_3d_mass_conservation_full_size(gpu):
    """3D workload (N = 2^22 Float32, 256^3, WendlandC6): with weights = pixel
    side and q = rho, V_pix * sum(map) equals the mapped mass (cic_3D.jl:168-179
    closed form)."""
    from sphtogrid_gb300 import synth
    d = synth.clumps_3d()
    par = gpu.mappingParameters(x_lim=[0, 1], y_lim=[0, 1], z_lim=[0, 1], Npixels=256)
    w = np.full(d["rho"].shape, par.pixelSideLength, dtype=np.float64)
    img, st = gpu.sphMapping(d["pos"].copy(order="F"), d["hsml"], d["mass"], d["rho"], d["rho"], w,
                             param=par, kernel=gpu.WendlandC6(3), dimensions=3,
                             reduce_image=False, show_progress=False, return_stats=True)
    vpix = par.pixelSideLength ** 3
    assert math.isclose(vpix * img.sum(), st["particle_mass"], rel_tol=1e-9)
    assert st["n_mapped"] > 0.85 * 2 ** 22


# --------------------------------------------------------------- FP32C path

@pytest.mark.parametrize("kernel", KERNELS)
@pytest.mark.parametrize("dims", [2, 3])
def test_fp32c_kernels(gpu, oracle, kernel, dims):
    if dims == 2:
        _compare(gpu, oracle, _case(21, 3000), 48, 2, kernel, precision="fp32c")
    else:
        _compare(gpu, oracle, _case(22, 800, hmax=0.2), 24, 3, kernel, precision="fp32c")


@pytest.mark.parametrize("nq", [1, 2, 3, 4, 6])
@pytest.mark.parametrize("return_both_maps", [True, False])
def test_fp32c_multi_quantity(gpu, oracle, nq, return_both_maps):
    _compare(gpu, oracle, _case(23 + nq, 2500, nq=nq), 40, 2, "wendlandc4", precision="fp32c",
             return_both_maps=return_both_maps, reduce_image=True)


def test_fp32c_reduce_and_mean_options(gpu, oracle):
    _compare(gpu, oracle, _case(30, 2500, nq=2), 40, 2, "quintic", precision="fp32c",
             reduce_image=False, calc_mean=True)
    _compare(gpu, oracle, _case(31, 800), 20, 3, "cubic", precision="fp32c", reduce_image=False)


def test_fp32c_float32_inputs(gpu, oracle):
    _compare(gpu, oracle, _case(32, 3000, dtype=np.float32), 48, 2, "cubic", precision="fp32c")
    _compare(gpu, oracle, _case(33, 800, dtype=np.float32, hmax=0.2), 24, 3, "wendlandc6",
             precision="fp32c")


def test_fp32c_tiny_particles_take_the_fp64_branch(gpu, oracle):
    # sub-pixel particles: the fallback selection must match the reference's
    _compare(gpu, oracle, _case(34, 4000, hmin=1e-4, hmax=5e-3), 32, 2, "cubic",
             precision="fp32c", return_both_maps=True)
    _compare(gpu, oracle, _case(35, 2000, hmin=1e-4, hmax=5e-3), 16, 3, "wendlandc6",
             precision="fp32c")


def test_fp32c_edges_and_empty(gpu, oracle):
    _compare(gpu, oracle, _case(36, 50, hmin=0.5, hmax=3.0), 64, 2, "wendlandc8",
             precision="fp32c", return_both_maps=True)
    _compare(gpu, oracle, _case(37, 10, hmin=0.3, hmax=1.5), 24, 3, "cubic", precision="fp32c")
    z = np.zeros(0)
    _compare(gpu, oracle, (np.zeros((3, 0), order="F"), z, z, z, z, z), 8, 2, "cubic",
             precision="fp32c")
    pos = np.asfortranarray(np.full((3, 5), 10.0))
    one = np.ones(5)
    _compare(gpu, oracle, (pos, one, one, one, one, one), 8, 3, "cubic", precision="fp32c")


def test_fp32c_odd_image_sizes(gpu, oracle):
    # image sides that are not multiples of the tile sides
    _compare(gpu, oracle, _case(38, 2000), 37, 2, "cubic", precision="fp32c")
    _compare(gpu, oracle, _case(39, 600, hmax=0.2), 19, 3, "wendlandc4", precision="fp32c")


def test_fp32c_pair_list_regrowth(gpu, oracle):
    # many large particles -> more (particle, tile) pairs than the first guess
    _compare(gpu, oracle, _case(40, 400, hmin=0.2, hmax=0.6), 96, 2, "cubic", precision="fp32c",
             return_both_maps=True)


def test_fp32c_uniform_2d_workload_full_size(gpu, oracle):
    from sphtogrid_gb300 import synth
    d = synth.uniform_2d()
    par = gpu.mappingParameters(x_lim=[0, 1], y_lim=[0, 1], z_lim=[0, 1], Npixels=256)
    opar = oracle.mapping_parameters(x_lim=[0, 1], y_lim=[0, 1], z_lim=[0, 1], Npixels=256)
    img, st = gpu.sphMapping(d["pos"].copy(order="F"), d["hsml"], d["mass"], d["rho"], d["bin_q"],
                             d["weights"], param=par, kernel=gpu.Cubic(2), show_progress=False,
                             precision="fp32c", return_stats=True)
    ref, info = oracle.sph_mapping(d["pos"].copy(order="F"), d["hsml"], d["mass"], d["rho"],
                                   d["bin_q"], d["weights"], param=opar, kernel="cubic",
                                   kernel_dim=2)
    assert st["deposits"] == info["deposits"]
    assert rel_linf(img, ref, FLOOR) <= TOL["fp32c"]


def test_fp32c_clumps_3d_full_size(gpu, oracle):
    """3D workload at full size: FP32C against the oracle (all host threads)
    and against the plain FP64 GPU method, and mass conservation."""
    import os
    from sphtogrid_gb300 import synth
    d = synth.clumps_3d()
    par = gpu.mappingParameters(x_lim=[0, 1], y_lim=[0, 1], z_lim=[0, 1], Npixels=256)
    args = (d["hsml"], d["mass"], d["rho"], d["bin_q"], d["weights"])
    a, sa = gpu.sphMapping(d["pos"].copy(order="F"), *args, param=par, kernel=gpu.WendlandC6(3),
                           dimensions=3, show_progress=False, precision="fp32c", return_stats=True)
    b, sb = gpu.sphMapping(d["pos"].copy(order="F"), *args, param=par, kernel=gpu.WendlandC6(3),
                           dimensions=3, show_progress=False, precision="fp64", return_stats=True)
    assert sa["deposits"] == sb["deposits"] and sa["n_mapped"] == sb["n_mapped"]
    assert rel_linf(a, b, FLOOR) <= TOL["fp32c"]
    assert math.isclose(sa["grid_mass"], sb["grid_mass"], rel_tol=1e-5)
    opar = oracle.mapping_parameters(x_lim=[0, 1], y_lim=[0, 1], z_lim=[0, 1], Npixels=256)
    ref, info = oracle.sph_mapping(d["pos"].copy(order="F"), *args, param=opar, kernel="wendlandc6",
                                   dimensions=3, nthreads=os.cpu_count() or 1)
    assert info["deposits"] == sa["deposits"]
    assert rel_linf(a, ref, FLOOR) <= TOL["fp32c"]


# ------------------------------------------------------- deterministic mode

@pytest.mark.parametrize("dims", [2, 3])
def test_deterministic_mode_is_bitwise_reproducible(gpu, oracle, dims):
    case = _case(41, 3000 if dims == 2 else 900, nq=2 if dims == 2 else 1, qneg=True)
    P = 40 if dims == 2 else 20
    kw = dict(precision="fp32c", deterministic=True)
    if dims == 2:
        kw["return_both_maps"] = True
    a, _, sa, _ = _compare(gpu, oracle, case, P, dims, "wendlandc4", **kw)
    b, _, sb, _ = _compare(gpu, oracle, case, P, dims, "wendlandc4", **kw)
    assert np.array_equal(a, b)  # same bits, whatever the atomic order


def test_deterministic_full_size_2d(gpu, oracle):
    from sphtogrid_gb300 import synth
    d = synth.uniform_2d()
    par = gpu.mappingParameters(x_lim=[0, 1], y_lim=[0, 1], z_lim=[0, 1], Npixels=256)
    outs = []
    for _ in range(2):
        outs.append(gpu.sphMapping(d["pos"].copy(order="F"), d["hsml"], d["mass"], d["rho"],
                                   d["bin_q"], d["weights"], param=par, kernel=gpu.Cubic(2),
                                   show_progress=False, precision="fp32c", deterministic=True))
    assert np.array_equal(outs[0], outs[1])
    opar = oracle.mapping_parameters(x_lim=[0, 1], y_lim=[0, 1], z_lim=[0, 1], Npixels=256)
    ref, _ = oracle.sph_mapping(d["pos"].copy(order="F"), d["hsml"], d["mass"], d["rho"],
                                d["bin_q"], d["weights"], param=opar, kernel="cubic", kernel_dim=2)
    assert rel_linf(outs[0], ref, FLOOR) <= TOL["fp32c"]


@pytest.mark.parametrize("on_device", [False, True])
@pytest.mark.parametrize("det", [False, True])
def test_overflow_rerun_centres_once(gpu, oracle, on_device, det):
    """A fresh context's tile-pair list is sized for 8 pairs per particle;
    particles of h = 0.3 on a 256^2 map overlap ~100 tiles each, so the first
    pass overflows and the map is run again with a grown list.  The re-run
    must give the oracle's map and leave the caller's positions centred once
    (SPHG_CENTER_INPLACE), for host and device inputs."""
    import torch
    rng = np.random.default_rng(11)
    n = 1500
    pos = np.asfortranarray(rng.uniform(2.0, 4.0, (3, n)))
    hsml = np.full(n, 0.3)
    m = rng.uniform(0.5, 1.5, n) / n
    rho = rng.uniform(0.5, 2.0, n)
    q = rng.uniform(0.5, 2.0, n)
    kw = dict(center=[3.0, 3.0, 3.0], x_size=2.0, y_size=2.0, z_size=2.0, Npixels=256)
    opar = oracle.mapping_parameters(**kw)
    ref, info = oracle.sph_mapping(pos, hsml, m, rho, q, rho, param=opar, kernel="cubic",
                                   copy_pos=True)
    centred = pos.copy(order="F")
    oracle.center_particles(centred, opar)
    ctx = gpu.Context(0)
    try:
        p_in = pos.copy(order="F")
        args = [hsml, m, rho, q, rho]
        if on_device:
            dev = torch.device("cuda", 0)
            p_in = torch.from_numpy(np.ascontiguousarray(pos.T)).to(dev).T
            args = [torch.from_numpy(a).to(dev) for a in args]
        img, st = gpu.sphMapping(p_in, *args, param=gpu.mappingParameters(**kw),
                                 kernel=gpu.Cubic(2), precision="fp32c", deterministic=det,
                                 show_progress=False, return_stats=True, context=ctx)
    finally:
        ctx.close()
    assert st["n_reruns"] >= 1
    assert st["deposits"] == info["deposits"]
    img = img.cpu().numpy() if hasattr(img, "cpu") else img
    assert rel_linf(img, ref, 1e-9) <= 1e-5
    got_pos = p_in.cpu().numpy() if hasattr(p_in, "cpu") else p_in
    assert np.array_equal(got_pos, centred)
