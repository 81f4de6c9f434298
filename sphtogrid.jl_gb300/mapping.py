"""``sphMapping``: the reference's entry point (SPHtoGrid.jl
src/cic_interpolation/cic_interpolation.jl:35-272) over the CUDA library.

Host (numpy) inputs go through the C ABI's host path (copies in, map, copy
out); CUDA tensors (torch) are mapped in place on their device.  Layouts and
results follow the reference:

* ``Pos`` is (3, N); it is centred IN PLACE on ``param.center`` as the
  reference does (filter_shift.jl:15).
* ``Bin_Quant`` is (N,) or (Nq, N) (2D maps only take Nq > 1).
* 2D returns an array of shape (P, P, Nq) indexed ``[x, y, q]``; with
  ``return_both_maps`` the raw (P*P, Nq+1) accumulator (row ``i*P + j``,
  columns Q_1..Q_Nq, W); 3D returns (P, P, P) indexed ``[z, y, x]``.  Arrays
  are Fortran-ordered so their memory is the Julia array's memory.
* ``dimensions`` other than 2 or 3 centres the positions and returns None.
"""
from __future__ import annotations

import ctypes as C
import logging
import math
import time

import numpy as np

from . import _lib
from .parameters import MappingParameters, SPHKernel

log = logging.getLogger("sphtogrid_gb300")

_np_dt = {np.dtype(np.float32): _lib.SPHG_F32, np.dtype(np.float64): _lib.SPHG_F64}

def _is_torch_cuda(x) -> bool:
    return type(x).__module__.startswith("torch") and getattr(x, "is_cuda", False)

def _center_numpy(pos: np.ndarray, param: MappingParameters) -> None:
    """center_particles (filter_shift.jl:6-32) on a host array, in place."""
    cen = np.asarray(param.center, dtype=np.float64)
    v = pos.astype(np.float64) - cen[:, None]
    v = v.astype(pos.dtype).astype(np.float64)
    if param.periodic:
        half = param.boxsize / 2
        big = np.abs(v) > half
        v = np.where(big, np.where(v > 0, v - half, v + half), v)
    pos[...] = v.astype(pos.dtype)

def _options(param, kernel: SPHKernel, dims, reduce_image, return_both_maps, calc_mean, precision,
             deterministic, center, filt, memspace):
    o = _lib.SphgOptions()
    o.dimensions = dims
    o.kernel = kernel.kind
    o.kernel_dim = kernel.dim
    o.reduce_image = int(bool(reduce_image))
    o.return_both_maps = int(bool(return_both_maps))
    o.calc_mean = int(bool(calc_mean))
    if precision not in _lib.PREC:
        raise ValueError(f"precision must be one of {sorted(_lib.PREC)}")
    o.precision = _lib.PREC[precision]
    o.deterministic = int(bool(deterministic))
    o.center = center
    o.filter = int(filt)
    o.memspace = memspace
    return o

def _shape_out(flat, P, nq, dims, raw):
    if dims == 2 and raw:
        shape = (P * P, nq + 1)
    elif dims == 2:
        shape = (P, P, nq)
    else:
        shape = (P, P, P)
    if isinstance(flat, np.ndarray):
        return flat.reshape(shape, order="F")
    strides, s = [], 1
    for d in shape:
        strides.append(s)
        s *= d
    return flat.as_strided(shape, tuple(strides))

def _stats_dict(st: _lib.SphgStats):
    return {"n_in": st.n_in, "n_mapped": st.n_mapped, "deposits": st.deposits,
            "grid_mass": st.grid_mass, "particle_mass": st.particle_mass,
            "centred_param": MappingParameters(_lib.SphgParams.from_buffer_copy(st.centred)),
            "n_launches": st.n_launches, "n_reruns": st.n_reruns,
            "phase_ms": list(st.phase_ms)}

def sphMapping(Pos, HSML, M, Rho, Bin_Quant, Weights=None, RM=None, *, param: MappingParameters,
               kernel: SPHKernel, show_progress: bool = True, parallel: bool = False,
               reduce_image: bool = True, return_both_maps: bool = False, dimensions: int = 2,
               calc_mean: bool = False, stokes: bool = False, sort_z: bool = False,
               precision: str = "fp64", deterministic: bool = False, device: int = 0,
               return_stats: bool = False, center_in_place: bool = True, context=None):
    """Map particle quantities to a 2D projected or 3D gridded image.

    Arguments and keywords are those of the reference; ``parallel`` is
    accepted and ignored (one GPU maps everything).  Extra keywords:
    ``precision`` ("fp64": the reference's arithmetic; "fp32c": FP32 weights
    with compensated sums), ``deterministic`` (bitwise reproducible sums),
    ``device`` (host inputs: which GPU), ``return_stats`` (also return a dict
    with particle / deposit counts and the 3D mass diagnostic),
    ``center_in_place`` (False: centre on the fly and leave ``Pos`` as it is),
    ``context`` (a ``Context`` to map in instead of the device's default one).
    """
    if RM is not None or stokes:
        raise NotImplementedError(
            "Faraday rotation / Stokes mapping (cic_shared.jl:129-159) is not supported")
    if Weights is None:
        Weights = Rho
    t0 = time.perf_counter()
    if dimensions not in (2, 3):
        # the reference centres and filters, then returns `nothing`
        if isinstance(Pos, np.ndarray):
            _center_numpy(Pos, param)
        return None
    on_device = _is_torch_cuda(Pos)
    if on_device:
        out = _map_torch(Pos, HSML, M, Rho, Bin_Quant, Weights, param, kernel, reduce_image,
                         return_both_maps, dimensions, calc_mean, sort_z, precision, deterministic,
                         center_in_place, context)
    else:
        out = _map_numpy(Pos, HSML, M, Rho, Bin_Quant, Weights, param, kernel, reduce_image,
                         return_both_maps, dimensions, calc_mean, sort_z, precision, deterministic,
                         device, center_in_place, context)
    image, stats = out
    if show_progress:
        log.info("sphMapping: %d / %d particles mapped, %d deposits, %.3f s",
                 stats["n_mapped"], stats["n_in"], stats["deposits"], time.perf_counter() - t0)
    return (image, stats) if return_stats else image

def _map_numpy(Pos, HSML, M, Rho, Bin_Quant, Weights, param, kernel, reduce_image, return_both_maps,
               dims, calc_mean, sort_z, precision, deterministic, device, center_in_place=True,
               context=None, projection=None):
    if not isinstance(Pos, np.ndarray) or Pos.ndim != 2 or Pos.shape[0] != 3:
        raise ValueError("Pos must be a (3, N) array")
    n = Pos.shape[1]
    pos = Pos
    writeback = None
    es = pos.itemsize
    if (pos.dtype not in _np_dt or any(s < 0 or s % es for s in pos.strides)
            or not pos.flags.writeable):
        pos = np.array(Pos, dtype=np.float64 if pos.dtype not in _np_dt else pos.dtype, order="F")
        writeback = Pos if Pos.flags.writeable else None
    attrs = [np.asarray(a) for a in (HSML, M, Rho, Weights)]
    q = np.asarray(Bin_Quant)
    adt = np.float32 if all(a.dtype == np.float32 for a in attrs + [q]) else np.float64
    hsml, m, rho, w = [np.ascontiguousarray(a, dtype=adt).reshape(-1) for a in attrs]
    q = np.asarray(q, dtype=adt)
    if q.ndim == 1:
        nq = 1
    elif q.ndim == 2:
        nq = q.shape[0]
    else:
        raise ValueError("Bin_Quant must be (N,) or (Nq, N)")
    if q.strides and any(s < 0 or s % q.itemsize for s in q.strides):
        q = np.ascontiguousarray(q)
    for a in (hsml, m, rho, w):
        if a.shape[0] != n:
            raise ValueError("particle arrays must have N entries")
    if q.shape[-1] != n:
        raise ValueError("Bin_Quant must have N columns")
    center_mode = _lib.CENTER_INPLACE if center_in_place else _lib.CENTER_READONLY
    filt = 1
    if sort_z:
        # filter_shift.jl:61-63: z-sorted (descending) index list, selected by
        # the mask in input order -- the reference's selection, kept as is.
        _center_numpy(pos, param)
        cpar = _centred_params(param)
        lo = np.asarray(cpar.center) - np.asarray(cpar.halfsize)
        hi = np.asarray(cpar.center) + np.asarray(cpar.halfsize)
        p64 = pos.astype(np.float64)
        mask = np.all((lo[:, None] <= p64) & (p64 <= hi[:, None]), axis=0)
        order = np.argsort(p64[2], kind="stable")[::-1]
        sel = order[mask]
        pos_sel = np.asfortranarray(pos[:, sel])
        hsml, m, rho, w = hsml[sel], m[sel], rho[sel], w[sel]
        q = np.ascontiguousarray(q[..., sel])
        posv, n_call = pos_sel, sel.shape[0]
        center_mode, filt = _lib.CENTER_NONE, 0
    else:
        posv, n_call = pos, n
    P = int(param.Npixels[0])
    opts = _options(param, kernel, dims, reduce_image, return_both_maps, calc_mean, precision,
                    deterministic, center_mode, filt, _lib.MEM_HOST)
    out_len = _lib.lib().sphg_output_len(C.byref(param._c), C.byref(opts), nq)
    flat = np.zeros(out_len, dtype=np.float64)
    pt = _lib.SphgParticles()
    pt.n = n_call
    pt.pos_dtype = _np_dt[posv.dtype]
    pt.attr_dtype = _np_dt[np.dtype(adt)]
    pt.pos = posv.ctypes.data
    pt.pos_stride_p = posv.strides[1] // posv.itemsize
    pt.pos_stride_c = posv.strides[0] // posv.itemsize
    pt.hsml, pt.mass, pt.rho, pt.weights = (a.ctypes.data for a in (hsml, m, rho, w))
    pt.bin_q = q.ctypes.data
    pt.n_q = nq
    if q.ndim == 1:
        pt.q_stride_p, pt.q_stride_k = q.strides[0] // q.itemsize, 0
    else:
        pt.q_stride_p, pt.q_stride_k = q.strides[1] // q.itemsize, q.strides[0] // q.itemsize
    st = _lib.SphgStats()
    ctx = context if context is not None else _lib.default_context(device)
    if projection is None:
        _lib.check(_lib.lib().sphg_map(ctx.handle, C.byref(param._c), C.byref(opts), C.byref(pt),
                                       flat.ctypes.data, None, C.byref(st)), ctx.handle)
    else:
        _lib.check(_lib.lib().sphg_map_projected(ctx.handle, C.byref(param._c), C.byref(opts),
                                                 C.byref(pt), C.byref(projection), flat.ctypes.data,
                                                 None, C.byref(st)), ctx.handle)
    if writeback is not None:
        writeback[...] = pos
    return _shape_out(flat, P, nq, dims, return_both_maps and dims == 2), _stats_dict(st)

def _centred_params(param: MappingParameters) -> MappingParameters:
    from .parameters import mappingParameters
    c = param.center
    return mappingParameters(center=(0.0, 0.0, 0.0),
                             x_lim=(param.x_lim[0] - c[0], param.x_lim[1] - c[0]),
                             y_lim=(param.y_lim[0] - c[1], param.y_lim[1] - c[1]),
                             z_lim=(param.z_lim[0] - c[2], param.z_lim[1] - c[2]),
                             Npixels=max(param.Npixels), boxsize=param.boxsize)

def _torch_dt(t):
    import torch
    if t.dtype == torch.float32:
        return _lib.SPHG_F32
    if t.dtype == torch.float64:
        return _lib.SPHG_F64
    raise TypeError(f"unsupported dtype {t.dtype}")

def _map_torch(Pos, HSML, M, Rho, Bin_Quant, Weights, param, kernel, reduce_image, return_both_maps,
               dims, calc_mean, sort_z, precision, deterministic, center_in_place=True, context=None,
               projection=None):
    import torch
    if Pos.dim() != 2 or Pos.shape[0] != 3:
        raise ValueError("Pos must be a (3, N) tensor")
    if sort_z:
        raise NotImplementedError("sort_z with device tensors: pass host arrays")
    dev = Pos.device
    n = Pos.shape[1]
    attrs = [HSML, M, Rho, Weights, Bin_Quant]
    for a in attrs:
        if not _is_torch_cuda(a) or a.device != dev:
            raise ValueError("all particle arrays must be CUDA tensors on the device of Pos")
    adt = torch.float32 if all(a.dtype == torch.float32 for a in attrs) else torch.float64
    hsml, m, rho, w = [a.to(adt).contiguous().reshape(-1) for a in attrs[:4]]
    q = Bin_Quant.to(adt)
    nq = 1 if q.dim() == 1 else q.shape[0]
    if any(s < 0 for s in Pos.stride()):
        raise ValueError("Pos strides must be non-negative")
    P = int(param.Npixels[0])
    opts = _options(param, kernel, dims, reduce_image, return_both_maps, calc_mean, precision,
                    deterministic, _lib.CENTER_INPLACE if center_in_place else _lib.CENTER_READONLY,
                    1, _lib.MEM_DEVICE)
    out_len = _lib.lib().sphg_output_len(C.byref(param._c), C.byref(opts), nq)
    flat = torch.empty(out_len, dtype=torch.float64, device=dev)
    pt = _lib.SphgParticles()
    pt.n = n
    pt.pos_dtype = _torch_dt(Pos)
    pt.attr_dtype = _torch_dt(hsml)
    pt.pos = Pos.data_ptr()
    pt.pos_stride_p, pt.pos_stride_c = Pos.stride(1), Pos.stride(0)
    pt.hsml, pt.mass, pt.rho, pt.weights = (a.data_ptr() for a in (hsml, m, rho, w))
    pt.bin_q = q.data_ptr()
    pt.n_q = nq
    if q.dim() == 1:
        pt.q_stride_p, pt.q_stride_k = q.stride(0), 0
    else:
        pt.q_stride_p, pt.q_stride_k = q.stride(1), q.stride(0)
    st = _lib.SphgStats()
    ctx = context if context is not None else _lib.default_context(dev.index if dev.index is not None else 0)
    stream = _lib.stream_handle(torch.cuda.current_stream(dev))
    if projection is None:
        _lib.check(_lib.lib().sphg_map(ctx.handle, C.byref(param._c), C.byref(opts), C.byref(pt),
                                       C.c_void_p(flat.data_ptr()), stream, C.byref(st)),
                   ctx.handle)
    else:
        _lib.check(_lib.lib().sphg_map_projected(ctx.handle, C.byref(param._c), C.byref(opts),
                                                 C.byref(pt), C.byref(projection),
                                                 C.c_void_p(flat.data_ptr()), stream, C.byref(st)),
                   ctx.handle)
    return _shape_out(flat, P, nq, dims, return_both_maps and dims == 2), _stats_dict(st)


def sph_footprints(Pos, HSML, Bin_Quant, *, param: MappingParameters, dimensions=2, calc_mean=False,
                   context=None):
    """Per-particle state and integer pixel ranges as the mapping computes
    them on the device (sphg_footprints): centring and filter
    (filter_shift.jl:6-58), the quantity skip (cic_2D.jl:154-168) and
    pix_index_min_max (cic_shared.jl:46-52).  CUDA tensors in, on one device;
    the positions are not written.  Returns ``(ranges, state)``: int64
    (N, 6) ``[iMin, iMax, jMin, jMax, kMin, kMax]`` and int8 (N,) with 0
    filtered, 1 skipped, 2 mapped."""
    import torch
    dims = dimensions
    if dims not in (2, 3):
        raise ValueError("dimensions must be 2 or 3")
    if Pos.dim() != 2 or Pos.shape[0] != 3:
        raise ValueError("Pos must be a (3, N) tensor")
    dev = Pos.device
    for a in (HSML, Bin_Quant):
        if not _is_torch_cuda(a) or a.device != dev:
            raise ValueError("all particle arrays must be CUDA tensors on the device of Pos")
    adt = torch.float32 if HSML.dtype == torch.float32 and Bin_Quant.dtype == torch.float32 else torch.float64
    hsml = HSML.to(adt).contiguous().reshape(-1)
    q = Bin_Quant.to(adt)
    nq = 1 if q.dim() == 1 else q.shape[0]
    n = Pos.shape[1]
    opts = _lib.SphgOptions()
    opts.dimensions = dims
    opts.kernel = 0
    opts.kernel_dim = dims
    opts.calc_mean = int(calc_mean)
    opts.center = _lib.CENTER_READONLY
    opts.filter = 1
    opts.memspace = _lib.MEM_DEVICE
    pt = _lib.SphgParticles()
    pt.n = n
    pt.pos_dtype = _torch_dt(Pos)
    pt.attr_dtype = _torch_dt(hsml)
    pt.pos = Pos.data_ptr()
    pt.pos_stride_p, pt.pos_stride_c = Pos.stride(1), Pos.stride(0)
    pt.hsml = hsml.data_ptr()
    pt.bin_q = q.data_ptr()
    pt.n_q = nq
    if q.dim() == 1:
        pt.q_stride_p, pt.q_stride_k = q.stride(0), 0
    else:
        pt.q_stride_p, pt.q_stride_k = q.stride(1), q.stride(0)
    ranges = torch.empty((n, 6), dtype=torch.int64, device=dev)
    state = torch.empty(n, dtype=torch.int8, device=dev)
    ctx = context if context is not None else _lib.default_context(dev.index if dev.index is not None else 0)
    stream = _lib.stream_handle(torch.cuda.current_stream(dev))
    _lib.check(_lib.lib().sphg_footprints(ctx.handle, C.byref(param._c), C.byref(opts), C.byref(pt),
                                          C.c_void_p(ranges.data_ptr()), C.c_void_p(state.data_ptr()), stream),
               ctx.handle)
    return ranges, state


def rotation_matrix_xyz(alpha: float, beta: float, gamma: float) -> np.ndarray:
    """RotXYZ(alpha, beta, gamma) = Rx(alpha) Ry(beta) Rz(gamma), angles in
    degrees, as rotate_3D builds it (rotate_particles.jl:7-14); row-major."""
    a, b, c = (math.radians(float(x)) for x in (alpha, beta, gamma))
    sa, ca, sb, cb, sc, cc = math.sin(a), math.cos(a), math.sin(b), math.cos(b), math.sin(c), math.cos(c)
    return np.array([[cb * cc, -(cb * sc), sb],
                     [ca * sc + sa * sb * cc, ca * cc - sa * sb * sc, -(sa * cb)],
                     [sa * sc - ca * sb * cc, sa * cc + ca * sb * sc, ca * cb]], dtype=np.float64)


def _projection(projection):
    pr = _lib.SphgProjection()
    if isinstance(projection, str):
        kinds = {"xy": _lib.PROJ_XY, "xz": _lib.PROJ_XZ, "yz": _lib.PROJ_YZ}
        if projection not in kinds:
            raise ValueError("projection must be either along in 'xy', 'xz', or 'yz' plane of "
                             "defined by a vector of Euler angles!")
        pr.kind = kinds[projection]
        return pr, projection
    angles = [float(x) for x in projection]
    if len(angles) != 3:
        raise ValueError("projection must be either along in 'xy', 'xz', or 'yz' plane of "
                         "defined by a vector of Euler angles!")
    pr.kind = _lib.PROJ_MATRIX
    for k, v in enumerate(rotation_matrix_xyz(*angles).reshape(-1)):
        pr.matrix[k] = v
    name = "alpha=%0.2fbeta=%0.2fgamma=%0.2f" % tuple(angles)
    return pr, name


def map_it(pos_in, hsml, mass, rho, bin_q, weights, RM=None, *, param: MappingParameters,
           kernel: SPHKernel | None = None, snap: int = 0, units: str = "",
           image_prefix: str = "dummy", reduce_image: bool = True, parallel: bool = True,
           calc_mean: bool = True, show_progress: bool = True, sort_z: bool = False,
           stokes: bool = False, renorm: bool = False, projection="xy", precision: str = "fp64",
           deterministic: bool = False, device: int = 0, write_fits: bool = True):
    """map_it (cic_interpolation.jl:314-380): map the particles seen along a
    projection ('xy', 'xz', 'yz' or three Euler angles in degrees) and write
    ``<image_prefix>.<projection>.fits`` with the caller's parameters.

    The projection is applied while the positions are read (K1), so
    ``pos_in`` is left intact as the reference's copy leaves it.  Defaults
    are the reference's (``calc_mean=True``, WendlandC6 in 2D).  Returns the
    map (the reference returns nothing)."""
    from .parameters import WendlandC6
    if RM is not None or stokes:
        raise NotImplementedError(
            "Faraday rotation / Stokes mapping (cic_shared.jl:129-159) is not supported")
    if sort_z:
        raise NotImplementedError("sort_z of projected positions is not supported")
    kernel = kernel if kernel is not None else WendlandC6(2)
    pr, name = _projection(projection)
    if weights is None:
        weights = rho
    t0 = time.perf_counter()
    if _is_torch_cuda(pos_in):
        image, stats = _map_torch(pos_in, hsml, mass, rho, bin_q, weights, param, kernel, reduce_image,
                                  False, 2, calc_mean, False, precision, deterministic, False, None, pr)
    else:
        image, stats = _map_numpy(pos_in, hsml, mass, rho, bin_q, weights, param, kernel, reduce_image,
                                  False, 2, calc_mean, False, precision, deterministic, device, False,
                                  None, pr)
    if renorm:
        image = image / image.max()
    if show_progress:
        log.info("map_it %s: %d / %d particles mapped, %d deposits, %.3f s", name, stats["n_mapped"],
                 stats["n_in"], stats["deposits"], time.perf_counter() - t0)
    if write_fits:
        from .io import write_fits_image
        write_fits_image(f"{image_prefix}.{name}.fits", image, param, snap=snap, units=units)
    return image
