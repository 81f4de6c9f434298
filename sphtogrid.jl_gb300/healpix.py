"""``healpix_map`` (SPHtoGrid.jl src/healpix_interpolation/main.jl:92-227):
an all-sky map of the particles as seen from ``center``, on a HEALPix RING
grid of ``Nside``, deposited on the GPU in FP64 (``sphg_healpix_map``).

The particle selection is the reference's filter_sort_particles
(filter_particles.jl:19-53) as written, done here on the host (numpy
inputs) or on the device (CUDA tensors): the caller's ``Pos`` is centred in
place, and the input-order shell mask picks entries of the
descending-distance permutation (``sorted[sel]``).  Returns
``(allsky_map, weight_map)``, 12 Nside^2 FP64 values each in RING order;
divide the first by the second to reduce, as the reference documents.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from . import _lib
from .parameters import SPHKernel


def _select_numpy(Pos, arrays, center, radius_limits, calc_mean):
    Pos -= np.asarray(center, dtype=Pos.dtype)[:, None]
    dx = np.sqrt(Pos[0] ** 2 + Pos[1] ** 2 + Pos[2] ** 2)
    sel = (radius_limits[0] <= dx) & (dx <= radius_limits[1])
    if not calc_mean:
        q = arrays[3]
        qs = q[sel] > 0.0
        if qs.shape[0] != sel.shape[0]:  # the reference's sel[Bin_q[sel] .> 0] needs equal lengths
            raise IndexError("filter_sort_particles: boolean index of length "
                             f"{qs.shape[0]} into {sel.shape[0]} particles")
        sel = sel[qs]
    order = np.argsort(dx, kind="stable")[::-1]
    idx = order[sel]
    return np.ascontiguousarray(Pos[:, idx].T), [np.ascontiguousarray(a[idx]) for a in arrays]


def _select_torch(Pos, arrays, center, radius_limits, calc_mean):
    import torch
    Pos -= torch.as_tensor(center, dtype=Pos.dtype, device=Pos.device)[:, None]
    dx = torch.sqrt(Pos[0] ** 2 + Pos[1] ** 2 + Pos[2] ** 2)
    sel = (radius_limits[0] <= dx) & (dx <= radius_limits[1])
    if not calc_mean:
        qs = arrays[3][sel] > 0.0
        if qs.shape[0] != sel.shape[0]:
            raise IndexError("filter_sort_particles: boolean index of length "
                             f"{qs.shape[0]} into {sel.shape[0]} particles")
        sel = sel[qs]
    order = torch.flip(torch.sort(dx, stable=True).indices, dims=(0,))
    idx = order[sel]
    return Pos[:, idx].T.contiguous(), [a[idx].contiguous() for a in arrays]


def healpix_map(Pos, Hsml, M, Rho, Bin_q, Weights, *, center=(0.0, 0.0, 0.0),
                radius_limits=(0.0, math.inf), Nside: int = 1024, kernel: SPHKernel,
                show_progress: bool = True, output_from_all_workers: bool = False,
                calc_mean: bool = True, device: int = 0, return_stats: bool = False):
    """The reference's healpix_map on the GPU; see the module docstring.
    numpy inputs give numpy maps, CUDA tensors give CUDA tensors."""
    import torch
    on_device = isinstance(Pos, torch.Tensor) and Pos.is_cuda
    npix = 12 * int(Nside) * int(Nside)
    if on_device:
        dev = Pos.device
        arrays = [torch.as_tensor(a, device=dev) for a in (Hsml, M, Rho, Bin_q, Weights)]
        dt = torch.float64 if any(a.dtype == torch.float64 for a in [Pos] + arrays) else torch.float32
        allsky = torch.zeros(npix, dtype=torch.float64, device=dev)
        weight = torch.zeros(npix, dtype=torch.float64, device=dev)
        if not calc_mean and float(arrays[3].sum()) == 0.0:
            return (allsky, weight, {}) if return_stats else (allsky, weight)
        pos, arrs = _select_torch(Pos, arrays, center, radius_limits, calc_mean)
        pos, arrs = pos.to(dt).contiguous(), [a.to(dt).contiguous() for a in arrs]
        keep = (pos, arrs)
        ptrs = [pos.data_ptr()] + [a.data_ptr() for a in arrs]
        dtype = _lib.SPHG_F64 if dt == torch.float64 else _lib.SPHG_F32
        stream = _lib.stream_handle(torch.cuda.current_stream(dev))
        ctx = _lib.default_context(dev.index if dev.index is not None else 0)
        out_a, out_w = allsky, weight
    else:
        arrays = [np.asarray(a) for a in (Hsml, M, Rho, Bin_q, Weights)]
        allsky = np.zeros(npix)
        weight = np.zeros(npix)
        if not calc_mean and float(np.sum(arrays[3])) == 0.0:
            return (allsky, weight, {}) if return_stats else (allsky, weight)
        pos, arrs = _select_numpy(Pos, arrays, center, radius_limits, calc_mean)
        dev = torch.device("cuda", device)
        dt = torch.float64 if any(a.dtype == np.float64 for a in [pos] + arrs) else torch.float32
        keep = [torch.as_tensor(np.ascontiguousarray(pos), device=dev).to(dt)] + \
               [torch.as_tensor(a, device=dev).to(dt) for a in arrs]
        ptrs = [t.data_ptr() for t in keep]
        dtype = _lib.SPHG_F64 if dt == torch.float64 else _lib.SPHG_F32
        stream = _lib.stream_handle(torch.cuda.current_stream(dev))
        ctx = _lib.default_context(device)
        out_a = torch.zeros(npix, dtype=torch.float64, device=dev)
        out_w = torch.zeros(npix, dtype=torch.float64, device=dev)
    hp = _lib.SphgHealpixParams()
    hp.nside = int(Nside)
    hp.kernel, hp.kernel_dim = kernel.kind, kernel.dim
    hp.calc_mean = int(bool(calc_mean))
    hp.dtype = dtype
    st = _lib.SphgStats()
    n = len(arrs[0])
    _lib.check(_lib.lib().sphg_healpix_map(ctx.handle, C.byref(hp), n, *[C.c_void_p(p) for p in ptrs],
                                           C.c_void_p(out_a.data_ptr()), C.c_void_p(out_w.data_ptr()),
                                           stream, C.byref(st)), ctx.handle)
    del keep
    if not on_device:
        allsky, weight = out_a.cpu().numpy(), out_w.cpu().numpy()
    stats = {"n_in": len(Hsml), "selected": n, "n_mapped": st.n_mapped, "deposits": st.deposits,
             "grid_mass": st.grid_mass, "particle_mass": st.particle_mass}
    return (allsky, weight, stats) if return_stats else (allsky, weight)
