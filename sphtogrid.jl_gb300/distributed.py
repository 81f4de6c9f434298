"""``distributed_cic_map`` (SPHtoGrid.jl src/distributed_mapping/cic.jl:24-110)
without the file output: maps a snapshot stored in sub-files and sums the
per-sub-file raw maps.

The reference farms sub-files out to Julia worker processes through a job
channel and sums the returned maps on the master, skipping NaN and Inf
entries (cic.jl:55-78), then reduces (reduce_image_2D/3D).  Here every rank of
a ``torch.distributed`` group (one per GPU) maps sub-files rank, rank + W,
... with its own GPU, sums them with ``sphg_accumulate`` (finite entries
only), and the per-rank sums meet in one all-reduce -- the only exchange
step, over the raw (P^D, Nimages+1) FP64 accumulator.  Every rank returns the
reduced image.
"""
from __future__ import annotations

import ctypes as C

from . import _lib
from .parameters import MappingParameters


def _as_raw(result, n_images):
    """The mapping function's result -- ``(maps, weight_map)`` as in the
    reference's example (docs/src/mapping.md:190-198) or the raw
    ``return_both_maps`` array -- as a (P^D, Nimages+1) tensor."""
    import torch
    if result is None:
        return None
    if isinstance(result, tuple):
        maps, wmap = result
        if maps is None:
            return None
        maps = torch.as_tensor(maps)
        wmap = torch.as_tensor(wmap)
        if maps.dim() == 1:
            maps = maps[:, None]
        return torch.cat([maps.to(torch.float64), wmap.to(torch.float64).reshape(-1, 1)], dim=1)
    raw = torch.as_tensor(result).to(torch.float64)
    if raw.shape[-1] != n_images + 1:
        raise ValueError("the mapping function must return Nimages quantity maps and a weight map")
    return raw


def _gpu_accumulate(ctx):
    import torch

    def acc(total, part):
        _lib.check(_lib.lib().sphg_accumulate(
            ctx.handle, part.numel(), C.c_void_p(part.data_ptr()), C.c_void_p(total.data_ptr()),
            _lib.stream_handle(torch.cuda.current_stream(total.device))), ctx.handle)
    return acc


def _gpu_reduce(ctx, param, n_images, ndim, reduce_image):
    import torch

    def red(total):
        o = _lib.SphgOptions()
        o.dimensions = ndim
        # reduce_image_3D always divides where Q > 0 (cic.jl:88)
        o.reduce_image = int(reduce_image or ndim == 3)
        P = int(param.Npixels[0])
        out = torch.empty(P ** ndim * (n_images if ndim == 2 else 1), dtype=torch.float64,
                          device=total.device)
        _lib.check(_lib.lib().sphg_reduce(ctx.handle, C.byref(param._c), C.byref(o), n_images,
                                          C.c_void_p(total.data_ptr()),
                                          C.c_void_p(out.data_ptr()),
                                          _lib.stream_handle(torch.cuda.current_stream(total.device))),
                   ctx.handle)
        shape = (P, P, n_images) if ndim == 2 else (P, P, P)
        strides, s = [], 1
        for d in shape:
            strides.append(s)
            s *= d
        return out.as_strided(shape, tuple(strides))
    return red


def distributed_cic_map(Nsubfiles: int, mapping_function, param: MappingParameters,
                        Nimages: int = 1, *, reduce_image: bool = True, Ndim: int = 2, group=None,
                        device=None, accumulate=None, reduce=None):
    """Sum the raw maps ``mapping_function(subfile)`` of sub-files
    0..Nsubfiles-1 over the ranks of ``group`` and reduce the sum.

    ``mapping_function`` returns ``(maps, weight_map)`` or the raw
    ``return_both_maps`` array (CUDA tensors for the GPU path).
    ``accumulate(total, part)`` (add the finite entries of ``part`` into
    ``total``, both (P^D, Nimages+1) column-major) and ``reduce(total)``
    default to the library's kernels (``sphg_accumulate`` / ``sphg_reduce``)
    on CUDA device ``device``; when both are given, the sum is kept in host
    memory.  A sub-file whose result is ``None`` adds nothing (cic.jl:61)."""
    import torch
    import torch.distributed as dist
    if Ndim not in (2, 3):
        raise ValueError("Only 2D and 3D are possible")
    initialized = dist.is_available() and dist.is_initialized()
    rank = dist.get_rank(group) if initialized else 0
    world = dist.get_world_size(group) if initialized else 1
    P = int(param.Npixels[0])
    PD = P ** Ndim
    if accumulate is None or reduce is None:
        dev = torch.device("cuda", device if device is not None else torch.cuda.current_device())
        ctx = _lib.default_context(dev.index)
        accumulate = accumulate or _gpu_accumulate(ctx)
        reduce = reduce or _gpu_reduce(ctx, param, Nimages, Ndim, reduce_image)
    else:
        dev = torch.device("cpu")
    # the reference's [sum_map sum_weights]: (P^D, Nimages+1), column-major,
    # i.e. the contiguous buffer `cols` holds one column after another
    cols = torch.zeros(Nimages + 1, PD, dtype=torch.float64, device=dev)
    total = cols.t()
    for sub in range(rank, Nsubfiles, world):
        part = _as_raw(mapping_function(sub), Nimages)
        if part is None:
            continue
        if tuple(part.shape) != (PD, Nimages + 1):
            raise ValueError(f"sub-file {sub}: map of shape {tuple(part.shape)}, "
                             f"expected {(PD, Nimages + 1)}")
        part = part.to(dev).t().contiguous().t()
        accumulate(total, part)
    if world > 1:
        dist.all_reduce(cols, op=dist.ReduceOp.SUM, group=group)
    return reduce(total)
