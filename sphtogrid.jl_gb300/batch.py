"""Batched maps: many ``sphMapping`` calls (uneven particle counts,
resolutions, quantity counts and kernel shapes) planned once, autotuned,
captured in a CUDA graph and replayed (``sphg_batch_*`` in include/sphgrid.h).

Inputs are CUDA tensors that stay where they are; to map new data, write it
into the same tensors and launch again.
"""
from __future__ import annotations

import ctypes as C

import torch

from . import _lib
from .parameters import MappingParameters, SPHKernel


def _dt(t):
    if t.dtype == torch.float32:
        return _lib.SPHG_F32
    if t.dtype == torch.float64:
        return _lib.SPHG_F64
    raise TypeError(f"unsupported dtype {t.dtype}")


class SphgMapDesc(C.Structure):
    _fields_ = [("par", _lib.SphgParams), ("opt", _lib.SphgOptions),
                ("parts", _lib.SphgParticles), ("out", C.c_void_p)]


class SphgBatchTuning(C.Structure):
    _fields_ = [("tile_x", C.c_int32), ("tile_y", C.c_int32), ("ctas_per_sm", C.c_int32),
                ("large_cells", C.c_int32), ("tuned_ms", C.c_float), ("reserved", C.c_int32 * 3)]


def _bind(L):
    if getattr(L, "_batch_bound", False):
        return
    vp = C.c_void_p
    L.sphg_batch_create.argtypes = [vp, C.c_int32, C.POINTER(SphgMapDesc),
                                    C.POINTER(SphgBatchTuning), C.POINTER(vp)]
    L.sphg_batch_create.restype = C.c_int
    L.sphg_batch_launch.argtypes = [vp, vp]
    L.sphg_batch_launch.restype = C.c_int
    L.sphg_batch_wait.argtypes = [vp, C.POINTER(_lib.SphgStats)]
    L.sphg_batch_wait.restype = C.c_int
    L.sphg_batch_get_tuning.argtypes = [vp, C.POINTER(SphgBatchTuning)]
    L.sphg_batch_get_tuning.restype = C.c_int
    L.sphg_batch_last_error.argtypes = [vp]
    L.sphg_batch_last_error.restype = C.c_char_p
    L.sphg_batch_destroy.argtypes = [vp]
    L.sphg_batch_destroy.restype = C.c_int
    L._batch_bound = True


class MapSpec:
    """One map of a batch: the arguments of ``sphMapping`` as CUDA tensors."""

    def __init__(self, Pos, HSML, M, Rho, Bin_Quant, Weights=None, *, param: MappingParameters,
                 kernel: SPHKernel, dimensions: int = 2, reduce_image: bool = True,
                 return_both_maps: bool = False, calc_mean: bool = False):
        self.tensors = [Pos, HSML, M, Rho, Bin_Quant, Rho if Weights is None else Weights]
        self.param, self.kernel, self.dims = param, kernel, dimensions
        self.reduce_image, self.return_both_maps, self.calc_mean = (
            reduce_image, return_both_maps, calc_mean)


class SPHBatch:
    """Plans and owns one batch (see module docstring)."""

    def __init__(self, specs, *, deterministic=False, tuning=None, device=None):
        L = _lib.lib()
        _bind(L)
        self.specs = list(specs)
        dev = self.specs[0].tensors[0].device
        if device is None:
            device = dev.index if dev.index is not None else 0
        self.ctx = _lib.default_context(device)
        n = len(self.specs)
        self._descs = (SphgMapDesc * n)()
        self.outputs = []
        for i, sp in enumerate(self.specs):
            pos, hsml, m, rho, q, w = sp.tensors
            adt = hsml.dtype
            for t in (m, rho, q, w):
                if t.dtype != adt:
                    raise TypeError("hsml, mass, rho, Bin_Quant and weights must share a dtype")
            for t in sp.tensors:
                if not t.is_cuda:
                    raise ValueError("batched maps take CUDA tensors")
            d = self._descs[i]
            d.par = _lib.SphgParams.from_buffer_copy(sp.param._c)
            o = d.opt
            o.dimensions = sp.dims
            o.kernel, o.kernel_dim = sp.kernel.kind, sp.kernel.dim
            o.reduce_image = int(sp.reduce_image)
            o.return_both_maps = int(sp.return_both_maps)
            o.calc_mean = int(sp.calc_mean)
            o.precision = _lib.PREC["fp32c"]
            o.deterministic = int(bool(deterministic))
            o.center = _lib.CENTER_READONLY
            o.filter = 1
            o.memspace = _lib.MEM_DEVICE
            pt = d.parts
            pt.n = pos.shape[1]
            pt.pos_dtype, pt.attr_dtype = _dt(pos), _dt(hsml)
            pt.pos = pos.data_ptr()
            pt.pos_stride_p, pt.pos_stride_c = pos.stride(1), pos.stride(0)
            pt.hsml, pt.mass, pt.rho, pt.weights = (t.data_ptr() for t in (hsml, m, rho, w))
            pt.bin_q = q.data_ptr()
            pt.n_q = 1 if q.dim() == 1 else q.shape[0]
            pt.q_stride_p, pt.q_stride_k = (q.stride(0), 0) if q.dim() == 1 else (q.stride(1),
                                                                                  q.stride(0))
            nout = L.sphg_output_len(C.byref(d.par), C.byref(o), pt.n_q)
            out = torch.empty(int(nout), dtype=torch.float64, device=pos.device)
            d.out = out.data_ptr()
            self.outputs.append(out)
        tun = None
        if tuning is not None:
            tun = SphgBatchTuning()
            tun.tile_x, tun.tile_y, tun.ctas_per_sm, tun.large_cells = tuning
        h = C.c_void_p()
        torch.cuda.synchronize(dev)  # the inputs must be ready: planning maps once
        st = L.sphg_batch_create(self.ctx.handle, n, self._descs,
                                 C.byref(tun) if tun is not None else None, C.byref(h))
        _lib.check(st, self.ctx.handle)
        self.handle = h

    def launch(self, stream=None):
        L = _lib.lib()
        s = stream if stream is not None else torch.cuda.current_stream(self.outputs[0].device)
        st = L.sphg_batch_launch(self.handle, _lib.stream_handle(s))
        if st:
            raise _lib.SPHtoGridError(st, L.sphg_batch_last_error(self.handle).decode())

    def wait(self):
        L = _lib.lib()
        stats = (_lib.SphgStats * len(self.specs))()
        st = L.sphg_batch_wait(self.handle, stats)
        if st:
            raise _lib.SPHtoGridError(st, L.sphg_batch_last_error(self.handle).decode())
        return [{"n_mapped": s.n_mapped, "deposits": s.deposits, "n_launches": s.n_launches,
                 "n_reruns": s.n_reruns} for s in stats]

    @property
    def tuning(self):
        t = SphgBatchTuning()
        _lib.lib().sphg_batch_get_tuning(self.handle, C.byref(t))
        return {"tile_x": t.tile_x, "tile_y": t.tile_y, "ctas_per_sm": t.ctas_per_sm,
                "large_cells": t.large_cells, "tuned_ms": t.tuned_ms}

    def image(self, i):
        """Output i shaped as sphMapping returns it (Fortran-ordered view)."""
        sp = self.specs[i]
        P = int(sp.param.Npixels[0])
        q = sp.tensors[4]
        nq = 1 if q.dim() == 1 else q.shape[0]
        if sp.dims == 2 and sp.return_both_maps:
            shape = (P * P, nq + 1)
        elif sp.dims == 2:
            shape = (P, P, nq)
        else:
            shape = (P, P, P)
        strides, s = [], 1
        for d in shape:
            strides.append(s)
            s *= d
        return self.outputs[i].as_strided(shape, tuple(strides))

    def close(self):
        if getattr(self, "handle", None):
            _lib.lib().sphg_batch_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
