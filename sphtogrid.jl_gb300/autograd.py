"""Differentiable ``sphMapping`` for torch: a ``torch.autograd.Function`` whose
backward is the library's hand-written adjoint (``sphg_adjoint``).  The
reference has no derivatives; this is the Python counterpart of the
ChainRulesCore ``rrule`` in julia/SPHtoGridGB300.jl.

The forward deposits once into the raw (P^D, Nq+1) accumulator, reduces it
with ``sphg_reduce`` and keeps the accumulator for the backward pass, which
recomputes the kernel weights (no particle-pixel list is stored).  Positions
are read, never centred in place, so the same tensors serve both passes.
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


def _particles(pos, hsml, m, rho, q, w):
    pt = _lib.SphgParticles()
    pt.n = pos.shape[1]
    pt.pos_dtype = _dt(pos)
    pt.attr_dtype = _dt(hsml)
    pt.pos = pos.data_ptr()
    pt.pos_stride_p, pt.pos_stride_c = pos.stride(1), pos.stride(0)
    pt.hsml, pt.mass, pt.rho, pt.weights = (a.data_ptr() for a in (hsml, m, rho, w))
    pt.bin_q = q.data_ptr()
    pt.n_q = 1 if q.dim() == 1 else q.shape[0]
    if q.dim() == 1:
        pt.q_stride_p, pt.q_stride_k = q.stride(0), 0
    else:
        pt.q_stride_p, pt.q_stride_k = q.stride(1), q.stride(0)
    return pt


def _options(kernel, dims, reduce_image, calc_mean, precision, raw):
    o = _lib.SphgOptions()
    o.dimensions = dims
    o.kernel = kernel.kind
    o.kernel_dim = kernel.dim
    o.reduce_image = int(bool(reduce_image))
    o.calc_mean = int(bool(calc_mean))
    o.precision = _lib.PREC[precision]
    o.center = _lib.CENTER_READONLY
    o.filter = 1
    o.memspace = _lib.MEM_DEVICE
    o.raw_accumulator = int(raw)
    return o


def _out_shape(P, nq, dims):
    return (P, P, nq) if dims == 2 else (P, P, P)


def _fortran_view(flat, shape):
    strides, s = [], 1
    for d in shape:
        strides.append(s)
        s *= d
    return flat.as_strided(shape, tuple(strides))


class SPHMapFunction(torch.autograd.Function):
    """out = sphMapping(pos, hsml, m, rho, q, w) with dL/d(all six) in backward."""

    @staticmethod
    def forward(ctx, pos, hsml, m, rho, q, w, spec):
        param, kernel, dims, reduce_image, calc_mean, precision, _ = spec
        dev = pos.device
        L = _lib.lib()
        hnd = _lib.default_context(dev.index or 0).handle
        stream = _lib.stream_handle(torch.cuda.current_stream(dev))
        pt = _particles(pos, hsml, m, rho, q, w)
        nq = pt.n_q
        P = int(param.Npixels[0])
        PD = P ** dims
        raw = torch.empty(PD * (nq + 1), dtype=torch.float64, device=dev)
        o = _options(kernel, dims, reduce_image, calc_mean, precision, True)
        st = _lib.SphgStats()
        _lib.check(L.sphg_map(hnd, C.byref(param._c), C.byref(o), C.byref(pt),
                              C.c_void_p(raw.data_ptr()), stream, C.byref(st)), hnd)
        out = torch.empty(P * P * nq if dims == 2 else PD, dtype=torch.float64, device=dev)
        o.raw_accumulator = 0
        _lib.check(L.sphg_reduce(hnd, C.byref(param._c), C.byref(o), nq,
                                 C.c_void_p(raw.data_ptr()), C.c_void_p(out.data_ptr()), stream), hnd)
        ctx.save_for_backward(pos, hsml, m, rho, q, w, raw)
        ctx.spec = spec
        return _fortran_view(out, _out_shape(P, nq, dims))

    @staticmethod
    def backward(ctx, gout):
        pos, hsml, m, rho, q, w, raw = ctx.saved_tensors
        param, kernel, dims, reduce_image, calc_mean, _, precision = ctx.spec
        dev = pos.device
        L = _lib.lib()
        hnd = _lib.default_context(dev.index or 0).handle
        stream = _lib.stream_handle(torch.cuda.current_stream(dev))
        P = int(param.Npixels[0])
        nq = 1 if q.dim() == 1 else q.shape[0]
        # dL/d(out) flattened in the output's column-major order
        g = gout.to(torch.float64).permute(*reversed(range(gout.dim()))).contiguous().reshape(-1)
        f64 = dict(dtype=torch.float64, device=dev)
        # gradients use the strides of the (dense) inputs
        dense = lambda t: t if t.is_contiguous() or (t.dim() == 2 and t.t().is_contiguous()) \
            else t.contiguous()
        pos_in, q_in = dense(pos), dense(q)
        d_pos = torch.zeros(pos_in.shape, **f64).as_strided(pos_in.shape, pos_in.stride())
        d_q = torch.zeros(q_in.shape, **f64).as_strided(q_in.shape, q_in.stride())
        d_h, d_m, d_r, d_w = (torch.zeros(hsml.shape[0], **f64) for _ in range(4))
        pt = _particles(pos_in, hsml.contiguous(), m.contiguous(), rho.contiguous(), q_in,
                        w.contiguous())
        gr = _lib.SphgGrads()
        gr.pos, gr.hsml, gr.mass, gr.rho, gr.weights, gr.bin_q = (
            t.data_ptr() for t in (d_pos, d_h, d_m, d_r, d_w, d_q))
        o = _options(kernel, dims, reduce_image, calc_mean, precision, False)
        _lib.check(L.sphg_adjoint(hnd, C.byref(param._c), C.byref(o), C.byref(pt),
                                  C.c_void_p(raw.data_ptr()), C.c_void_p(g.data_ptr()),
                                  C.byref(gr), stream), hnd)
        cast = lambda grad, like: grad.to(like.dtype)
        return (cast(d_pos, pos), cast(d_h, hsml), cast(d_m, m), cast(d_r, rho), cast(d_q, q),
                cast(d_w, w), None)


def sph_map_differentiable(Pos, HSML, M, Rho, Bin_Quant, Weights=None, *, param: MappingParameters,
                           kernel: SPHKernel, dimensions: int = 2, reduce_image: bool = True,
                           calc_mean: bool = False, precision: str = "fp64",
                           adjoint_precision: str | None = None):
    """``sphMapping`` on CUDA tensors with gradients for every particle input.
    Returns the reduced map ((P, P, Nq) 2D, (P, P, P) 3D) as a float64 tensor.
    ``precision`` is the forward's; ``adjoint_precision`` (default: the same)
    the backward's: "fp64", or "fp32c" (per-cell terms in FP32 with
    compensated sums; particles whose sums cancel beyond its rounding bound
    are redone in FP64)."""
    if adjoint_precision is None:
        adjoint_precision = precision
    for name, value in (("precision", precision), ("adjoint_precision", adjoint_precision)):
        if value not in _lib.PREC:
            raise ValueError(f"{name} must be one of {sorted(_lib.PREC)}, not {value!r}")
    if Weights is None:
        Weights = Rho
    spec = (param, kernel, dimensions, reduce_image, calc_mean, precision, adjoint_precision)
    return SPHMapFunction.apply(Pos, HSML, M, Rho, Bin_Quant, Weights, spec)
