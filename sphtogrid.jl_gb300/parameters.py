"""``mappingParameters`` and the SPHKernels kernel types, mirroring the Julia
interface of SPHtoGrid.jl (src/shared/parameters.jl:14-125) and SPHKernels.jl
(kernel constructors ``Cubic(dim)``, ``Quintic(dim)``, ``WendlandC4(dim)``,
``WendlandC6(dim)``, ``WendlandC8(dim)``; default dim 3)."""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

from . import _lib


class MappingParameters:
    """Parameter object of one map.  Fields as in ``mappingParameters``:
    ``x_lim, y_lim, z_lim, center, halfsize, len2pix, pixelSideLength,
    Npixels, boxsize, periodic``."""

    __slots__ = ("_c",)

    def __init__(self, c: _lib.SphgParams):
        self._c = c

    x_lim = property(lambda s: list(s._c.x_lim))
    y_lim = property(lambda s: list(s._c.y_lim))
    z_lim = property(lambda s: list(s._c.z_lim))
    center = property(lambda s: list(s._c.center))
    halfsize = property(lambda s: list(s._c.halfsize))
    len2pix = property(lambda s: s._c.len2pix)
    pixelSideLength = property(lambda s: s._c.pixelSideLength)
    Npixels = property(lambda s: list(s._c.Npixels))
    boxsize = property(lambda s: s._c.boxsize)
    periodic = property(lambda s: bool(s._c.periodic))

    def __repr__(self):
        return (f"mappingParameters(x_lim={self.x_lim}, y_lim={self.y_lim}, z_lim={self.z_lim}, "
                f"center={self.center}, Npixels={self.Npixels[0]}, "
                f"pixelSideLength={self.pixelSideLength}, boxsize={self.boxsize})")


def mappingParameters(T=None, *, x_lim=(-1.0, -1.0), y_lim=(-1.0, -1.0), z_lim=(-1.0, -1.0),
                      center=(-1.0, -1.0, -1.0), x_size=-1.0, y_size=-1.0, z_size=-1.0,
                      pixelSideLength=-1.0, Npixels=0, boxsize=-1.0) -> MappingParameters:
    """Define either ``*_lim``, or ``center`` and ``*_size``; resolution by
    ``pixelSideLength`` or ``Npixels``.  Raises ``SPHtoGridError`` with the
    reference's messages (parameters.jl:67,98).  ``T`` is accepted for
    signature compatibility; parameters are always Float64."""
    arr = lambda v: (C.c_double * len(v))(*[float(x) for x in v])
    out = _lib.SphgParams()
    st = _lib.lib().sphg_mapping_parameters(arr(x_lim), arr(y_lim), arr(z_lim), arr(center),
                                            float(x_size), float(y_size), float(z_size),
                                            float(pixelSideLength), int(Npixels), float(boxsize),
                                            C.byref(out))
    _lib.check(st)
    return MappingParameters(out)


@dataclass(frozen=True)
class SPHKernel:
    """An SPHKernels.jl kernel: ``kind`` is the ABI kernel id, ``dim`` the
    dimension its normalisation is defined for."""

    kind: int
    dim: int = 3
    name: str = ""


def Cubic(dim: int = 3) -> SPHKernel:
    return SPHKernel(0, _dim(dim), "Cubic")


def Quintic(dim: int = 3) -> SPHKernel:
    return SPHKernel(1, _dim(dim), "Quintic")


def WendlandC4(dim: int = 3) -> SPHKernel:
    return SPHKernel(2, _dim(dim), "WendlandC4")


def WendlandC6(dim: int = 3) -> SPHKernel:
    return SPHKernel(3, _dim(dim), "WendlandC6")


def WendlandC8(dim: int = 3) -> SPHKernel:
    return SPHKernel(4, _dim(dim), "WendlandC8")


_BY_NAME = {"cubic": Cubic, "quintic": Quintic, "wendlandc4": WendlandC4,
            "wendlandc6": WendlandC6, "wendlandc8": WendlandC8}


def kernel_from_name(name: str, dim: int = 3) -> SPHKernel:
    return _BY_NAME[name.lower()](dim)


def _dim(d: int) -> int:
    if d not in (2, 3):
        raise ValueError("kernel dimension must be 2 or 3")
    return int(d)
