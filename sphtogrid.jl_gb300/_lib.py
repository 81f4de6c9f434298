"""ctypes binding of libsphgrid.so (declared in include/sphgrid.h).

The library must exist: there is no CPU fallback.  Loading fails loudly with
the build command when it is missing.
"""
from __future__ import annotations

import atexit
import ctypes as C
import os
import threading

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG_DIR, "libsphgrid.so")

SPHG_OK = 0
SPHG_ERR_CENTER_EXTENT = 1
SPHG_ERR_PIXELS = 2
SPHG_ERR_DIMS = 3
SPHG_ERR_NONFINITE = 4
SPHG_ERR_NQ = 5
SPHG_ERR_ALLOC = 6
SPHG_ERR_ARG = 7
SPHG_ERR_CUDA = 8
SPHG_ERR_TIMEOUT = 9
SPHG_ERR_NO_DEVICE = 10
SPHG_ERR_UNSUPPORTED = 11

SPHG_F32, SPHG_F64 = 0, 1
PREC = {"fp64": 0, "fp32c": 1}
CENTER_NONE, CENTER_INPLACE, CENTER_READONLY = 0, 1, 2
MEM_DEVICE, MEM_HOST = 0, 1
PROJ_XY, PROJ_XZ, PROJ_YZ, PROJ_MATRIX = 0, 1, 2, 3


class SphgParams(C.Structure):
    """``sphg_params``: field-for-field ``mappingParameters`` (parameters.jl:14-27)."""

    _fields_ = [
        ("x_lim", C.c_double * 2),
        ("y_lim", C.c_double * 2),
        ("z_lim", C.c_double * 2),
        ("center", C.c_double * 3),
        ("halfsize", C.c_double * 3),
        ("len2pix", C.c_double),
        ("pixelSideLength", C.c_double),
        ("Npixels", C.c_int64 * 3),
        ("boxsize", C.c_double),
        ("periodic", C.c_int32),
        ("pad_", C.c_int32),
    ]


class SphgParticles(C.Structure):
    _fields_ = [
        ("n", C.c_int64),
        ("pos_dtype", C.c_int32),
        ("attr_dtype", C.c_int32),
        ("pos", C.c_void_p),
        ("pos_stride_p", C.c_int64),
        ("pos_stride_c", C.c_int64),
        ("hsml", C.c_void_p),
        ("mass", C.c_void_p),
        ("rho", C.c_void_p),
        ("weights", C.c_void_p),
        ("bin_q", C.c_void_p),
        ("n_q", C.c_int32),
        ("pad_", C.c_int32),
        ("q_stride_p", C.c_int64),
        ("q_stride_k", C.c_int64),
    ]


class SphgOptions(C.Structure):
    _fields_ = [
        ("dimensions", C.c_int32),
        ("kernel", C.c_int32),
        ("kernel_dim", C.c_int32),
        ("reduce_image", C.c_int32),
        ("return_both_maps", C.c_int32),
        ("calc_mean", C.c_int32),
        ("precision", C.c_int32),
        ("deterministic", C.c_int32),
        ("center", C.c_int32),
        ("filter", C.c_int32),
        ("memspace", C.c_int32),
        ("profile", C.c_int32),
        ("raw_accumulator", C.c_int32),
        ("reserved", C.c_int32 * 3),
    ]


class SphgHealpixParams(C.Structure):
    _fields_ = [("nside", C.c_int64), ("kernel", C.c_int32), ("kernel_dim", C.c_int32),
                ("calc_mean", C.c_int32), ("dtype", C.c_int32)]


class SphgProjection(C.Structure):
    _fields_ = [("kind", C.c_int32), ("reserved", C.c_int32), ("matrix", C.c_double * 9)]


class SphgStats(C.Structure):
    _fields_ = [
        ("n_in", C.c_int64),
        ("n_mapped", C.c_int64),
        ("deposits", C.c_int64),
        ("grid_mass", C.c_double),
        ("particle_mass", C.c_double),
        ("centred", SphgParams),
        ("n_launches", C.c_int32),
        ("n_reruns", C.c_int32),
        ("phase_ms", C.c_float * 4),
    ]


class SphgGrads(C.Structure):
    _fields_ = [
        ("pos", C.c_void_p),
        ("hsml", C.c_void_p),
        ("mass", C.c_void_p),
        ("rho", C.c_void_p),
        ("weights", C.c_void_p),
        ("bin_q", C.c_void_p),
    ]


def stream_handle(stream) -> C.c_void_p:
    """C-ABI stream argument for a torch stream.  torch reports the legacy
    default stream as handle 0, which the ABI reads as "the library's own
    stream"; pass cudaStreamLegacy (handle 1) instead so the work is ordered
    with the caller's."""
    return C.c_void_p(stream.cuda_stream or 1)


class SPHtoGridError(RuntimeError):
    """Error raised by the library; ``status`` is the ABI status code."""

    def __init__(self, status: int, message: str):
        super().__init__(message)
        self.status = status


_lib = None
# re-entrant: default_context() holds it while Context() loads the library
_lock = threading.RLock()


def lib():
    """Load libsphgrid.so (fails loudly when it was not built)."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(LIB_PATH):
            raise ImportError(
                f"{LIB_PATH} is missing: build it with "
                "`python -c 'import __graft_entry__ as g; g.build()'` (nvcc, sm_103a)")
        L = C.CDLL(LIB_PATH)
        vp, i32, i64 = C.c_void_p, C.c_int, C.c_int64
        dp = C.POINTER(C.c_double)
        L.sphg_abi_version.restype = i32
        L.sphg_status_string.argtypes = [i32]
        L.sphg_status_string.restype = C.c_char_p
        L.sphg_context_create.argtypes = [i32, C.POINTER(vp)]
        L.sphg_context_create.restype = i32
        L.sphg_context_destroy.argtypes = [vp]
        L.sphg_context_destroy.restype = i32
        L.sphg_last_error.argtypes = [vp]
        L.sphg_last_error.restype = C.c_char_p
        L.sphg_mapping_parameters.argtypes = [dp, dp, dp, dp, C.c_double, C.c_double, C.c_double,
                                              C.c_double, i64, C.c_double, C.POINTER(SphgParams)]
        L.sphg_mapping_parameters.restype = i32
        L.sphg_output_len.argtypes = [C.POINTER(SphgParams), C.POINTER(SphgOptions), i32]
        L.sphg_output_len.restype = i64
        L.sphg_map.argtypes = [vp, C.POINTER(SphgParams), C.POINTER(SphgOptions),
                               C.POINTER(SphgParticles), vp, vp, C.POINTER(SphgStats)]
        L.sphg_map.restype = i32
        L.sphg_reduce.argtypes = [vp, C.POINTER(SphgParams), C.POINTER(SphgOptions), i32, vp, vp, vp]
        L.sphg_reduce.restype = i32
        L.sphg_adjoint.argtypes = [vp, C.POINTER(SphgParams), C.POINTER(SphgOptions),
                                   C.POINTER(SphgParticles), vp, vp, C.POINTER(SphgGrads), vp]
        L.sphg_adjoint.restype = i32
        L.sphg_map_projected.argtypes = [vp, C.POINTER(SphgParams), C.POINTER(SphgOptions),
                                         C.POINTER(SphgParticles), C.POINTER(SphgProjection), vp,
                                         vp, C.POINTER(SphgStats)]
        L.sphg_map_projected.restype = i32
        L.sphg_healpix_map.argtypes = [vp, C.POINTER(SphgHealpixParams), i64, vp, vp, vp, vp, vp, vp,
                                       vp, vp, vp, C.POINTER(SphgStats)]
        L.sphg_healpix_map.restype = i32
        L.sphg_probe_smem_rate.argtypes = [vp, C.c_int, C.POINTER(C.c_double)]
        L.sphg_probe_smem_rate.restype = i32
        L.sphg_probe_wait_timeout.argtypes = [vp, i32, C.POINTER(i32)]
        L.sphg_probe_wait_timeout.restype = i32
        L.sphg_probe_fixed_chunks.argtypes = [vp, i32, vp, vp]
        L.sphg_probe_fixed_chunks.restype = i32
        L.sphg_accumulate.argtypes = [vp, i64, vp, vp, vp]
        L.sphg_accumulate.restype = i32
        L.sphg_footprints.argtypes = [vp, C.POINTER(SphgParams), C.POINTER(SphgOptions),
                                      C.POINTER(SphgParticles), vp, vp, vp]
        L.sphg_footprints.restype = i32
        _lib = L
    return _lib


def check(status: int, ctx=None) -> None:
    if status != SPHG_OK:
        msg = lib().sphg_last_error(ctx).decode()
        raise SPHtoGridError(status, msg or lib().sphg_status_string(status).decode())


class Context:
    """Owns one ``sphg_context`` (device workspace, stream, pinned status)."""

    def __init__(self, device: int = 0):
        h = C.c_void_p()
        check(lib().sphg_context_create(int(device), C.byref(h)))
        self.handle = h
        self.device = device

    def close(self) -> None:
        if self.handle:
            lib().sphg_context_destroy(self.handle)
            self.handle = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


_contexts: dict[int, Context] = {}


def default_context(device: int = 0) -> Context:
    with _lock:
        ctx = _contexts.get(device)
        if ctx is None:
            ctx = Context(device)
            _contexts[device] = ctx
        return ctx


@atexit.register
def _close_all():
    for ctx in list(_contexts.values()):
        ctx.close()
    _contexts.clear()
