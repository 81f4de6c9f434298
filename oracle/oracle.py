"""ctypes binding of the C oracle (``oracle/sph_oracle.c``).

TEST INFRASTRUCTURE ONLY: imported by ``tests/``, ``__graft_entry__.smoke()``
and the CPU-baseline leg of ``bench.py`` as the oracle.  The product never
imports this module.

The oracle restates SPHtoGrid.jl's FP64 ``sphMapping`` path
(src/cic_interpolation/*.jl, src/shared/parameters.jl); see the header of
``sph_oracle.c`` for what is pinned and what is not (kernel shapes: parity
unpinned).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
SRC_PATH = os.path.join(HERE, "sph_oracle.c")

KERNELS = {"cubic": 0, "quintic": 1, "wendlandc4": 2, "wendlandc6": 3, "wendlandc8": 4}

ERRORS = {
    1: "Giving a center position requires extent in x, y and z direction.",
    2: "Please specify pixelSideLength or number of pixels!",
    3: "dimensions must be 2 or 3",
    4: "non-finite pixel range (InexactError in floor)",
    5: "3D mapping takes one scalar quantity",
    6: "allocation failed",
    7: "bad argument",
}


class OrcParams(C.Structure):
    """Field-for-field image of ``mappingParameters`` (parameters.jl:14-27)."""

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

    def as_dict(self):
        return {
            "x_lim": list(self.x_lim), "y_lim": list(self.y_lim), "z_lim": list(self.z_lim),
            "center": list(self.center), "halfsize": list(self.halfsize),
            "len2pix": self.len2pix, "pixelSideLength": self.pixelSideLength,
            "Npixels": list(self.Npixels), "boxsize": self.boxsize, "periodic": bool(self.periodic),
        }


class OracleError(RuntimeError):
    pass


HP_SRC_PATH = os.path.join(HERE, "healpix_oracle.c")


def build(force: bool = False) -> str:
    """Compile the oracle with gcc (no FMA contraction, so the expression order
    of the reference is kept)."""
    newest = max(os.path.getmtime(SRC_PATH), os.path.getmtime(HP_SRC_PATH))
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < newest:
        subprocess.check_call(
            ["gcc", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared",
             "-o", LIB_PATH, SRC_PATH, HP_SRC_PATH, "-lm", "-lpthread"])
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB_PATH)
        dp, vp, i64, i32 = C.POINTER(C.c_double), C.c_void_p, C.c_int64, C.c_int
        L.orc_mapping_parameters.argtypes = [dp, dp, dp, dp, C.c_double, C.c_double, C.c_double,
                                             C.c_double, i64, C.c_double, C.POINTER(OrcParams)]
        L.orc_mapping_parameters.restype = i32
        L.orc_center_particles.argtypes = [i32, vp, i64, i64, i64, C.POINTER(OrcParams), C.POINTER(OrcParams)]
        L.orc_center_particles.restype = i32
        L.orc_filter_particles.argtypes = [i32, vp, i64, i64, i64, C.POINTER(OrcParams), vp]
        L.orc_filter_particles.restype = None
        L.orc_calculate_index_2d.argtypes = [i64, i64, i64]
        L.orc_calculate_index_2d.restype = i64
        L.orc_calculate_index_3d.argtypes = [i64, i64, i64, i64, i64]
        L.orc_calculate_index_3d.restype = i64
        L.orc_kernel_value.argtypes = [i32, i32, C.c_double, C.c_double]
        L.orc_kernel_value.restype = C.c_double
        L.orc_reduce_image_2d.argtypes = [vp, i64, i32, i32, vp]
        L.orc_reduce_image_3d.argtypes = [vp, i64, vp]
        L.orc_footprints.argtypes = [i32, C.POINTER(OrcParams), i32, vp, i64, i64, i32, vp, vp, i32,
                                     i64, i64, i32, i64, vp, vp]
        L.orc_footprints.restype = i32
        L.orc_sph_mapping.argtypes = [C.POINTER(OrcParams), i32, i32, i32, i32, vp, i64, i64, i32,
                                      vp, vp, vp, vp, i32, i64, i64, vp, i64, i32, i32, i32, i32, i32,
                                      vp, dp, C.POINTER(C.c_int64)]
        L.orc_sph_mapping.restype = i32
        L.orc_particle_contrib.argtypes = [i32, C.POINTER(OrcParams), i32, i32, C.c_double, C.c_double,
                                           C.c_double, C.c_double, C.c_double, C.c_double, C.c_double,
                                           i64, vp, vp]
        L.orc_particle_contrib.restype = i64
        L.hp_pix2vec_ring.argtypes = [i64, i64, dp]
        L.hp_pix2vec_ring.restype = None
        L.hp_ang2pix_ring.argtypes = [i64, C.c_double, C.c_double]
        L.hp_ang2pix_ring.restype = i64
        L.hp_vec2ang.argtypes = [C.c_double, C.c_double, C.c_double, dp, dp]
        L.hp_vec2ang.restype = None
        L.hp_query_disc_ring.argtypes = [i64, C.c_double, C.c_double, C.c_double, vp, i64]
        L.hp_query_disc_ring.restype = i64
        L.orc_healpix_map.argtypes = [i64, i32, i32, i32, i64, vp, vp, vp, vp, vp, vp, vp, vp, dp, dp]
        L.orc_healpix_map.restype = i64
        _lib = L
    return _lib


def mapping_parameters(x_lim=(-1.0, -1.0), y_lim=(-1.0, -1.0), z_lim=(-1.0, -1.0),
                       center=(-1.0, -1.0, -1.0), x_size=-1.0, y_size=-1.0, z_size=-1.0,
                       pixelSideLength=-1.0, Npixels=0, boxsize=-1.0) -> OrcParams:
    """``mappingParameters(...)`` (parameters.jl:44-125) with the reference's
    sentinel defaults."""
    arr = lambda v: (C.c_double * len(v))(*[float(x) for x in v])
    out = OrcParams()
    st = lib().orc_mapping_parameters(arr(x_lim), arr(y_lim), arr(z_lim), arr(center),
                                      float(x_size), float(y_size), float(z_size),
                                      float(pixelSideLength), int(Npixels), float(boxsize),
                                      C.byref(out))
    if st:
        raise OracleError(ERRORS[st])
    return out


def _dtype_code(a: np.ndarray) -> int:
    if a.dtype == np.float32:
        return 0
    if a.dtype == np.float64:
        return 1
    raise TypeError(f"unsupported dtype {a.dtype}")


def _pos_strides(pos: np.ndarray):
    """Element strides (particle, component) of a (3, N) array in any order."""
    if pos.ndim != 2 or pos.shape[0] != 3:
        raise ValueError("Pos must have shape (3, N)")
    es = pos.itemsize
    return pos.strides[1] // es, pos.strides[0] // es


def _q_layout(q: np.ndarray):
    """(nq, particle stride, quantity stride) for an (N,) or (Nq, N) array."""
    es = q.itemsize
    if q.ndim == 1:
        return 1, q.strides[0] // es, 0
    return q.shape[0], q.strides[1] // es, q.strides[0] // es


def center_particles(pos: np.ndarray, par: OrcParams) -> OrcParams:
    sp, sc = _pos_strides(pos)
    out = OrcParams()
    st = lib().orc_center_particles(_dtype_code(pos), pos.ctypes.data, pos.shape[1], sp, sc,
                                    C.byref(par), C.byref(out))
    if st:
        raise OracleError(ERRORS[st])
    return out


def filter_particles_in_image(pos: np.ndarray, par: OrcParams) -> np.ndarray:
    sp, sc = _pos_strides(pos)
    mask = np.zeros(pos.shape[1], dtype=np.uint8)
    lib().orc_filter_particles(_dtype_code(pos), pos.ctypes.data, pos.shape[1], sp, sc,
                               C.byref(par), mask.ctypes.data)
    return mask.astype(bool)


def calculate_index(*args) -> int:
    if len(args) == 3:
        return lib().orc_calculate_index_2d(*args)
    return lib().orc_calculate_index_3d(*args)


def kernel_value(kernel: str, kdim: int, u: float, h_inv: float) -> float:
    return lib().orc_kernel_value(KERNELS[kernel], kdim, u, h_inv)


def footprints(dims, par, pos, hsml, q, calc_mean=False):
    """Per-particle integer pixel ranges and state (see ``orc_footprints``) on
    already-centred positions."""
    sp, sc = _pos_strides(pos)
    nq, qsp, qsc = _q_layout(q)
    n = pos.shape[1]
    rng = np.zeros((n, 6), dtype=np.int64)
    state = np.zeros(n, dtype=np.int8)
    st = lib().orc_footprints(dims, C.byref(par), _dtype_code(pos), pos.ctypes.data, sp, sc,
                              _dtype_code(hsml), hsml.ctypes.data, q.ctypes.data, nq, qsp, qsc,
                              int(calc_mean), n, rng.ctypes.data, state.ctypes.data)
    if st:
        raise OracleError(ERRORS[st])
    return rng, state


def particle_contrib(dims, par, kernel, kdim, x, y, z, hsml, m, rho, w, cap=1 << 22):
    """(flat pixel indices, weights pw) of one particle with centred position."""
    idx = np.zeros(cap, dtype=np.int64)
    pw = np.zeros(cap)
    n = lib().orc_particle_contrib(dims, C.byref(par), KERNELS[kernel], kdim, x, y, z, hsml, m,
                                   rho, w, cap, idx.ctypes.data, pw.ctypes.data)
    if n < 0:
        raise OracleError("particle_contrib failed")
    return idx[:n].copy(), pw[:n].copy()


def sph_mapping(Pos, HSML, M, Rho, Bin_Quant, Weights=None, *, param: OrcParams, kernel="cubic",
                kernel_dim=None, reduce_image=True, return_both_maps=False, dimensions=2,
                calc_mean=False, sort_z=False, nthreads=1, copy_pos=True, raw3d=False):
    """Oracle ``sphMapping`` (cic_interpolation.jl:35-272).

    Positions are centred in place as in the reference unless ``copy_pos``.
    Returns ``(image, info)`` with ``info = {grid_mass, deposits, param}``.
    Layouts of ``image``: numpy arrays in Fortran order whose indices equal the
    reference's (0-based): 2D ``[x, y, q]``, 3D ``[z, y, x]``, raw
    ``[pixel, channel]``.
    """
    if Weights is None:
        Weights = Rho
    pos = np.array(Pos, copy=True) if copy_pos else Pos
    attrs = [np.asarray(a) for a in (HSML, M, Rho, Bin_Quant, Weights)]
    adt = np.float64 if any(a.dtype == np.float64 or a.dtype.kind in "iu" for a in attrs) else np.float32
    hsml, m, rho, q, w = [np.ascontiguousarray(a, dtype=adt) for a in attrs]
    nq, qsp, qsc = _q_layout(q)
    sp, sc = _pos_strides(pos)
    P = int(param.Npixels[0])
    if dimensions == 2:
        out = np.zeros(P * P * (nq + 1) if return_both_maps else P * P * nq)
    elif dimensions == 3:
        out = np.zeros(2 * P ** 3 if raw3d else P ** 3)
    else:
        raise OracleError(ERRORS[3])
    par = OrcParams.from_buffer_copy(param)
    gm = C.c_double(0.0)
    dep = C.c_int64(0)
    kdim = dimensions if kernel_dim is None else kernel_dim
    st = lib().orc_sph_mapping(C.byref(par), dimensions, KERNELS[kernel], kdim, _dtype_code(pos),
                               pos.ctypes.data, sp, sc, _dtype_code(hsml), hsml.ctypes.data,
                               m.ctypes.data, rho.ctypes.data, q.ctypes.data, nq, qsp, qsc,
                               w.ctypes.data, pos.shape[1], int(reduce_image),
                               2 if (raw3d and dimensions == 3) else int(return_both_maps),
                               int(calc_mean), int(sort_z), int(nthreads), out.ctypes.data,
                               C.byref(gm), C.byref(dep))
    if st:
        raise OracleError(ERRORS[st])
    if dimensions == 2 and return_both_maps:
        image = out.reshape((P * P, nq + 1), order="F")
    elif dimensions == 3 and raw3d:
        image = out.reshape((P ** 3, 2), order="F")
    elif dimensions == 2:
        image = out.reshape((P, P, nq), order="F")
    else:
        image = out.reshape((P, P, P), order="F")
    return image, {"grid_mass": gm.value, "deposits": dep.value, "param": par}


# ---------------------------------------------------------------- HEALPix

def hp_pix2vec(nside: int, pix: int) -> np.ndarray:
    v = (C.c_double * 3)()
    lib().hp_pix2vec_ring(int(nside), int(pix), v)
    return np.array(v[:])


def hp_ang2pix(nside: int, theta: float, phi: float) -> int:
    return int(lib().hp_ang2pix_ring(int(nside), float(theta), float(phi)))


def hp_vec2ang(x: float, y: float, z: float):
    t, p = C.c_double(), C.c_double()
    lib().hp_vec2ang(float(x), float(y), float(z), C.byref(t), C.byref(p))
    return t.value, p.value


def hp_query_disc(nside: int, theta: float, phi: float, radius: float) -> np.ndarray:
    cap = 1024
    while True:
        out = np.empty(cap, dtype=np.int64)
        n = lib().hp_query_disc_ring(int(nside), float(theta), float(phi), float(radius), out.ctypes.data, cap)
        if n <= cap:
            return out[:n].copy()
        cap = int(n)


def filter_sort_particles(Pos, Hsml, M, Rho, Bin_q, Weights, center, radius_limits, calc_mean):
    """filter_sort_particles (filter_particles.jl:19-53) with its selection as
    written: the input-order shell mask `sel` picks entries of the descending
    distance permutation, `sorted[sel]`.  Centres the caller's Pos in place."""
    Pos -= np.asarray(center, dtype=Pos.dtype)[:, None]
    dx = np.sqrt(Pos[0] ** 2 + Pos[1] ** 2 + Pos[2] ** 2)
    sel = (radius_limits[0] <= dx) & (dx <= radius_limits[1])
    if not calc_mean:
        sel = sel[Bin_q[sel] > 0.0]  # raises unless the lengths agree, as the reference does
    order = np.argsort(dx, kind="stable")[::-1]
    idx = order[sel]
    return (np.ascontiguousarray(Pos[:, idx].T), Hsml[idx], M[idx], Rho[idx], Bin_q[idx], Weights[idx])


def healpix_map(Pos, Hsml, M, Rho, Bin_q, Weights, *, center=(0.0, 0.0, 0.0),
                radius_limits=(0.0, np.inf), Nside=1024, kernel="cubic", kernel_dim=3, calc_mean=True):
    """healpix_map (main.jl:92-227) in FP64 (the reference's path takes
    Float64 inputs only: calculate_weights ties its Float64 weight arrays to
    the position type).  Returns (allsky_map, weight_map, info)."""
    npix = 12 * Nside * Nside
    allsky = np.zeros(npix)
    weight = np.zeros(npix)
    if not calc_mean and np.sum(Bin_q) == 0:
        return allsky, weight, {"mapped": 0}
    pos, h, m, rho, q, w = filter_sort_particles(Pos, np.asarray(Hsml, np.float64),
                                                 np.asarray(M, np.float64), np.asarray(Rho, np.float64),
                                                 np.asarray(Bin_q, np.float64),
                                                 np.asarray(Weights, np.float64), center,
                                                 radius_limits, calc_mean)
    arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (pos, h, m, rho, q, w)]
    gm, pm = C.c_double(), C.c_double()
    mapped = lib().orc_healpix_map(int(Nside), KERNELS[kernel], int(kernel_dim), int(bool(calc_mean)),
                                   arrs[1].shape[0], *[a.ctypes.data for a in arrs],
                                   allsky.ctypes.data, weight.ctypes.data, C.byref(gm), C.byref(pm))
    return allsky, weight, {"mapped": mapped, "grid_mass": gm.value, "particle_mass": pm.value,
                            "selected": arrs[1].shape[0]}
