"""sphg_map_noalloc: the map for callers that cannot allocate device memory
-- code inside a host application that owns all device memory through its own
pool (an in-situ map under a fixed memory budget, a plugin whose host forbids
allocations during a time step).  Its scratch is a static device array of
SPHG_NOALLOC_SCRATCH_BYTES shared by all calls.

Checked through the C ABI against sphg_map (the entry point that allocates its
workspace) on two calls in a row and after calls of other shapes, within the
FP32C tolerance of the other tests; against the oracle; bitwise in the
deterministic mode; on the full-scratch error (with in-place centring left
undone); and for unchanged free device memory.  This file is collected last
(test_zz_...).
"""
import ctypes as C

import numpy as np
import pytest

from conftest import rel_linf

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

TOL = 1e-5  # the FP32C tolerance used by the parity tests
FLOOR = 1e-9


def _lib():
    from sphtogrid_gb300 import _lib as L
    lib = L.lib()
    lib.sphg_map_noalloc.argtypes = [C.POINTER(L.SphgParams), C.POINTER(L.SphgOptions),
                                     C.POINTER(L.SphgParticles), C.c_void_p, C.c_void_p,
                                     C.POINTER(L.SphgStats)]
    lib.sphg_map_noalloc.restype = C.c_int
    return L, lib


def _case(gpu, dims, n, P, nq, seed):
    L, _ = _lib()
    rng = np.random.default_rng(seed)
    dev = "cuda"
    pos = torch.tensor(rng.random((n, 3)), dtype=torch.float32, device=dev).T  # Julia layout
    hsml = torch.tensor(np.clip(np.exp(np.log(0.03) + 0.5 * rng.standard_normal(n)), 0.003, 0.2),
                        dtype=torch.float32, device=dev)
    m = torch.full((n,), 1.0 / n, dtype=torch.float32, device=dev)
    rho = torch.tensor(rng.uniform(0.5, 2.0, n), dtype=torch.float32, device=dev)
    q = torch.tensor(rng.uniform(0.5, 2.0, (nq, n)) if nq > 1 else rng.uniform(0.5, 2.0, n),
                     dtype=torch.float32, device=dev)
    par = gpu.mappingParameters(x_lim=[0, 1], y_lim=[0, 1], z_lim=[0, 1], Npixels=P)
    pt = L.SphgParticles()
    pt.n = n
    pt.pos_dtype = pt.attr_dtype = L.SPHG_F32
    pt.pos = pos.data_ptr()
    pt.pos_stride_p, pt.pos_stride_c = pos.stride(1), pos.stride(0)
    pt.hsml, pt.mass, pt.rho, pt.weights = (t.data_ptr() for t in (hsml, m, rho, rho))
    pt.bin_q = q.data_ptr()
    pt.n_q = nq
    pt.q_stride_p, pt.q_stride_k = (1, 0) if nq == 1 else (q.stride(1), q.stride(0))
    o = L.SphgOptions()
    o.dimensions = dims
    o.kernel = gpu.WendlandC4(dims).kind
    o.kernel_dim = dims
    o.reduce_image = 1
    o.precision = L.PREC["fp32c"]
    o.center = L.CENTER_READONLY
    o.filter = 1
    o.memspace = L.MEM_DEVICE
    keep = (pos, hsml, m, rho, q)
    return par, pt, o, keep


@pytest.mark.parametrize("dims,n,P,nq", [(2, 20000, 64, 2), (3, 3000, 24, 1)])
def test_noalloc_matches_sphg_map_on_two_calls(gpu, dims, n, P, nq):
    L, lib = _lib()
    par, pt, o, keep = _case(gpu, dims, n, P, nq, seed=dims)
    nout = lib.sphg_output_len(C.byref(par._c), C.byref(o), nq)
    ctx = gpu.default_context(0)
    ref = torch.empty(nout, dtype=torch.float64, device="cuda")
    st_ref = L.SphgStats()
    stream = torch.cuda.current_stream().cuda_stream
    L.check(lib.sphg_map(ctx.handle, C.byref(par._c), C.byref(o), C.byref(pt),
                         C.c_void_p(ref.data_ptr()), C.c_void_p(stream), C.byref(st_ref)), ctx.handle)
    for _ in range(2):  # the second call finds the first call's scratch contents
        out = torch.full((nout,), -1.0, dtype=torch.float64, device="cuda")
        st = L.SphgStats()
        status = lib.sphg_map_noalloc(C.byref(par._c), C.byref(o), C.byref(pt),
                                      C.c_void_p(out.data_ptr()), C.c_void_p(stream), C.byref(st))
        assert status == 0, lib.sphg_last_error(None).decode()
        assert st.deposits == st_ref.deposits and st.n_mapped == st_ref.n_mapped
        assert rel_linf(out.cpu().numpy(), ref.cpu().numpy(), FLOOR) <= TOL


def test_noalloc_rejects_calls_beyond_its_scratch(gpu):
    L, lib = _lib()
    par, pt, o, keep = _case(gpu, 2, 16, 32, 1, seed=5)
    pt.n = 2_000_000  # records alone need more than the scratch: rejected before any access
    out = torch.empty(32 * 32, dtype=torch.float64, device="cuda")
    status = lib.sphg_map_noalloc(C.byref(par._c), C.byref(o), C.byref(pt),
                                  C.c_void_p(out.data_ptr()), None, None)
    assert status == L.SPHG_ERR_ARG
    assert b"no-allocation scratch" in lib.sphg_last_error(None)


def _map_ref(gpu, L, lib, par, o, pt, nout):
    ctx = gpu.default_context(0)
    ref = torch.empty(nout, dtype=torch.float64, device="cuda")
    st = L.SphgStats()
    stream = torch.cuda.current_stream().cuda_stream
    L.check(lib.sphg_map(ctx.handle, C.byref(par._c), C.byref(o), C.byref(pt), C.c_void_p(ref.data_ptr()),
                         C.c_void_p(stream), C.byref(st)), ctx.handle)
    return ref, st


def _noalloc(L, lib, par, o, pt, nout):
    out = torch.full((nout,), -1.0, dtype=torch.float64, device="cuda")
    st = L.SphgStats()
    stream = torch.cuda.current_stream().cuda_stream
    status = lib.sphg_map_noalloc(C.byref(par._c), C.byref(o), C.byref(pt), C.c_void_p(out.data_ptr()),
                                  C.c_void_p(stream), C.byref(st))
    return status, out, st


def test_noalloc_against_oracle_and_deterministic(gpu, oracle):
    """The no-allocation map against the oracle on the pixels carrying
    weight, and in the deterministic mode bitwise equal to sphg_map's."""
    L, lib = _lib()
    dims, n, P, nq = 2, 20000, 64, 2
    par, pt, o, keep = _case(gpu, dims, n, P, nq, seed=11)
    pos, hsml, m, rho, q = keep
    nout = lib.sphg_output_len(C.byref(par._c), C.byref(o), nq)
    status, out, st = _noalloc(L, lib, par, o, pt, nout)
    assert status == 0, lib.sphg_last_error(None).decode()
    opar = oracle.mapping_parameters(x_lim=[0, 1], y_lim=[0, 1], z_lim=[0, 1], Npixels=P)
    host = [t.cpu().numpy() for t in (hsml, m, rho, q, rho)]
    pos_h = np.asfortranarray(pos.cpu().numpy())
    ref, info = oracle.sph_mapping(pos_h.copy(order="F"), *host, param=opar, kernel="wendlandc4", dimensions=2)
    raw, _ = oracle.sph_mapping(pos_h.copy(order="F"), *host, param=opar, kernel="wendlandc4", dimensions=2,
                                return_both_maps=True)
    assert st.deposits == info["deposits"]
    W = raw[:, -1].reshape(P, P)  # rows x*P + y
    keep_px = W >= 1e-6 * W.max()
    got = out.cpu().numpy().reshape(nq, P, P).transpose(2, 1, 0)  # stored [x, y, q], x fastest
    ref = np.asarray(ref).reshape(P, P, nq)
    for k in range(nq):
        err = np.abs(got[..., k] - ref[..., k])[keep_px] / np.abs(ref[..., k])[keep_px]
        assert err.max() <= TOL
    o.deterministic = 1
    ref_det, _ = _map_ref(gpu, L, lib, par, o, pt, nout)
    for _ in range(2):
        status, out_det, _ = _noalloc(L, lib, par, o, pt, nout)
        assert status == 0, lib.sphg_last_error(None).decode()
        assert torch.equal(out_det, ref_det)


def test_noalloc_after_a_call_of_another_shape(gpu):
    """Calls of different layouts in a row (a large 2D map, a 3D map, a 2D
    raw accumulator): stale scratch contents sit at other offsets."""
    L, lib = _lib()
    for dims, n, P, nq, raw in ((2, 40000, 128, 3, 0), (3, 5000, 32, 1, 0), (2, 8000, 48, 1, 1)):
        par, pt, o, keep = _case(gpu, dims, n, P, nq, seed=20 + dims)
        o.return_both_maps = raw
        nout = lib.sphg_output_len(C.byref(par._c), C.byref(o), nq)
        ref, st_ref = _map_ref(gpu, L, lib, par, o, pt, nout)
        status, out, st = _noalloc(L, lib, par, o, pt, nout)
        assert status == 0, lib.sphg_last_error(None).decode()
        assert st.deposits == st_ref.deposits
        assert rel_linf(out.cpu().numpy(), ref.cpu().numpy(), FLOOR) <= TOL


def test_noalloc_full_scratch_leaves_positions_uncentred(gpu):
    """A call that passes the up-front size check but fills the pair records
    (a hundred particles of h = 0.2 on 4096^2) returns SPHG_ERR_ALLOC; with
    in-place centring the positions are left as they were, so the retry
    through sphg_map with the same options centres them once."""
    L, lib = _lib()
    n, P = 100, 4096
    rng = np.random.default_rng(9)
    pos0 = torch.tensor(rng.uniform(0.2, 0.8, (n, 3)), dtype=torch.float32, device="cuda")
    pos = pos0.clone().T  # (3, N), xyz contiguous per particle
    h = torch.full((n,), 0.2, dtype=torch.float32, device="cuda")
    m = torch.full((n,), 1.0 / n, dtype=torch.float32, device="cuda")
    rho = torch.tensor(rng.uniform(0.5, 2.0, n), dtype=torch.float32, device="cuda")
    par = gpu.mappingParameters(center=[0.5, 0.5, 0.5], x_size=1.0, y_size=1.0, z_size=1.0, Npixels=P)
    pt = L.SphgParticles()
    pt.n = n
    pt.pos_dtype = pt.attr_dtype = L.SPHG_F32
    pt.pos = pos.data_ptr()
    pt.pos_stride_p, pt.pos_stride_c = pos.stride(1), pos.stride(0)
    pt.hsml, pt.mass, pt.rho, pt.weights = (t.data_ptr() for t in (h, m, rho, rho))
    pt.bin_q = rho.data_ptr()
    pt.n_q = 1
    pt.q_stride_p, pt.q_stride_k = 1, 0
    o = L.SphgOptions()
    o.dimensions = 2
    o.kernel = gpu.Cubic(2).kind
    o.kernel_dim = 2
    o.reduce_image = 1
    o.precision = L.PREC["fp32c"]
    o.center = L.CENTER_INPLACE
    o.filter = 1
    o.memspace = L.MEM_DEVICE
    nout = lib.sphg_output_len(C.byref(par._c), C.byref(o), 1)
    status, _, _ = _noalloc(L, lib, par, o, pt, nout)
    assert status == L.SPHG_ERR_ALLOC
    assert b"positions were left uncentred" in lib.sphg_last_error(None)
    assert torch.equal(pos.T, pos0)
    ref_pos = pos0.clone().T
    o_ro = L.SphgOptions.from_buffer_copy(o)
    o_ro.center = L.CENTER_READONLY
    pt_ro = L.SphgParticles.from_buffer_copy(pt)
    pt_ro.pos = ref_pos.data_ptr()
    ref, _ = _map_ref(gpu, L, lib, par, o_ro, pt_ro, nout)
    out, _ = _map_ref(gpu, L, lib, par, o, pt, nout)  # the retry, centring in place
    assert rel_linf(out.cpu().numpy(), ref.cpu().numpy(), FLOOR) <= TOL
    assert torch.equal(pos.T, (pos0 - 0.5))  # centred once (exact: x - 0.5 in Float32)


def test_noalloc_takes_no_device_memory(gpu):
    """Free device memory is the same before and after a call (after a first
    call, which may load the library's device code and its static array)."""
    L, lib = _lib()
    par, pt, o, keep = _case(gpu, 2, 20000, 64, 1, seed=31)
    nout = lib.sphg_output_len(C.byref(par._c), C.byref(o), 1)
    out = torch.empty(nout, dtype=torch.float64, device="cuda")
    st = L.SphgStats()

    def call():
        return lib.sphg_map_noalloc(C.byref(par._c), C.byref(o), C.byref(pt), C.c_void_p(out.data_ptr()), None,
                                    C.byref(st))

    assert call() == 0
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(3):
        assert call() == 0
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0
