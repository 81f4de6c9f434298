"""sphg_map_noalloc: the map for callers that cannot allocate device memory
-- code inside a host application that owns all device memory through its own
pool (an in-situ map under a fixed memory budget, a plugin whose host forbids
allocations during a time step).  Its scratch is a static device array of
SPHG_NOALLOC_SCRATCH_BYTES shared by all calls.

Checked through the C ABI against sphg_map (the entry point that allocates its
workspace) on two calls in a row, within the FP32C tolerance of the other
tests.  This file is collected last (test_zz_...).
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
