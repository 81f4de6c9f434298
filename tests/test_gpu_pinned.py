"""Page-locked (pinned) host buffers on the FP32C path are read and written in
place over the host link (no staging copies).  The map equals the staged
(pageable host) path's and the device path's, bit for bit in the
deterministic mode, and in-place centring lands in the caller's pinned
array as it does in a pageable one."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _case(seed, n, dims, nq):
    rng = np.random.default_rng(seed)
    pos = (0.5 + 0.25 * rng.standard_normal((3, n))).astype(np.float32)
    hsml = np.clip(np.exp(np.log(0.03) + 0.5 * rng.standard_normal(n)), 0.005, 0.2).astype(np.float32)
    m = np.full(n, 1.0 / n, np.float32)
    rho = rng.uniform(0.5, 2.0, n).astype(np.float32)
    q = rng.uniform(0.5, 2.0, (nq, n)).astype(np.float32) if nq > 1 else rng.uniform(0.5, 2.0, n).astype(np.float32)
    return pos, hsml, m, rho, q


def _map(gpu, arrays, n, nq, dims, P, det, mem, inplace):
    """One sphg_map call; `arrays` are (pos (N, 3) rows, hsml, m, rho, w, q)
    as torch tensors (CUDA, pinned or pageable CPU); returns the output and
    the positions after the call."""
    from sphtogrid_gb300 import _lib
    from sphtogrid_gb300.mapping import _options
    par = gpu.mappingParameters(x_lim=[0, 1], y_lim=[0, 1], z_lim=[0, 1], Npixels=P)
    kern = gpu.WendlandC6(dims) if dims == 3 else gpu.WendlandC4(2)
    center = _lib.CENTER_INPLACE if inplace else _lib.CENTER_READONLY
    o = _options(par, kern, dims, True, dims == 2, False, "fp32c", det, center, 1, mem)
    out_len = _lib.lib().sphg_output_len(C.byref(par._c), C.byref(o), nq)
    pos, hsml, m, rho, w, q = arrays
    if mem == _lib.MEM_DEVICE:
        out = torch.zeros(out_len, dtype=torch.float64, device=pos.device)
    else:
        out = torch.zeros(out_len, dtype=torch.float64).pin_memory() if pos.is_pinned() \
            else torch.zeros(out_len, dtype=torch.float64)
    pt = _lib.SphgParticles()
    pt.n = n
    pt.pos_dtype = pt.attr_dtype = _lib.SPHG_F32
    pt.pos, pt.hsml, pt.mass, pt.rho, pt.weights, pt.bin_q = (t.data_ptr() for t in (pos, hsml, m, rho, w, q))
    pt.pos_stride_p, pt.pos_stride_c = 3, 1
    pt.n_q = nq
    pt.q_stride_p, pt.q_stride_k = (1, n) if nq > 1 else (1, 0)
    st = _lib.SphgStats()
    ctx = _lib.default_context(0)
    _lib.check(_lib.lib().sphg_map(ctx.handle, C.byref(par._c), C.byref(o), C.byref(pt),
                                   C.c_void_p(out.data_ptr()), None, C.byref(st)), ctx.handle)
    torch.cuda.synchronize()
    return out.cpu().numpy(), pos.cpu().numpy(), st.deposits


@pytest.mark.parametrize("dims,nq,P", [(3, 1, 48), (2, 3, 96)])
@pytest.mark.parametrize("det", [True, False])
def test_pinned_host_buffers_in_place(gpu, dims, nq, P, det):
    from sphtogrid_gb300 import _lib
    n = 20000
    pos, hsml, m, rho, q = _case(5 + dims, n, dims, nq)
    host = [np.ascontiguousarray(pos.T), hsml, m, rho, rho.copy(), np.ascontiguousarray(q)]

    def tensors(kind):
        ts = [torch.from_numpy(a.copy()) for a in host]
        if kind == "pinned":
            ts = [t.pin_memory() for t in ts]
        elif kind == "device":
            ts = [t.cuda() for t in ts]
        return ts

    res = {}
    for kind in ("pinned", "pageable", "device"):
        mem = _lib.MEM_DEVICE if kind == "device" else _lib.MEM_HOST
        res[kind] = _map(gpu, tensors(kind), n, nq, dims, P, det, mem, inplace=True)
    img_p, pos_p, dep_p = res["pinned"]
    for kind in ("pageable", "device"):
        img, pos_k, dep = res[kind]
        assert dep == dep_p
        assert np.array_equal(pos_p, pos_k), kind  # centred once, in the caller's array
        if det:
            assert np.array_equal(img_p, img), kind
        else:
            scale = np.abs(img).max()
            assert np.abs(img_p - img).max() <= 1e-12 * scale, kind
    # the map is not empty and the positions moved by the centring
    assert np.abs(img_p).max() > 0
    assert not np.array_equal(pos_p, host[0])
