"""The hand-written adjoint (sphg_adjoint through the torch autograd Function)
against FP64 central finite differences of the oracle and forward-mode dual
numbers through the Python restatement.

Tolerance: |adjoint - reference| <= 1e-4 * max(|reference|, 1e-3 * scale),
scale being the largest reference gradient of that parameter over the
sampled particles (absolute floor for gradients that are near zero).
"""
import numpy as np
import pytest

from adjoint_ref import PARAMS, dual_grad, fd_grad, reduce_rows, rows_to_output

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _case(seed, n, nq=1, hmin=0.02, hmax=0.2, spread=0.5):
    rng = np.random.default_rng(seed)
    pos = np.asfortranarray(rng.uniform(-spread, spread, (3, n)))
    hsml = np.exp(rng.uniform(np.log(hmin), np.log(hmax), n))
    m = rng.uniform(0.5, 1.5, n) / n
    rho = rng.uniform(0.5, 2.0, n)
    q = rng.uniform(0.5, 2.0, (nq, n)) if nq > 1 else rng.uniform(0.5, 2.0, n)
    w = rng.uniform(0.5, 2.0, n)
    return pos, hsml, m, rho, q, w


def _gpu_grads(gpu, case, P, dims, kernel, target_out, precision="fp64", adjoint_precision=None):
    pos, hsml, m, rho, q, w = case
    par = gpu.mappingParameters(center=[0.0, 0.0, 0.0], x_size=1.0, y_size=1.0, z_size=1.0,
                                Npixels=P)
    dev = "cuda"
    tpos = torch.tensor(np.ascontiguousarray(pos.T), device=dev).T.requires_grad_(True)
    ts = [torch.tensor(np.ascontiguousarray(a), device=dev, requires_grad=True)
          for a in (hsml, m, rho, q, w)]
    out = gpu.sph_map_differentiable(tpos, ts[0], ts[1], ts[2], ts[3], ts[4], param=par,
                                     kernel=gpu.kernel_from_name(kernel, dims), dimensions=dims,
                                     precision=precision, adjoint_precision=adjoint_precision)
    t = torch.tensor(target_out, device=dev)
    flat = out.permute(*reversed(range(out.dim()))).reshape(-1)
    loss = ((flat - t) ** 2).sum()
    loss.backward()
    g = {"x": tpos.grad[0], "y": tpos.grad[1], "z": tpos.grad[2], "hsml": ts[0].grad,
         "mass": ts[1].grad, "rho": ts[2].grad, "q": ts[3].grad, "weights": ts[4].grad}
    return {k: v.detach().cpu().numpy() for k, v in g.items()}, out.detach().cpu().numpy()


def _setup(oracle, case, P, dims, kernel, seed=3):
    par = oracle.mapping_parameters(center=[0.0, 0.0, 0.0], x_size=1.0, y_size=1.0, z_size=1.0,
                                    Npixels=P)
    raw, _ = oracle.sph_mapping(*case, param=par, kernel=kernel, dimensions=dims,
                                return_both_maps=True, raw3d=True)
    out = reduce_rows(raw, dims)
    target = out * np.random.default_rng(seed).lognormal(0.0, 0.1, out.shape)
    return par, raw, out, target


@pytest.mark.parametrize("precision,adjoint", [("fp64", "fp64"), ("fp64", "fp32c")])
@pytest.mark.parametrize("dims,kernel,nq", [(2, "cubic", 1), (2, "wendlandc4", 3),
                                            (2, "quintic", 1), (3, "wendlandc6", 1),
                                            (3, "wendlandc8", 1)])
def test_adjoint_vs_finite_differences(gpu, oracle, dims, kernel, nq, precision, adjoint):
    """FP64 throughout, and the FP32C adjoint (per-cell weights and
    derivatives in FP32 with compensated sums, FP64 redo where its error
    estimate exceeds 1e-5) after the FP64 forward.  (After the FP32C forward
    the adjoint differentiates the FP32C map's loss, which differs from the
    FP64 loss at pixels of tiny W: test_adjoint_fp32c_forward.)"""
    n, P = (400, 32) if dims == 2 else (150, 16)
    case = _case(dims * 10 + nq, n, nq)
    par, raw, out, target = _setup(oracle, case, P, dims, kernel)
    grads, out_gpu = _gpu_grads(gpu, case, P, dims, kernel, rows_to_output(target, dims, P),
                                precision=precision, adjoint_precision=adjoint)
    # the forward matches the oracle
    ref_out = rows_to_output(out, dims, P)
    if precision == "fp64":
        assert np.allclose(out_gpu.reshape(-1, order="F"), ref_out, rtol=1e-11,
                           atol=1e-13 * np.abs(out).max())
    else:
        assert np.abs(out_gpu.reshape(-1, order="F") - ref_out).max() <= 1e-5 * np.abs(ref_out).max()
    parts = np.random.default_rng(1).choice(n, size=24, replace=False)
    for name in PARAMS:
        if dims == 2 and name == "z":
            continue
        ks = range(nq) if name == "q" else [0]
        for k in ks:
            ref = np.array([fd_grad(oracle, case, par, dims, kernel, dims, raw, target, int(p), name, k)
                            for p in parts])
            if name == "q":
                got = grads["q"].reshape(nq, -1)[k, parts] if nq > 1 else grads["q"][parts]
            else:
                got = grads[name][parts]
            scale = np.abs(ref).max()
            tol = 1e-4 * np.maximum(np.abs(ref), 1e-3 * scale) + 1e-300
            bad = np.abs(got - ref) > tol
            assert not bad.any(), (name, k, parts[bad], got[bad], ref[bad])


def test_adjoint_vs_dual_numbers(gpu, oracle, pyoracle):
    dims, kernel, n, P = 2, "wendlandc6", 30, 12
    case = _case(77, n, 1, hmin=0.05, hmax=0.3)
    par, raw, out, target = _setup(oracle, case, P, dims, kernel)
    grads, _ = _gpu_grads(gpu, case, P, dims, kernel, rows_to_output(target, dims, P))
    for p in (0, 7, 19):
        for name in ("x", "y", "hsml", "mass", "rho", "weights", "q"):
            du = dual_grad(pyoracle, case, par, dims, kernel, dims, target, p, name)
            got = grads[name][p]
            assert abs(got - du) <= 1e-6 * abs(du) + 1e-12, (p, name, got, du)


@pytest.mark.parametrize("adjoint", ["fp64", "fp32c"])
def test_adjoint_fallback_and_tiny_particles(gpu, oracle, adjoint):
    # sub-pixel particles: g = A in the fallback branch (the FP32C adjoint
    # takes these through its FP64 path, next to FP32 particles)
    dims, kernel, n, P = 2, "cubic", 300, 24
    case = _case(5, n, 1, hmin=0.002, hmax=0.03)
    par, raw, out, target = _setup(oracle, case, P, dims, kernel)
    grads, _ = _gpu_grads(gpu, case, P, dims, kernel, rows_to_output(target, dims, P),
                          adjoint_precision=adjoint)
    for name in ("x", "hsml", "mass", "q"):
        ref = np.array([fd_grad(oracle, case, par, dims, kernel, dims, raw, target, p, name)
                        for p in range(0, n, 10)])
        got = grads[name][0:n:10]
        scale = np.abs(ref).max()
        assert np.all(np.abs(got - ref) <= 1e-4 * np.maximum(np.abs(ref), 1e-3 * scale) + 1e-300)


def test_adjoint_fp32c_forward(gpu, oracle):
    """The differentiable path in FP32C (forward and adjoint): map within 1e-5
    and the adjoint within 1e-4 of the finite differences."""
    dims, kernel, n, P = 2, "wendlandc4", 400, 32
    case = _case(9, n, 1)
    par, raw, out, target = _setup(oracle, case, P, dims, kernel)
    grads, out_gpu = _gpu_grads(gpu, case, P, dims, kernel, rows_to_output(target, dims, P),
                                precision="fp32c")
    ref_out = rows_to_output(out, dims, P)
    assert np.abs(out_gpu.reshape(-1, order="F") - ref_out).max() <= 1e-5 * np.abs(ref_out).max()
    ref = np.array([fd_grad(oracle, case, par, dims, kernel, dims, raw, target, p, "hsml")
                    for p in range(0, n, 20)])
    got = grads["hsml"][0:n:20]
    assert np.all(np.abs(got - ref) <= 1e-4 * np.maximum(np.abs(ref), 1e-3 * np.abs(ref).max()))
