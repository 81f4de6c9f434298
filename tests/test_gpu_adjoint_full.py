"""The differentiable-deposition workload at full size: N = 2^20 particles
(positions uniform in the unit cube, hsml lognormal median 0.01 sigma 0.5
clipped to [0.002, 0.1], rho in [0.5, 2], Bin_Quant = Weights = rho)
projected to 512^2 with WendlandC4; loss L = sum((map - target)^2) with the
target the map of a perturbed copy (positions jittered by 0.1 hsml,
quantity scaled lognormal sigma 0.1).  Gradients with respect to Bin_Quant,
M, Rho, HSML and Pos from the hand-written adjoint against FP64 central
differences of the oracle on 256 random particles."""
import numpy as np
import pytest

from adjoint_ref import fd_grad, reduce_rows, rows_to_output

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.mark.parametrize("precision,adjoint", [("fp64", "fp64"), ("fp64", "fp32c")])
def test_adjoint_full_size(gpu, oracle, precision, adjoint):
    from sphtogrid_gb300 import synth
    d = synth.differentiable_2d(N=2 ** 20, npix=512)
    n, P = d["pos"].shape[1], 512
    rng = np.random.default_rng(4)
    pos = np.asfortranarray(d["pos"].astype(np.float64) - 0.5)  # the unit cube centred at 0
    case = (pos, d["hsml"].astype(np.float64), d["mass"].astype(np.float64),
            d["rho"].astype(np.float64), d["bin_q"].astype(np.float64).copy(),
            d["weights"].astype(np.float64))
    par = oracle.mapping_parameters(center=[0.0, 0.0, 0.0], x_size=1.0, y_size=1.0, z_size=1.0,
                                    Npixels=P)
    raw, _ = oracle.sph_mapping(*case, param=par, kernel="wendlandc4", kernel_dim=2,
                                return_both_maps=True, copy_pos=True)
    # target: the map of a perturbed copy
    jit = case[0] + 0.1 * case[1] * rng.standard_normal((3, n))
    qj = case[4] * rng.lognormal(0.0, 0.1, n)
    traw, _ = oracle.sph_mapping(np.asfortranarray(jit), case[1], case[2], case[3], qj, case[5],
                                 param=par, kernel="wendlandc4", kernel_dim=2, return_both_maps=True)
    target = reduce_rows(traw, 2)
    gpar = gpu.mappingParameters(center=[0.0, 0.0, 0.0], x_size=1.0, y_size=1.0, z_size=1.0,
                                 Npixels=P)
    dev = "cuda"
    tpos = torch.tensor(np.ascontiguousarray(case[0].T), device=dev).T.requires_grad_(True)
    ts = [torch.tensor(np.ascontiguousarray(a), device=dev, requires_grad=True) for a in case[1:]]
    out = gpu.sph_map_differentiable(tpos, ts[0], ts[1], ts[2], ts[3], ts[4], param=gpar,
                                     kernel=gpu.WendlandC4(2), dimensions=2, precision=precision,
                                     adjoint_precision=adjoint)
    t = torch.tensor(rows_to_output(target, 2, P), device=dev)
    loss = ((out.permute(2, 1, 0).reshape(-1) - t) ** 2).sum()
    loss.backward()
    grads = {"x": tpos.grad[0], "y": tpos.grad[1], "hsml": ts[0].grad, "mass": ts[1].grad,
             "rho": ts[2].grad, "q": ts[3].grad, "weights": ts[4].grad}
    grads = {k: v.detach().cpu().numpy() for k, v in grads.items()}
    # the forward is the oracle's map (FP32C: within its 1e-5)
    got_out = out.detach().permute(2, 1, 0).reshape(-1).cpu().numpy()
    ref_out = rows_to_output(reduce_rows(raw, 2), 2, P)
    if precision == "fp64":
        assert np.allclose(got_out, ref_out, rtol=1e-10, atol=1e-12 * np.abs(raw[:, 0]).max())
    else:
        assert np.abs(got_out - ref_out).max() <= 1e-5 * np.abs(ref_out).max()
    parts = rng.choice(n, size=256, replace=False)
    for name in ("x", "y", "hsml", "mass", "rho", "weights", "q"):
        ref = np.array([fd_grad(oracle, case, par, 2, "wendlandc4", 2, raw, target, int(p), name)
                        for p in parts])
        got = grads[name][parts]
        scale = np.abs(ref).max()
        tol = 1e-4 * np.maximum(np.abs(ref), 1e-3 * scale) + 1e-300
        bad = np.abs(got - ref) > tol
        assert not bad.any(), (name, parts[bad][:5], got[bad][:5], ref[bad][:5])
