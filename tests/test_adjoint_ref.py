"""The two gradient references agree: forward-mode dual numbers through the
Python restatement against FP64 central differences through the C oracle."""
import numpy as np
import pytest

from adjoint_ref import PARAMS, dual_grad, fd_grad, reduce_rows


def _small_case(seed, n, dims, nq=1):
    rng = np.random.default_rng(seed)
    pos = np.asfortranarray(rng.uniform(-0.45, 0.45, (3, n)))
    hsml = np.exp(rng.uniform(np.log(0.08), np.log(0.25), n))
    m = rng.uniform(0.5, 1.5, n) / n
    rho = rng.uniform(0.5, 2.0, n)
    q = rng.uniform(0.5, 2.0, (nq, n)) if nq > 1 else rng.uniform(0.5, 2.0, n)
    w = rng.uniform(0.5, 2.0, n)
    return pos, hsml, m, rho, q, w


@pytest.mark.parametrize("dims,kernel,nq", [(2, "cubic", 1), (2, "wendlandc4", 2),
                                            (3, "wendlandc6", 1)])
def test_dual_numbers_match_finite_differences(oracle, pyoracle, dims, kernel, nq):
    n, P = (25, 12) if dims == 2 else (8, 8)
    case = _small_case(dims + nq, n, dims, nq)
    par = oracle.mapping_parameters(center=[0.0, 0.0, 0.0], x_size=1.0, y_size=1.0, z_size=1.0,
                                    Npixels=P)
    raw, _ = oracle.sph_mapping(*case, param=par, kernel=kernel, dimensions=dims,
                                return_both_maps=True, raw3d=True)
    rng = np.random.default_rng(7)
    out = reduce_rows(raw, dims)
    target = out * rng.lognormal(0.0, 0.1, out.shape)
    for p in (0, n // 2):
        for name in PARAMS:
            if dims == 2 and name == "z":
                continue
            fd = fd_grad(oracle, case, par, dims, kernel, dims, raw, target, p, name)
            du = dual_grad(pyoracle, case, par, dims, kernel, dims, target, p, name)
            assert abs(fd - du) <= 1e-6 * max(abs(du), 1e-12) + 1e-9 * abs(out).max() ** 2, \
                (p, name, fd, du)
