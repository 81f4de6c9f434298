"""``distributed_cic_map`` (distributed_mapping/cic.jl:24-110): sub-file maps
summed over their finite entries, across ranks by one all-reduce, then
reduced.  CPU tests run the host logic (one process, and two ``gloo`` ranks);
the GPU test sums device maps with ``sphg_accumulate`` and reduces with
``sphg_reduce``."""
import os
import socket
import tempfile

import numpy as np
import pytest

import dist_worker as DW

NSUB = 6


def _expected(oracle, dims, P):
    case, cuts = DW.subfile_case(dims, NSUB)
    total = None
    for sub in range(NSUB):
        maps, wmap = DW.subfile_map(oracle, case, cuts, sub, dims, P)
        if maps is None:
            continue
        raw = np.concatenate([maps, wmap[:, None]], axis=1)
        raw = np.where(np.isfinite(raw), raw, 0.0)
        total = raw if total is None else total + raw
    import torch
    return DW.host_reduce(dims, P)(torch.from_numpy(total)), case, cuts


@pytest.mark.parametrize("dims,P", [(2, 20), (3, 10)])
def test_single_process_host(pkg, oracle, dims, P):
    ref, case, cuts = _expected(oracle, dims, P)
    nimg = 2 if dims == 2 else 1
    par = pkg.mappingParameters(center=[0.0, 0.0, 0.0], x_size=1.0, y_size=1.0, z_size=1.0,
                                Npixels=P)
    img = pkg.distributed_cic_map(NSUB, lambda s: DW.subfile_map(oracle, case, cuts, s, dims, P),
                                  par, nimg, Ndim=dims, accumulate=DW.host_accumulate,
                                  reduce=DW.host_reduce(dims, P))
    assert np.isfinite(img).all()
    np.testing.assert_allclose(img, ref, rtol=1e-13, atol=0)


def test_bad_shape_and_ndim(pkg, oracle):
    par = pkg.mappingParameters(center=[0.0, 0.0, 0.0], x_size=1.0, y_size=1.0, z_size=1.0,
                                Npixels=8)
    with pytest.raises(ValueError):
        pkg.distributed_cic_map(1, lambda s: None, par, Ndim=4, accumulate=DW.host_accumulate,
                                reduce=DW.host_reduce(2, 8))
    with pytest.raises(ValueError):
        pkg.distributed_cic_map(1, lambda s: (np.zeros((10, 1)), np.zeros(10)), par,
                                accumulate=DW.host_accumulate, reduce=DW.host_reduce(2, 8))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


@pytest.mark.parametrize("dims,P", [(2, 20), (3, 10)])
def test_two_ranks_gloo(pkg, oracle, dims, P):
    import torch.multiprocessing as mp
    ref, _, _ = _expected(oracle, dims, P)
    with tempfile.TemporaryDirectory() as tmp:
        mp.spawn(DW.run, args=(2, _free_port(), tmp, dims, P, NSUB), nprocs=2, join=True)
        res = [dict(np.load(os.path.join(tmp, f"rank{r}.npz"))) for r in range(2)]
    # round-robin sub-files, every rank ends with the same reduced image
    assert list(res[0]["seen"]) == [0, 2, 4] and list(res[1]["seen"]) == [1, 3, 5]
    assert np.array_equal(res[0]["image"], res[1]["image"])
    np.testing.assert_allclose(res[0]["image"], ref, rtol=1e-13, atol=0)


@pytest.mark.gpu
def test_gpu_accumulate_reduce(gpu, oracle):
    """Device sub-file maps (sphMapping with return_both_maps on CUDA
    tensors) summed by sphg_accumulate and reduced by sphg_reduce."""
    import torch
    dims, P = 2, 24
    ref, case, cuts = _expected(oracle, dims, P)
    pos, hsml, m, rho, q, w = case
    par = gpu.mappingParameters(center=[0.0, 0.0, 0.0], x_size=1.0, y_size=1.0, z_size=1.0,
                                Npixels=P)
    dev = torch.device("cuda", 0)

    def mapping_function(sub):
        if sub == 4:
            return None
        s = slice(cuts[sub], cuts[sub + 1])
        t = lambda a: torch.as_tensor(np.ascontiguousarray(a), device=dev)
        raw = gpu.sphMapping(t(pos[:, s]), t(hsml[s]), t(m[s]), t(rho[s]), t(q[:, s]), t(w[s]),
                             param=par, kernel=gpu.Cubic(2), return_both_maps=True,
                             show_progress=False, center_in_place=False).clone()
        if sub == 3:  # planted non-finite entries are skipped
            raw[5, 0] = float("nan")
            raw[7, -1] = float("inf")
            raw[11, :] = float("-inf")
        return raw

    img = gpu.distributed_cic_map(NSUB, mapping_function, par, 2, Ndim=dims)
    torch.cuda.synchronize()
    assert img.is_cuda and tuple(img.shape) == (P, P, 2)
    got = img.cpu().numpy()
    assert np.isfinite(got).all()
    np.testing.assert_allclose(got, ref, rtol=1e-11, atol=1e-300)
