"""Rank body of the world-size-2 ``distributed_cic_map`` test: each rank maps
its sub-files with the oracle, sums them with a host
accumulator and reduces on the host, so the test exercises the sub-file
assignment and the cross-rank all-reduce without a GPU."""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def subfile_case(dims, nsub, seed=7, n=600, nq=2):
    rng = np.random.default_rng(seed)
    pos = np.asfortranarray(rng.uniform(-0.5, 0.5, (3, n)))
    hsml = np.exp(rng.uniform(np.log(0.02), np.log(0.2), n))
    m = rng.uniform(0.5, 1.5, n) / n
    rho = rng.uniform(0.5, 2.0, n)
    q = rng.uniform(0.1, 2.0, (nq, n)) if dims == 2 else rng.uniform(0.1, 2.0, n)
    w = rng.uniform(0.5, 2.0, n)
    cuts = np.linspace(0, n, nsub + 1).astype(int)
    return (pos, hsml, m, rho, q, w), cuts


def subfile_map(oracle, case, cuts, sub, dims, P, kernel="cubic", bad=(3,)):
    """Raw (P^D, Nq+1) map of sub-file `sub`; sub-files in `bad` get NaN and
    Inf entries planted (the reference skips them when summing); sub-file 4
    returns None (nothing to add)."""
    if sub == 4:
        return (None, None)
    pos, hsml, m, rho, q, w = case
    s = slice(cuts[sub], cuts[sub + 1])
    qq = q[:, s] if q.ndim == 2 else q[s]
    par = oracle.mapping_parameters(center=[0.0, 0.0, 0.0], x_size=1.0, y_size=1.0, z_size=1.0,
                                    Npixels=P)
    raw, _ = oracle.sph_mapping(np.asfortranarray(pos[:, s]), hsml[s], m[s], rho[s], qq, w[s],
                                param=par, kernel=kernel, dimensions=dims,
                                return_both_maps=True, raw3d=True)
    raw = raw.copy()
    if sub in bad:
        raw[5, 0] = np.nan
        raw[7, -1] = np.inf
        raw[11, :] = -np.inf
    return raw[:, :-1], raw[:, -1]


def host_accumulate(total, part):
    import torch
    total += torch.where(torch.isfinite(part), part, torch.zeros_like(part))


def host_reduce(dims, P, reduce_image=True):
    def red(total):
        raw = total.numpy()
        Q, W = raw[:, :-1], raw[:, -1:]
        if dims == 2:
            out = np.where((W > 0) & reduce_image, Q / np.where(W > 0, W, 1.0), Q)
            return out.reshape(P, P, -1)
        out = np.where(Q > 0, Q / np.where(Q > 0, W, 1.0), Q)
        return out[:, 0].reshape(P, P, P).transpose(2, 1, 0)
    return red


def run(rank, world, port, outdir, dims, P, nsub):
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import torch.distributed as dist

    import __graft_entry__ as graft
    import oracle as O
    pkg = graft.load_package()
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank,
                            world_size=world)
    try:
        case, cuts = subfile_case(dims, nsub)
        nimg = case[4].shape[0] if case[4].ndim == 2 else 1
        par = pkg.mappingParameters(center=[0.0, 0.0, 0.0], x_size=1.0, y_size=1.0, z_size=1.0,
                                    Npixels=P)
        seen = []

        def mapping_function(sub):
            seen.append(sub)
            return subfile_map(O, case, cuts, sub, dims, P)

        img = pkg.distributed_cic_map(nsub, mapping_function, par, nimg, Ndim=dims,
                                      accumulate=host_accumulate, reduce=host_reduce(dims, P))
        np.savez(os.path.join(outdir, f"rank{rank}.npz"), image=np.asarray(img),
                 seen=np.array(seen))
    finally:
        dist.destroy_process_group()
