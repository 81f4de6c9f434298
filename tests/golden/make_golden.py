"""Generates the golden fixtures of tests/golden/ (run from the repository
root: `python tests/golden/make_golden.py`).

Each fixture holds seeded inputs and the FP64 oracle's output, plus the raw
map of |q| (`raw_absq`): the magnitude each pixel sums, against which the
FP32-compensated path's error is judged where quantities of both signs cancel.  Generation
asserts that the independent pure-Python restatement reproduces every raw
accumulator bit for bit, so a fixture pins both restatements; the two known-
answer cases restate the reference's self-contained tests
(test/runtests.jl:324-342 and :718-738).  The reference itself (Julia) cannot
run here, so kernel-shape values in these fixtures are the restatement's.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import oracle as O  # noqa: E402
import pyoracle as PO  # noqa: E402

KERNELS = ["cubic", "quintic", "wendlandc4", "wendlandc6", "wendlandc8"]


def case(seed, n, nq, dtype):
    rng = np.random.default_rng(seed)
    pos = np.asfortranarray(rng.uniform(-0.55, 0.55, (3, n)))
    hsml = np.exp(rng.uniform(np.log(0.01), np.log(0.3), n))
    m = rng.uniform(0.5, 1.5, n) / n
    rho = rng.uniform(0.5, 2.0, n)
    q = rng.uniform(-0.5, 2.0, (nq, n)) if nq > 1 else rng.uniform(0.5, 2.0, n)
    w = rng.uniform(0.5, 2.0, n)
    c = lambda a: np.asarray(a, dtype=dtype)
    return np.asfortranarray(c(pos)), c(hsml), c(m), c(rho), c(q), c(w)


def check_python(dims, P, kernel, pos, hsml, m, rho, q, w, raw):
    par = O.mapping_parameters(center=[0.0, 0.0, 0.0], x_size=1.0, y_size=1.0, z_size=1.0, Npixels=P)
    mask = O.filter_particles_in_image(pos, par)
    idx = np.nonzero(mask)[0]
    qq = q.reshape(-1, pos.shape[1])
    nq = qq.shape[0]
    chans, _ = PO.cic_map(dims, [tuple(pos[:, i]) for i in idx], hsml[idx], m[idx], rho[idx],
                          [tuple(qq[:, i]) for i in idx], w[idx], par.len2pix, P, kernel)
    for ch in range(nq + 1):
        dense = np.zeros(P ** dims)
        for k, v in chans[ch].items():
            dense[k] = v
        assert np.array_equal(dense, raw[:, ch]), (dims, kernel, ch)


def main():
    out = {}
    for i, kernel in enumerate(KERNELS):
        pos, hsml, m, rho, q, w = case(100 + i, 160, 2, np.float64)
        P = 24
        par = O.mapping_parameters(center=[0.0, 0.0, 0.0], x_size=1.0, y_size=1.0, z_size=1.0,
                                   Npixels=P)
        raw, info = O.sph_mapping(pos, hsml, m, rho, q, w, param=par, kernel=kernel,
                                  return_both_maps=True)
        check_python(2, P, kernel, pos, hsml, m, rho, q, w, raw)
        red, _ = O.sph_mapping(pos, hsml, m, rho, q, w, param=par, kernel=kernel)
        absq, _ = O.sph_mapping(pos, hsml, m, rho, np.abs(q), w, param=par, kernel=kernel,
                                return_both_maps=True)
        out[f"map2d_{kernel}"] = dict(pos=pos, hsml=hsml, m=m, rho=rho, q=q, w=w, P=P, raw=raw,
                                      reduced=red, deposits=info["deposits"], raw_absq=absq)
    for kernel in ("cubic", "wendlandc6"):
        pos, hsml, m, rho, q, w = case(200, 60, 1, np.float32)
        P = 12
        par = O.mapping_parameters(center=[0.0, 0.0, 0.0], x_size=1.0, y_size=1.0, z_size=1.0,
                                   Npixels=P)
        raw, info = O.sph_mapping(pos, hsml, m, rho, q, w, param=par, kernel=kernel, dimensions=3,
                                  raw3d=True)
        check_python(3, P, kernel, pos.astype(np.float64), hsml, m, rho, q, w, raw)
        red, _ = O.sph_mapping(pos, hsml, m, rho, q, w, param=par, kernel=kernel, dimensions=3)
        absq, _ = O.sph_mapping(pos, hsml, m, rho, np.abs(q), w, param=par, kernel=kernel,
                                dimensions=3, raw3d=True)
        out[f"map3d_{kernel}"] = dict(pos=pos, hsml=hsml, m=m, rho=rho, q=q, w=w, P=P, raw=raw,
                                      reduced=red, deposits=info["deposits"], raw_absq=absq)
    # runtests.jl:718-738: particle not overlapping pixel centres (fallback branch)
    par = O.mapping_parameters(x_lim=[-10, 10], y_lim=[-10, 10], z_lim=[-10, 10], Npixels=4)
    one = np.ones(1)
    red, _ = O.sph_mapping(np.array([[0.5], [0.0], [0.0]]), one, one, one, one,
                           one * par.pixelSideLength, param=par, kernel="cubic", kernel_dim=3,
                           reduce_image=False)
    out["kat_fallback_2d"] = dict(image=red)
    # runtests.jl:324-342: 3D mass conservation, single particle (nonzeros only)
    par = O.mapping_parameters(x_lim=[-64, 64], y_lim=[-64, 64], z_lim=[-64, 64], Npixels=200)
    img, _ = O.sph_mapping(np.array([[0.0101], [-0.001], [0.001]]), np.array([5.0]),
                           np.array([3.0]), one, one, one * par.pixelSideLength, param=par,
                           kernel="cubic", dimensions=3, reduce_image=False)
    flat = img.reshape(-1, order="F")
    nz = np.nonzero(flat)[0]
    out["kat_mass_3d"] = dict(index=nz, value=flat[nz])
    for name, d in out.items():
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **d)
    print("wrote", len(out), "fixtures")


if __name__ == "__main__":
    main()
