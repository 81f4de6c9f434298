"""Batched maps (one persistent deposit over all maps' tiles, CUDA graph,
autotuner) against the single-map path and the oracle."""
import numpy as np
import pytest

from conftest import rel_linf

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _maps(seed):
    rng = np.random.default_rng(seed)
    out = []
    for i, (n, P, nq, kern, dims) in enumerate([(3000, 48, 1, "quintic", 2), (12000, 64, 3, "wendlandc4", 2),
                                                (500, 32, 2, "cubic", 2), (20000, 40, 4, "wendlandc4", 2),
                                                (900, 24, 1, "wendlandc6", 3), (1, 16, 1, "cubic", 2),
                                                (6000, 37, 2, "quintic", 2)]):
        pos = np.asfortranarray(rng.random((3, n)).astype(np.float32))
        hsml = np.clip(np.exp(np.log(0.02) + 0.6 * rng.standard_normal(n)), 0.002, 0.3).astype(np.float32)
        rho = rng.uniform(0.5, 2.0, n).astype(np.float32)
        q = (rng.uniform(0.5, 2.0, (nq, n)) if nq > 1 else rng.uniform(0.5, 2.0, n)).astype(np.float32)
        out.append(dict(pos=pos, hsml=hsml, m=np.full(n, 1.0 / n, np.float32), rho=rho, q=q, w=rho.copy(),
                        P=P, kernel=kern, dims=dims))
    return out


def _dev(a):
    return torch.tensor(np.ascontiguousarray(a), device="cuda")


def _specs(gpu, maps):
    from sphtogrid_gb300.batch import MapSpec
    specs, host = [], []
    for d in maps:
        par = gpu.mappingParameters(x_lim=[0, 1], y_lim=[0, 1], z_lim=[0, 1], Npixels=d["P"])
        tpos = _dev(d["pos"].T).T
        ts = [_dev(d[k]) for k in ("hsml", "m", "rho", "q", "w")]
        specs.append(MapSpec(tpos, *ts, param=par, kernel=gpu.kernel_from_name(d["kernel"], d["dims"]),
                             dimensions=d["dims"]))
        host.append((par, tpos, ts))
    return specs, host


def _single(gpu, d, par, deterministic=False):
    return gpu.sphMapping(d["pos"].copy(order="F"), d["hsml"], d["m"], d["rho"], d["q"], d["w"],
                          param=par, kernel=gpu.kernel_from_name(d["kernel"], d["dims"]),
                          dimensions=d["dims"], precision="fp32c", deterministic=deterministic,
                          show_progress=False)


def test_batch_matches_single_maps(gpu, oracle):
    from sphtogrid_gb300.batch import SPHBatch
    maps = _maps(1)
    specs, host = _specs(gpu, maps)
    b = SPHBatch(specs)  # autotuned
    tun = b.tuning
    assert (tun["tile_x"], tun["tile_y"]) in ((16, 16), (32, 16), (32, 32))
    assert tun["ctas_per_sm"] >= 1 and tun["tuned_ms"] > 0
    b.launch()
    stats = b.wait()
    for i, d in enumerate(maps):
        got = b.image(i).cpu().numpy()
        ref = _single(gpu, d, host[i][0])
        assert got.shape == ref.shape
        assert rel_linf(got, ref, 1e-9) <= 1e-6, i
        opar = oracle.mapping_parameters(x_lim=[0, 1], y_lim=[0, 1], z_lim=[0, 1], Npixels=d["P"])
        oref, info = oracle.sph_mapping(d["pos"].copy(order="F"), d["hsml"], d["m"], d["rho"], d["q"],
                                        d["w"], param=opar, kernel=d["kernel"], dimensions=d["dims"])
        assert stats[i]["deposits"] == info["deposits"]
        assert stats[i]["n_launches"] == 6
        # the batched map itself against the oracle, on the pixels carrying
        # weight (W >= 1e-6 max W), relative to each pixel's value (q > 0)
        raw, _ = oracle.sph_mapping(d["pos"].copy(order="F"), d["hsml"], d["m"], d["rho"], d["q"], d["w"],
                                    param=opar, kernel=d["kernel"], dimensions=d["dims"],
                                    return_both_maps=True, raw3d=True)
        P = d["P"]
        W = raw[:, -1]
        keep = W >= 1e-6 * W.max() if W.max() > 0 else np.zeros_like(W, bool)
        keep = keep.reshape(P, P, 1) if d["dims"] == 2 else keep.reshape(P, P, P).transpose(2, 1, 0)
        keep = np.broadcast_to(keep, got.shape)
        oref = np.asarray(oref).reshape(got.shape)
        if keep.any():
            assert (np.abs(got - oref)[keep] / np.abs(oref)[keep]).max() <= 1e-5, i
    b.close()


def test_batch_deterministic_is_bitwise_single(gpu):
    """Deterministic sums are exact int64 with a per-tile scale: with the
    single-map tile shape (16 x 16) the batch reproduces the single-map
    result bit for bit; another tile shape changes only the scale's rounding
    quantum (far below 1e-12 relative here)."""
    from sphtogrid_gb300.batch import SPHBatch
    maps = _maps(2)
    specs, host = _specs(gpu, maps)
    refs = [_single(gpu, d, host[i][0], deterministic=True) for i, d in enumerate(maps)]
    b = SPHBatch(specs, deterministic=True, tuning=(16, 16, 4, 8192))
    b.launch()
    b.wait()
    for i in range(len(maps)):
        assert np.array_equal(b.image(i).cpu().numpy(), refs[i]), i
    b.close()
    b = SPHBatch(specs, deterministic=True, tuning=(32, 16, 4, 8192))
    b.launch()
    b.wait()
    for i in range(len(maps)):
        got = b.image(i).cpu().numpy()
        assert np.allclose(got, refs[i], rtol=1e-12, atol=1e-12 * np.abs(refs[i]).max()), i
    b.close()


def test_batch_relaunch_sees_new_inputs(gpu):
    from sphtogrid_gb300.batch import SPHBatch
    maps = _maps(3)[:4]
    specs, host = _specs(gpu, maps)
    b = SPHBatch(specs, tuning=(16, 16, 4, 8192))
    b.launch()
    b.wait()
    first = [b.image(i).clone() for i in range(len(maps))]
    for par, tpos, ts in host:
        ts[3].mul_(2.0)  # Bin_Quant doubled in place: Q/W doubles
    torch.cuda.synchronize()
    for _ in range(3):
        b.launch()
    b.wait()
    for i in range(len(maps)):
        got = b.image(i)
        assert torch.allclose(got, 2.0 * first[i], rtol=1e-6, atol=1e-12 * float(first[i].abs().max()))
    b.close()


def _dense_maps(seed):
    """Maps with many particles on few pixels: their tiles hold tens of
    thousands of pairs each and are split over several CTAs (2D and 3D,
    reduced and raw outputs), next to an ordinary map.  With 16 x 16 tiles
    (8^3 in 3D) and 4096 expected pairs per chunk the first three maps take
    14, 5 and 6 chunks per tile, the last one."""
    rng = np.random.default_rng(seed)
    out = []
    for n, P, nq, kern, dims, raw in [(150000, 32, 2, "wendlandc4", 2, False), (120000, 48, 1, "quintic", 2, True),
                                      (60000, 16, 1, "wendlandc6", 3, False), (4000, 64, 3, "cubic", 2, False)]:
        pos = np.asfortranarray(rng.random((3, n)).astype(np.float32))
        hsml = np.clip(np.exp(np.log(0.03) + 0.5 * rng.standard_normal(n)), 0.005, 0.2).astype(np.float32)
        rho = rng.uniform(0.5, 2.0, n).astype(np.float32)
        q = (rng.uniform(0.5, 2.0, (nq, n)) if nq > 1 else rng.uniform(0.5, 2.0, n)).astype(np.float32)
        out.append(dict(pos=pos, hsml=hsml, m=np.full(n, 1.0 / n, np.float32), rho=rho, q=q, w=rho.copy(),
                        P=P, kernel=kern, dims=dims, raw=raw))
    return out


def _dense_specs(gpu, maps):
    from sphtogrid_gb300.batch import MapSpec
    specs, pars = [], []
    for d in maps:
        par = gpu.mappingParameters(x_lim=[0, 1], y_lim=[0, 1], z_lim=[0, 1], Npixels=d["P"])
        tpos = _dev(d["pos"].T).T
        ts = [_dev(d[k]) for k in ("hsml", "m", "rho", "q", "w")]
        specs.append(MapSpec(tpos, *ts, param=par, kernel=gpu.kernel_from_name(d["kernel"], d["dims"]),
                             dimensions=d["dims"], return_both_maps=d["raw"]))
        pars.append(par)
    return specs, pars


def _dense_single(gpu, d, par, deterministic):
    return gpu.sphMapping(d["pos"].copy(order="F"), d["hsml"], d["m"], d["rho"], d["q"], d["w"],
                          param=par, kernel=gpu.kernel_from_name(d["kernel"], d["dims"]),
                          dimensions=d["dims"], precision="fp32c", deterministic=deterministic,
                          return_both_maps=d["raw"], show_progress=False)


@pytest.mark.parametrize("deterministic", [False, True])
def test_batch_split_tiles(gpu, oracle, deterministic):
    """Split tiles (each chunk's partial sums added to the map's raw sums,
    the last chunk writing the output) against the single-map path, where
    one CTA takes each tile: deterministic sums are exact int64 at the same
    per-tile scale, so with the same tile shape they agree bit for bit."""
    from sphtogrid_gb300.batch import SPHBatch
    maps = _dense_maps(7)
    specs, pars = _dense_specs(gpu, maps)
    b = SPHBatch(specs, deterministic=deterministic, tuning=(16, 16, 4, 8192))
    b.launch()
    stats = b.wait()
    for _ in range(2):  # graph replays start from zeroed partial sums
        b.launch()
    b.wait()
    for i, d in enumerate(maps):
        got = b.image(i).cpu().numpy()
        ref = _dense_single(gpu, d, pars[i], deterministic)
        assert got.shape == ref.shape, i
        if deterministic:
            assert np.array_equal(got, ref), i
        else:
            assert rel_linf(got, ref, 1e-9) <= 1e-6, i
        opar = oracle.mapping_parameters(x_lim=[0, 1], y_lim=[0, 1], z_lim=[0, 1], Npixels=d["P"])
        _, info = oracle.sph_mapping(d["pos"].copy(order="F"), d["hsml"], d["m"], d["rho"], d["q"],
                                     d["w"], param=opar, kernel=d["kernel"], dimensions=d["dims"])
        assert stats[i]["deposits"] == info["deposits"], i
    b.close()
