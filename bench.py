#!/usr/bin/env python
"""Benchmark of the sphMapping deposition on one GB300.

Workload (default): the 3D gridded deposition -- N = 2^22 Float32 particles
drawn as 64 Gaussian clumps plus a 20% uniform background in the unit cube,
hsml from the local density, Bin_Quant = lognormal temperature, WendlandC6,
256^3 grid, reduce_image = true.  A step is one ``sphg_map`` call over that
map; ``value`` is particle-pixel deposits per second with the inputs already
resident in HBM, ``e2e`` the same through the C ABI with pinned host buffers
(host->device copies of the inputs and device->host copy of the map inside
the timed region).

``--impl reference`` times the CPU restatement of the reference's FP64
algorithm (the oracle, all host threads, the reference's parallel=true
decomposition) on the same workload and metric.

With torchrun (N > 1) every rank maps its own copy of the workload on its own
GPU (replicas: the path has no exchange step); rank 0 prints the line.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = ("particle-pixel deposits/s & maps/s: batched FP32-comp vs plain FP64 on GB300 "
          "at ≤1e-5 rel err")
WORKLOAD = ("3D gridded deposition: N=2^22 Float32 particles, 64 Gaussian clumps (sigma "
            "0.02-0.08) + 20% uniform background, hsml from local density, Bin_Quant = "
            "lognormal temperature, WendlandC6, 256^3 grid, reduce_image=true, seed 0")


def _env_int(k, d):
    try:
        return int(os.environ.get(k, d))
    except ValueError:
        return d


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.thread.join(timeout=5)

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                mx = float(parts[1])
            except ValueError:
                continue
            for nm, v in zip(names, parts[3:7]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


def load_workload(dtype=np.float32):
    import __graft_entry__ as graft
    pkg = graft.load_package()
    from sphtogrid_gb300 import synth
    return pkg, synth.clumps_3d(dtype=dtype)


def oracle_module():
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle  # test infrastructure: only the CPU-baseline leg runs it
    oracle.build()
    return oracle


def run_oracle(O, d, frac=1.0, threads=None):
    """One oracle map of (a contiguous fraction of) the workload; returns
    (seconds, deposits, image)."""
    n = d["pos"].shape[1]
    m = max(1, int(round(n * frac)))
    par = O.mapping_parameters(x_lim=[0, 1], y_lim=[0, 1], z_lim=[0, 1], Npixels=d["npix"])
    threads = threads or os.cpu_count()
    sl = slice(0, m)
    # a fresh copy per call: the mapping centres its positions in place, as
    # the reference's does (copied outside the timed region)
    pos = np.array(d["pos"][:, sl], order="F", copy=True)
    t0 = time.perf_counter()
    img, info = O.sph_mapping(pos, d["hsml"][sl], d["mass"][sl], d["rho"][sl], d["bin_q"][sl],
                              d["weights"][sl], param=par, kernel=d["kernel"], dimensions=3,
                              nthreads=threads, copy_pos=False)
    dt = time.perf_counter() - t0
    return dt, info["deposits"], img, threads, m


def bench_reference(args):
    """CPU restatement of the reference (the oracle) on the host cores."""
    rank = _env_int("RANK", 0)
    if rank != 0:
        return 0
    O = oracle_module()
    _, d = load_workload()
    # size each step to keep the whole run within a few minutes
    t_est, _, _, threads, _ = run_oracle(O, d, frac=1.0 / 16)
    per_step_budget = 150.0 / max(1, args.steps + args.warmup)
    frac = min(1.0, per_step_budget / max(1e-3, 16 * t_est))
    for _ in range(args.warmup):
        run_oracle(O, d, frac=frac)
    times, deps = [], 0
    for _ in range(args.steps):
        dt, dep, _, threads, m = run_oracle(O, d, frac=frac)
        times.append(dt)
        deps = dep
    tot = sum(times)
    value = deps * len(times) / tot
    sample = (f"{m} of {d['pos'].shape[1]} particles (first {frac:.3f} of the shuffled set) "
              f"mapped onto the full 256^3 grid per step")
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "deposits/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * tot / len(times), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": WORKLOAD, "parallelism": f"cpu threads={threads}",
                   "deposits_per_step": deps},
        "cpu_baseline": {"value": value, "unit": "deposits/s", "cores": threads, "kind": "port",
                         "sample": sample},
        "e2e": {"value": value, "unit": "deposits/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def _particles_struct(_lib, arrs, n, pos_dtype, attr_dtype, nq=1):
    pt = _lib.SphgParticles()
    pt.n = n
    pt.pos_dtype = pos_dtype
    pt.attr_dtype = attr_dtype
    pt.pos, pt.hsml, pt.mass, pt.rho, pt.weights, pt.bin_q = arrs
    pt.pos_stride_p, pt.pos_stride_c = 3, 1
    pt.n_q = nq
    pt.q_stride_p, pt.q_stride_k = 1, 0
    return pt


def bench_gpu(args):
    import torch

    rank, world = _env_int("RANK", 0), _env_int("WORLD_SIZE", 1)
    local = _env_int("LOCAL_RANK", 0)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if args.workload == "differentiable":
        import __graft_entry__ as graft
        out = bench_differentiable(graft.load_package(), dev, args.steps, args.warmup)
        if rank == 0:
            print(json.dumps(out), flush=True)
        return 0
    if args.workload == "projection_2d":
        import __graft_entry__ as graft
        out = bench_config1(graft.load_package(), dev, args.steps, args.warmup)
        if rank == 0:
            print(json.dumps(out), flush=True)
        return 0
    if args.workload == "healpix":
        import __graft_entry__ as graft
        out = bench_healpix(graft.load_package(), dev, args.steps, args.warmup, n=args.healpix_particles)
        if rank == 0:
            print(json.dumps(out), flush=True)
        return 0
    if args.workload == "large_hdr":
        import __graft_entry__ as graft
        out = bench_large(graft.load_package(), dev, args.steps, args.warmup, n=args.large_particles,
                          npix=args.large_npix, seed_grid=512 if args.large_particles >= 2 ** 25 else 128)
        if rank == 0:
            print(json.dumps(out), flush=True)
        return 0
    if args.batched_only:  # profiling runs: the batched workload alone
        import __graft_entry__ as graft
        tun = tuple(int(x) for x in args.batched_tuning.split(",")) if args.batched_tuning else None
        b = bench_batched(graft.load_package(), dev, args.steps, args.warmup, args.batched_maps,
                          args.deterministic, tun, with_oracle=False)
        if rank == 0:
            b.pop("rel_err_per_map")
            print(json.dumps(b), flush=True)
        return 0
    pkg, d = load_workload()
    from sphtogrid_gb300 import _lib
    L = _lib.lib()
    ctx = pkg.default_context(local)
    n = d["pos"].shape[1]
    P = d["npix"]
    par = pkg.mappingParameters(x_lim=[0, 1], y_lim=[0, 1], z_lim=[0, 1], Npixels=P)

    def opts(prec, mem, profile=1, det=None):
        o = _lib.SphgOptions()
        o.dimensions = 3
        o.kernel = pkg.WendlandC6(3).kind
        o.kernel_dim = 3
        o.reduce_image = 1
        o.precision = _lib.PREC[prec]
        o.center = _lib.CENTER_READONLY  # identical inputs every step
        o.filter = 1
        o.memspace = mem
        o.profile = profile
        o.deterministic = int((args.deterministic if det is None else det) and prec == "fp32c")
        return o

    # device-resident inputs (Julia layout: xyz contiguous per particle)
    t_pos = torch.from_numpy(np.ascontiguousarray(d["pos"].T)).to(dev)
    t_attr = [torch.from_numpy(np.ascontiguousarray(d[k])).to(dev)
              for k in ("hsml", "mass", "rho", "weights", "bin_q")]
    ptrs = [t_pos.data_ptr()] + [t.data_ptr() for t in t_attr]
    pt_dev = _particles_struct(_lib, ptrs, n, _lib.SPHG_F32, _lib.SPHG_F32)
    out_len = P ** 3
    t_out = torch.empty(out_len, dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream(dev)
    sh = _lib.stream_handle(stream)  # the events below bracket work on this stream

    def step(prec, st, pt=pt_dev, out=None, mem=_lib.MEM_DEVICE, profile=1, det=None):
        o = opts(prec, mem, profile, det)
        dst = C.c_void_p(t_out.data_ptr()) if out is None else out
        _lib.check(L.sphg_map(ctx.handle, C.byref(par._c), C.byref(o), C.byref(pt), dst, sh,
                              C.byref(st)), ctx.handle)

    def timed(prec, steps, warmup, det=None):
        st = _lib.SphgStats()
        for _ in range(warmup):
            step(prec, st, det=det)
        torch.cuda.synchronize(dev)
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize(dev)
        phases = np.zeros(4)
        launches = 0
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            step(prec, st, det=det)
            phases += np.array(list(st.phase_ms))
            launches += st.n_launches
        e1.record(stream)
        torch.cuda.synchronize(dev)
        ms = e0.elapsed_time(e1)
        if dist is not None:
            t = torch.tensor([ms], device=dev)
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            ms = float(t.item())
            dist.barrier()
        return ms, st, phases / steps, launches

    prec = args.precision
    with ClockSampler(local) as clk:
        ms, st, phases, launches = timed(prec, args.steps, args.warmup)
    deposits = st.deposits
    ms_step = ms / args.steps
    value = deposits * args.steps * world / (ms * 1e-3)
    if args.only_device:  # profiling runs: the timed device-resident loop alone
        if rank == 0:
            print(json.dumps({"metric": METRIC, "value": value, "unit": "deposits/s",
                              "ms_per_step": ms_step, "steps": args.steps, "warmup": args.warmup,
                              "phases_ms": [float(x) for x in phases], "gpu_launches": launches}),
                  flush=True)
        if dist is not None:
            dist.destroy_process_group()
        return 0

    # plain FP64 method on the same map (the speed-up denominator)
    ms64, st64, ph64, _ = timed("fp64", max(2, args.steps // 4), 1)
    img_fp64 = t_out.clone()
    step(prec, _lib.SphgStats())
    torch.cuda.synchronize(dev)
    img_main = t_out.clone()
    rel_vs_fp64 = _rel_linf(img_main.cpu().numpy(), img_fp64.cpu().numpy())
    other = None  # the other accumulation mode of the FP32C method, same map
    if prec == "fp32c":
        det2 = not args.deterministic
        ms2, _, ph2, _ = timed(prec, args.steps, args.warmup, det=det2)
        step(prec, _lib.SphgStats(), det=det2)
        torch.cuda.synchronize(dev)
        other = {"deterministic": det2, "ms_per_step": ms2 / args.steps,
                 "value": deposits * args.steps / (ms2 * 1e-3),
                 "phases_ms": {"prep": float(ph2[0]), "norm": float(ph2[1]),
                               "deposit": float(ph2[2]), "reduce": float(ph2[3])},
                 "rel_linf_vs_fp64": _rel_linf(t_out.cpu().numpy(), img_fp64.cpu().numpy())}
    batched = config1 = diff = None
    if rank == 0 and world == 1 and not args.no_batched:
        batched = bench_batched(pkg, dev, args.steps, args.warmup, with_oracle=not args.no_cpu_baseline)
    if rank == 0 and world == 1 and not args.no_sub_workloads:
        config1 = bench_config1(pkg, dev, args.steps, args.warmup)
        diff = bench_differentiable(pkg, dev, min(args.steps, 3), 1)

    # end to end through the C ABI with pinned host buffers
    h_pos = torch.from_numpy(np.ascontiguousarray(d["pos"].T)).pin_memory()
    h_attr = [torch.from_numpy(np.ascontiguousarray(d[k])).pin_memory()
              for k in ("hsml", "mass", "rho", "weights", "bin_q")]
    h_out = torch.empty(out_len, dtype=torch.float64).pin_memory()
    pt_host = _particles_struct(_lib, [h_pos.data_ptr()] + [t.data_ptr() for t in h_attr], n,
                                _lib.SPHG_F32, _lib.SPHG_F32)
    e2e_steps = max(3, args.steps // 2)
    ste = _lib.SphgStats()
    for _ in range(2):
        step(prec, ste, pt=pt_host, out=C.c_void_p(h_out.data_ptr()), mem=_lib.MEM_HOST, profile=0)
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        step(prec, ste, pt=pt_host, out=C.c_void_p(h_out.data_ptr()), mem=_lib.MEM_HOST, profile=0)
    e2e_s = (time.perf_counter() - t0) / e2e_steps
    h2d = h_pos.numel() * 4 + sum(t.numel() * t.element_size() for t in h_attr)
    d2h = out_len * 8

    # roofline of the dominant kernel (the tile deposit)
    peaks = _peaks()
    dep_ms = float(phases[2])
    n_rec = st.n_mapped
    dep_bytes = n_rec * (16 + 16 + 16 + 8 + 4) + out_len * 8
    achieved = dep_bytes / (dep_ms * 1e-3) / 1e9 if dep_ms > 0 else None
    traffic = _traffic_per_launch()

    line = {
        "metric": METRIC, "value": value, "unit": "deposits/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_step,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "fp32" if prec == "fp32c" else "f64", "data": "synthetic",
        "config": {"workload": WORKLOAD, "precision": prec, "deterministic": bool(args.deterministic),
                   "particles": n,
                   "deposits_per_step": deposits, "maps_per_s": 1e3 / ms_step,
                   "parallelism": "replicas" if world > 1 else "single GPU",
                   "l2": "working set (134 MB inputs + 60 B/particle records + 134 MB map) "
                         "larger than the 129 MB L2; no flush"},
        "phases_ms": {"prep": float(phases[0]), "norm": float(phases[1]),
                      "deposit": float(phases[2]), "reduce": float(phases[3])},
        "plain_fp64": {"ms_per_step": ms64 / max(2, args.steps // 4),
                       "deposits_per_s": deposits * max(2, args.steps // 4) / (ms64 * 1e-3),
                       "speedup_of_" + prec: (ms64 / max(2, args.steps // 4)) / ms_step,
                       "rel_linf_" + prec + "_vs_fp64": rel_vs_fp64},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peaks[0], "unit": "GB/s",
                     "frac": (achieved / peaks[0]) if achieved else None, "traffic": traffic,
                     "kernel": "k_deposit", "peak_source": peaks[1],
                     "algorithmic_bytes_per_launch": dep_bytes},
        "e2e": {"value": deposits / e2e_s, "unit": "deposits/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h, "ms_per_step": e2e_s * 1e3,
                "transfer": ("pinned host buffers read and written in place by the kernels over the "
                             "host link (no staging copies; host wall clock per call)")},
        "gpu_launches": launches,
        "clocks": clk.summary(),
    }
    if other is not None:
        line["fp32c_other_mode"] = other
    if rank == 0:
        line["onchip_ceiling"] = _onchip_ceiling(L, ctx, _lib, value, other, args.deterministic)
    if batched is not None:
        line["batched"] = batched
    if config1 is not None:
        line["projection_2d"] = config1
    if diff is not None:
        line["differentiable"] = diff
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        O = oracle_module()
        dt, dep, img_ref, threads, m = run_oracle(O, d, frac=args.cpu_frac)
        line["cpu_baseline"] = {
            "value": dep / dt, "unit": "deposits/s", "cores": threads, "kind": "port",
            "sample": (f"{m} of {n} particles mapped onto the full 256^3 grid by the FP64 "
                       f"oracle, {threads} threads (parallel=true decomposition)")}
        if m == n:
            line["config"]["rel_linf_vs_oracle"] = _rel_linf(img_main.cpu().numpy(),
                                                             np.asarray(img_ref).reshape(-1, order="F"))
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()
    return 0


CONFIG1_WORKLOAD = ("2D projected map: N=2^18 Float64 particles uniform in the unit cube, hsml lognormal "
                    "(median 0.01, sigma 0.5) clipped to [0.002, 0.1], m = 1/N, rho uniform in [0.5, 2], "
                    "Bin_Quant = Weights = rho, Cubic, 256^2, reduce_image=true, seed 0")


def _weighted_errors(got, ref, W, absq_ref=None):
    """Relative L-infinity of `got` against `ref` on the pixels carrying
    weight (W >= 1e-6 max W): plainly relative to each pixel's value, and
    relative to the map of |q| (the same map where every q > 0)."""
    got = np.asarray(got, dtype=np.float64).reshape(-1)
    ref = np.asarray(ref, dtype=np.float64).reshape(-1)
    W = np.asarray(W, dtype=np.float64).reshape(-1)
    keep = W >= 1e-6 * W.max()
    d = np.abs(got - ref)
    a = np.abs(ref)
    plain = float((d[keep & (a > 0)] / a[keep & (a > 0)]).max()) if (keep & (a > 0)).any() else 0.0
    if absq_ref is None:
        return plain, plain
    sc = np.maximum(a, np.abs(np.asarray(absq_ref, dtype=np.float64).reshape(-1)))
    sel = keep & (sc > 0)
    return plain, (float((d[sel] / sc[sel]).max()) if sel.any() else 0.0)


def bench_config1(pkg, dev, steps, warmup):
    """The 2D projected map (the reference's CPU-runnable case) at full size:
    FP32C and plain FP64 maps/s on the GPU, each against the oracle on the
    pixels carrying weight, and the oracle on all host threads."""
    import torch
    from sphtogrid_gb300 import synth
    d = synth.uniform_2d()
    P = d["npix"]
    par = pkg.mappingParameters(x_lim=[0, 1], y_lim=[0, 1], z_lim=[0, 1], Npixels=P)
    tp = torch.from_numpy(np.ascontiguousarray(d["pos"].T)).to(dev).T
    ts = [torch.from_numpy(np.ascontiguousarray(d[k])).to(dev) for k in ("hsml", "mass", "rho", "bin_q", "weights")]
    stream = torch.cuda.current_stream(dev)

    def run(prec, k, w):
        img = st = None
        for _ in range(w):
            img, st = pkg.sphMapping(tp, *ts, param=par, kernel=pkg.Cubic(2), precision=prec, show_progress=False,
                                     return_stats=True, center_in_place=False)
        torch.cuda.synchronize(dev)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(k):
            img, st = pkg.sphMapping(tp, *ts, param=par, kernel=pkg.Cubic(2), precision=prec, show_progress=False,
                                     return_stats=True, center_in_place=False)
        e1.record(stream)
        torch.cuda.synchronize(dev)
        return e0.elapsed_time(e1) / k, img.cpu().numpy(), st

    ms32, img32, st = run("fp32c", steps, warmup)
    ms64, img64, _ = run("fp64", max(2, steps // 2), 1)
    O = oracle_module()
    opar = O.mapping_parameters(x_lim=[0, 1], y_lim=[0, 1], z_lim=[0, 1], Npixels=P)
    threads = os.cpu_count() or 1
    args = (d["hsml"], d["mass"], d["rho"], d["bin_q"], d["weights"])
    t0 = time.perf_counter()
    ref, info = O.sph_mapping(d["pos"].copy(order="F"), *args, param=opar, kernel="cubic", dimensions=2,
                              nthreads=threads)
    cpu_s = time.perf_counter() - t0
    raw, _ = O.sph_mapping(d["pos"].copy(order="F"), *args, param=opar, kernel="cubic", dimensions=2,
                           return_both_maps=True, nthreads=threads)
    W = raw[:, -1].reshape(P, P)  # raw rows x*P + y -> [x, y]
    ref = np.asarray(ref).reshape(P, P)
    e32 = _weighted_errors(img32.reshape(P, P), ref, W)[0]
    e64 = _weighted_errors(img64.reshape(P, P), ref, W)[0]
    dep = st["deposits"]
    assert dep == info["deposits"], (dep, info["deposits"])
    return {"workload": CONFIG1_WORKLOAD, "particles": int(d["pos"].shape[1]), "deposits_per_map": int(dep),
            "fp32c": {"ms_per_map": ms32, "maps_per_s": 1e3 / ms32, "deposits_per_s": dep / (ms32 * 1e-3),
                      "rel_linf_vs_oracle": e32},
            "plain_fp64": {"ms_per_map": ms64, "maps_per_s": 1e3 / ms64, "deposits_per_s": dep / (ms64 * 1e-3),
                           "rel_linf_vs_oracle": e64},
            "speedup_fp32c_vs_fp64": ms64 / ms32,
            "error_norm": "relative L-infinity on pixels with W >= 1e-6 max W (q = rho > 0)",
            "cpu_baseline": {"kind": "port", "cores": threads, "sample": "the whole map",
                             "ms_per_map": cpu_s * 1e3, "deposits_per_s": dep / cpu_s}}


BATCH_WORKLOAD = ("96 independent 2D maps, particle counts lognormal in [1e4, 2e6], Npixels in "
                  "{128, 256, 512, 1024}, 1-4 quantities (rho, lognormal temperature, Gaussian "
                  "velocity component sigma 300, lognormal |B|), Quintic and WendlandC4 mixed, "
                  "Float32, seed 0; one persistent work-queue launch per phase, CUDA graph replay, "
                  "autotuned tiles")


def bench_batched(pkg, dev, steps, warmup, n_maps=96, deterministic=False, tuning=None, with_oracle=True):
    """The batched uneven-maps workload: maps/s of one graph-replayed batch
    against the plain FP64 method called map by map, each map's error against
    the plain FP64 map (on pixels with W >= 1e-6 max W, relative to the value
    and relative to the map of |q| where quantities of both signs cancel),
    and eight maps spanning the particle counts against the oracle."""
    import torch
    from sphtogrid_gb300 import synth
    from sphtogrid_gb300.batch import MapSpec, SPHBatch
    maps = synth.batched_2d(n_maps=n_maps)
    specs, host = [], []
    for d in maps:
        par = pkg.mappingParameters(x_lim=[0, 1], y_lim=[0, 1], z_lim=[0, 1], Npixels=d["npix"])
        tp = torch.from_numpy(np.ascontiguousarray(d["pos"].T)).to(dev).T
        ts = [torch.from_numpy(np.ascontiguousarray(d[k])).to(dev)
              for k in ("hsml", "mass", "rho", "bin_q", "weights")]
        kern = pkg.kernel_from_name(d["kernel"], 2)
        specs.append(MapSpec(tp, *ts, param=par, kernel=kern, dimensions=2))
        host.append((par, tp, ts, kern))
    t0 = time.perf_counter()
    # plans, autotunes (unless the tuning is given) and captures the graph
    b = SPHBatch(specs, deterministic=deterministic, tuning=tuning)
    plan_s = time.perf_counter() - t0
    for _ in range(warmup):
        b.launch()
    stats = b.wait()
    deposits = sum(x["deposits"] for x in stats)
    stream = torch.cuda.current_stream(dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        b.launch()
    e1.record(stream)
    b.wait()
    ms_batch = e0.elapsed_time(e1) / steps

    def one(par, tp, ts, kern, q=None, raw=False):
        h, m, rho, bq, w = ts
        return pkg.sphMapping(tp, h, m, rho, bq if q is None else q, w, param=par, kernel=kern,
                              precision="fp64", return_both_maps=raw, show_progress=False,
                              center_in_place=False)

    for x in host[:4]:
        one(*x)
    torch.cuda.synchronize(dev)
    e0.record(stream)
    for x in host:
        one(*x)
    e1.record(stream)
    torch.cuda.synchronize(dev)
    ms64 = e0.elapsed_time(e1)
    errs, errs_plain = [], []
    # maps also checked against the oracle: 8 spanning the particle counts
    by_n = np.argsort([d["pos"].shape[1] for d in maps], kind="stable")
    pick = sorted(set(int(by_n[k]) for k in np.linspace(0, len(maps) - 1, min(8, len(maps))).round().astype(int)))
    vs_oracle = []
    O = oracle_module() if with_oracle else None
    for i, x in enumerate(host):
        par = x[0]
        P = int(par.Npixels[0])
        raw = one(*x, raw=True).cpu().numpy()
        absq = one(*x, q=x[2][3].abs(), raw=True).cpu().numpy()
        if O is not None and i in pick:
            dm = maps[i]
            opar = O.mapping_parameters(x_lim=[0, 1], y_lim=[0, 1], z_lim=[0, 1], Npixels=P)
            oraw, _ = O.sph_mapping(dm["pos"].copy(order="F"), dm["hsml"], dm["mass"], dm["rho"], dm["bin_q"],
                                    dm["weights"], param=opar, kernel=dm["kernel"], dimensions=2,
                                    return_both_maps=True, nthreads=os.cpu_count() or 1)
            oW = oraw[:, -1:]
            onq = oraw.shape[1] - 1
            oref = np.where(oW > 0, oraw[:, :onq] / np.where(oW > 0, oW, 1.0), oraw[:, :onq])
            oabs = np.where(oW > 0, absq[:, :onq] / np.where(oW > 0, oW, 1.0), absq[:, :onq])
            ogot = b.image(i).cpu().numpy().reshape(P * P, onq)
            ep, es = _weighted_errors(ogot, oref, np.repeat(oW, onq, axis=1), oabs)
            # channels whose quantity has one sign: there Q / W cannot cancel
            qk = np.asarray(dm["bin_q"], dtype=np.float64).reshape(onq, -1)
            one_sign = [k for k in range(onq) if qk[k].min() >= 0.0 or qk[k].max() <= 0.0]
            e1 = _weighted_errors(ogot[:, one_sign], oref[:, one_sign], np.repeat(oW, len(one_sign), axis=1))[0] \
                if one_sign else None
            vs_oracle.append({"map": i, "particles": int(dm["pos"].shape[1]), "npix": P, "quantities": onq,
                              "rel_linf_absq_scaled": es, "rel_linf_plain": ep,
                              "rel_linf_plain_single_sign_channels": e1})
        W = raw[:, -1:]
        nq = raw.shape[1] - 1
        ref = np.where(W > 0, raw[:, :nq] / np.where(W > 0, W, 1.0), raw[:, :nq])
        scale = np.where(W > 0, absq[:, :nq] / np.where(W > 0, W, 1.0), absq[:, :nq])
        got = b.image(i).cpu().numpy().reshape(P * P, nq)  # [x, y, q] -> rows x*P + y
        ep, es = _weighted_errors(got, ref, np.repeat(W, nq, axis=1), scale)
        errs.append(es)
        errs_plain.append(ep)
    n = len(maps)
    out = {"workload": BATCH_WORKLOAD, "maps": n,
           "particles": int(sum(d["pos"].shape[1] for d in maps)),
           "deposits_per_batch": int(deposits), "ms_per_batch": ms_batch,
           "maps_per_s": 1e3 * n / ms_batch, "deposits_per_s": deposits / (ms_batch * 1e-3),
           "plain_fp64_maps_per_s": 1e3 * n / ms64, "speedup_vs_plain_fp64": ms64 / ms_batch,
           "rel_err_max": max(errs), "rel_err_median": float(np.median(errs)),
           "rel_err_per_map": [float(f"{e:.3g}") for e in errs],
           "rel_err_plain_max": max(errs_plain),
           "error_norms": ("against the plain FP64 map of each map, on pixels with W >= 1e-6 max W: "
                           "rel_err_* relative to the map of |q| (the value itself where q > 0), "
                           "rel_err_plain_* relative to the value itself"),
           "vs_oracle": vs_oracle,
           "deterministic": bool(deterministic), "tuning": b.tuning,
           "plan_and_autotune_s": plan_s}
    b.close()
    return out


LARGE_WORKLOAD = ("large high-dynamic-range projection: N~2^27 Float32 particles sampled from a "
                  "log-normal density field (sigma_ln 2, P(k) ~ k^-3 on a 512^3 seed grid) in the unit "
                  "box, hsml from the density clipped to [1e-4, 0.2], Cubic, 4096^2, Bin_Quant = "
                  "Weights = rho, seed 0")


def bench_large(pkg, dev, steps, warmup, n=2 ** 27, npix=4096, seed_grid=512):
    """The large-particle workload: FP32C and deterministic against the plain
    FP64 method on the same resident inputs, with the FP32C error map against
    FP64 summarised (pixels carrying weight: W >= 1e-6 max W)."""
    import torch
    from sphtogrid_gb300 import synth
    t0 = time.perf_counter()
    d = synth.large_hdr_2d(N=n, npix=npix, seed_grid=seed_grid)
    gen_s = time.perf_counter() - t0
    par = pkg.mappingParameters(x_lim=[0, 1], y_lim=[0, 1], z_lim=[0, 1], Npixels=npix)
    tp = torch.from_numpy(np.ascontiguousarray(d["pos"].T)).to(dev).T
    ts = [torch.from_numpy(np.ascontiguousarray(d[k])).to(dev)
          for k in ("hsml", "mass", "rho", "bin_q", "weights")]
    stream = torch.cuda.current_stream(dev)

    def run(prec, det, k, w):
        out = None
        for _ in range(w):
            out, st = pkg.sphMapping(tp, *ts, param=par, kernel=pkg.Cubic(2), precision=prec,
                                     deterministic=det, return_both_maps=True, show_progress=False,
                                     return_stats=True, center_in_place=False)
        torch.cuda.synchronize(dev)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(k):
            out, st = pkg.sphMapping(tp, *ts, param=par, kernel=pkg.Cubic(2), precision=prec,
                                     deterministic=det, return_both_maps=True, show_progress=False,
                                     return_stats=True, center_in_place=False)
        e1.record(stream)
        torch.cuda.synchronize(dev)
        return e0.elapsed_time(e1) / k, out.cpu().numpy(), st

    ms32, raw32, st = run("fp32c", False, steps, warmup)
    msd, rawd, _ = run("fp32c", True, steps, warmup)
    ms64, raw64, _ = run("fp64", False, max(1, steps // 4), 1)
    W = raw64[:, -1]
    keep = W >= 1e-6 * W.max()
    dep = st["deposits"]

    def err(raw):
        e = np.abs(raw[keep] - raw64[keep]) / np.abs(raw64[keep])
        return e

    e32 = err(raw32)
    hist = np.histogram(np.log10(np.maximum(e32.reshape(-1), 1e-18)), bins=[-18, -9, -8, -7, -6, -5, 0])[0]
    return {"workload": LARGE_WORKLOAD, "particles": int(d["pos"].shape[1]), "npix": npix,
            "deposits_per_map": int(dep), "generation_s": gen_s,
            "hsml_px": {"min": float(d["hsml"].min()) * npix, "max": float(d["hsml"].max()) * npix},
            "fp32c": {"ms_per_map": ms32, "deposits_per_s": dep / (ms32 * 1e-3),
                      "rel_linf_vs_fp64": float(e32.max()), "rel_median_vs_fp64": float(np.median(e32))},
            "deterministic": {"ms_per_map": msd, "deposits_per_s": dep / (msd * 1e-3),
                              "rel_linf_vs_fp64": float(err(rawd).max())},
            "plain_fp64": {"ms_per_map": ms64, "deposits_per_s": dep / (ms64 * 1e-3)},
            "speedup_fp32c_vs_fp64": ms64 / ms32,
            "error_map_log10_histogram": {"bins": [-18, -9, -8, -7, -6, -5, 0],
                                          "pixels": [int(x) for x in hist]},
            "pixels_carrying_weight": int(keep.sum())}


DIFF_WORKLOAD = ("differentiable deposition: N=2^20 Float64 particles uniform in the unit cube, hsml "
                 "lognormal (median 0.01, sigma 0.5) clipped to [0.002, 0.1], m = 1/N, rho uniform in "
                 "[0.5, 2], Bin_Quant = Weights = rho, 2D-projected to 512^2 with WendlandC4; loss "
                 "sum((map - target)^2), target the map of a copy with positions jittered by 0.1 hsml "
                 "and Bin_Quant scaled lognormal sigma 0.1; seed 0")


def bench_differentiable(pkg, dev, steps, warmup, cpu_sample=2 ** 16):
    """The differentiable deposition: forward map, loss and the hand-written
    adjoint (dL/d positions, hsml, m, rho, weights, Bin_Quant) on the GPU,
    each timed with CUDA events, for the FP64 and the FP32C forward; the
    oracle's forward map on the host cores beside it.  The gradients' check
    against FP64 central differences (256 particles, 1e-4) is
    tests/test_gpu_adjoint_full.py."""
    import torch
    from sphtogrid_gb300 import synth
    d = synth.differentiable_2d()
    n, P = d["pos"].shape[1], 512
    par = pkg.mappingParameters(x_lim=[0, 1], y_lim=[0, 1], z_lim=[0, 1], Npixels=P)
    rng = np.random.default_rng(4)
    tpos = torch.from_numpy(np.ascontiguousarray(d["pos"].T)).to(dev).T
    ts = [torch.from_numpy(np.ascontiguousarray(d[k])).to(dev) for k in ("hsml", "mass", "rho", "bin_q", "weights")]
    with torch.no_grad():
        jit = tpos + 0.1 * ts[0] * torch.randn(3, n, dtype=torch.float64, device=dev)
        qj = ts[3] * torch.from_numpy(rng.lognormal(0.0, 0.1, n)).to(dev)
        target = pkg.sph_map_differentiable(jit, ts[0], ts[1], ts[2], qj, ts[4], param=par,
                                            kernel=pkg.WendlandC4(2), dimensions=2)
    stream = torch.cuda.current_stream(dev)
    out = {"workload": DIFF_WORKLOAD, "particles": n, "npix": P}
    for name, prec, adj in (("fp64", "fp64", "fp64"), ("fp64_forward_fp32c_adjoint", "fp64", "fp32c"),
                            ("fp32c", "fp32c", "fp32c")):
        leaves = [tpos.clone().requires_grad_(True)] + [t.clone().requires_grad_(True) for t in ts]
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
        fw = bw = 0.0
        for it in range(warmup + steps):
            for t in leaves:
                t.grad = None
            ev[0].record(stream)
            img = pkg.sph_map_differentiable(*leaves, param=par, kernel=pkg.WendlandC4(2),
                                             dimensions=2, precision=prec, adjoint_precision=adj)
            loss = ((img - target) ** 2).sum()
            ev[1].record(stream)
            loss.backward()
            ev[2].record(stream)
            torch.cuda.synchronize(dev)
            if it >= warmup:
                fw += ev[0].elapsed_time(ev[1])
                bw += ev[1].elapsed_time(ev[2])
        out[name] = {"ms_forward_and_loss": fw / steps, "ms_adjoint": bw / steps,
                     "ms_forward_backward": (fw + bw) / steps}
    # the oracle's forward map (the reference has no derivatives), host cores
    O = oracle_module()
    m_s = min(cpu_sample, n)
    opar = O.mapping_parameters(x_lim=[0, 1], y_lim=[0, 1], z_lim=[0, 1], Npixels=P)
    t0 = time.perf_counter()
    _, info = O.sph_mapping(np.asfortranarray(d["pos"][:, :m_s]).copy(order="F"), d["hsml"][:m_s],
                            d["mass"][:m_s], d["rho"][:m_s], d["bin_q"][:m_s], d["weights"][:m_s],
                            param=opar, kernel="wendlandc4", kernel_dim=2, nthreads=os.cpu_count())
    cpu_s = time.perf_counter() - t0
    out["cpu_baseline"] = {"kind": "port", "cores": os.cpu_count(),
                           "sample": f"{m_s} of {n} particles, forward map only (no derivatives in the reference)",
                           "deposits_per_s": info["deposits"] / cpu_s}
    return out


HEALPIX_WORKLOAD = ("all-sky HEALPix map: N=2^20 particles in a shell 2 < r < 6 around the observer "
                    "(directions isotropic), hsml uniform in [0.02, 0.8], m and rho uniform, Cubic, "
                    "Nside=512, FP64, seed 0")


def bench_healpix(pkg, dev, steps, warmup, n=2 ** 20, nside=512, cpu_sample=2 ** 12):
    """The all-sky path: GPU healpix_map (FP64) against the oracle's restated
    loop on one host core, on a bounded sample of the same particles."""
    import torch
    rng = np.random.default_rng(0)
    r = rng.uniform(2.0, 6.0, n)
    v = rng.standard_normal((3, n))
    v /= np.linalg.norm(v, axis=0)
    pos = np.asfortranarray(v * r)
    hsml = rng.uniform(0.02, 0.8, n)
    m = rng.uniform(0.5, 1.5, n)
    rho = rng.uniform(0.5, 2.0, n)
    q = rng.uniform(0.5, 2.0, n)
    t = [torch.from_numpy(np.ascontiguousarray(a)).to(dev) for a in (hsml, m, rho, q, rho)]
    tp = torch.from_numpy(np.ascontiguousarray(pos.T)).to(dev).T  # (3, N), xyz per particle

    def once(k):
        out = None
        for _ in range(k):
            p2 = tp.clone()
            out = pkg.healpix_map(p2, *t, Nside=nside, kernel=pkg.Cubic(3), show_progress=False,
                                  return_stats=True)
        return out
    once(warmup)
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    _, _, st = once(steps)
    torch.cuda.synchronize(dev)
    gpu_s = (time.perf_counter() - t0) / steps
    O = oracle_module()
    m_s = min(cpu_sample, n)
    t0 = time.perf_counter()
    ra, rw, info = O.healpix_map(np.asfortranarray(pos[:, :m_s]).copy(order="F"), hsml[:m_s], m[:m_s],
                                 rho[:m_s], q[:m_s], rho[:m_s], Nside=nside, kernel="cubic")
    cpu_s = time.perf_counter() - t0
    ga, gw, st_s = pkg.healpix_map(tp[:, :m_s].clone(), *[a[:m_s] for a in t], Nside=nside,
                                   kernel=pkg.Cubic(3), show_progress=False, return_stats=True)
    gw = gw.cpu().numpy()
    sel = rw > 1e-9 * rw.max()
    err = float((np.abs(gw[sel] - rw[sel]) / rw[sel]).max())
    return {"workload": HEALPIX_WORKLOAD, "particles": n, "nside": nside,
            "pixel_deposits": int(st["deposits"]), "gpu_s_per_map": gpu_s,
            "gpu_pixel_deposits_per_s": st["deposits"] / gpu_s,
            "cpu_baseline": {"kind": "port", "cores": 1, "sample": f"{m_s} of {n} particles",
                             "pixel_deposits_per_s": st_s["deposits"] / cpu_s},
            "speedup_vs_cpu_per_core": (st["deposits"] / gpu_s) / (st_s["deposits"] / cpu_s),
            "rel_linf_weight_map_vs_oracle_on_sample": err}


def _onchip_ceiling(L, ctx, _lib, value, other, det):
    """The deposit rate the shared-memory accumulation alone allows (3D map:
    one quantity + the weight = 2 channel additions per deposit), from the
    library's conflict-free microbenchmark, and the fraction reached."""
    names = {0: "fp32_atomic_with_return", 1: "fp32_atomic_no_return", 2: "int64_atomic",
             3: "fp32_compensated_add_two_atomics", 4: "fp32_compensated_pair_cas",
             5: "int64_fixed_point_two_u32_atomics", 6: "int64_fixed_point_three_chunk_reductions"}
    rates = {}
    for kind, nm in names.items():
        r = C.c_double()
        _lib.check(L.sphg_probe_smem_rate(ctx.handle, kind, C.byref(r)), ctx.handle)
        rates[nm] = r.value
    chans = 2
    ceil_c = rates["fp32_compensated_add_two_atomics"] / chans  # the FP32C deposit's accumulation
    ceil_d = rates["int64_fixed_point_three_chunk_reductions"] / chans  # the deterministic deposit's (tiles of <= 2047 pairs)
    v_c = value if not det else (other or {}).get("value")
    v_d = value if det else (other or {}).get("value")
    return {"smem_additions_per_s": rates, "channel_additions_per_deposit": chans,
            "deposit_ceiling_fp32c": ceil_c, "deposit_ceiling_deterministic": ceil_d,
            "frac_fp32c": (v_c / ceil_c) if v_c else None,
            "frac_deterministic": (v_d / ceil_d) if v_d else None}


def _rel_linf(a, b, floor=1e-9):
    a = np.asarray(a, dtype=np.float64).reshape(-1)
    b = np.asarray(b, dtype=np.float64).reshape(-1)
    top = np.abs(b).max()
    if top == 0:
        return float(np.abs(a).max())
    sel = np.abs(b) > floor * top
    rel = np.abs(a[sel] - b[sel]) / np.abs(b[sel])
    rest = np.abs(a[~sel] - b[~sel]).max() / top if (~sel).any() else 0.0
    return float(max(rel.max() if rel.size else 0.0, rest))


def _peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            j = json.load(f)
        return float(j["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def _traffic_per_launch():
    """DRAM bytes per deposit launch from the committed ncu summary, if any."""
    p = os.path.join(ROOT, "profiles", "deposit_traffic.json")
    try:
        with open(p) as f:
            return float(json.load(f)["dram_bytes_per_launch"])
    except (OSError, KeyError, ValueError):
        return None


def main():
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--precision", default="fp32c", choices=["fp32c", "fp64"])
    ap.add_argument("--cpu-frac", type=float, default=1.0,
                    help="fraction of the particles the CPU baseline maps")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--deterministic", action="store_true",
                    help="bitwise reproducible int64 fixed-point tile sums")
    ap.add_argument("--only-device", action="store_true",
                    help="time the device-resident loop only (for profiler runs)")
    ap.add_argument("--no-batched", action="store_true",
                    help="skip the batched 96-map workload")
    ap.add_argument("--no-sub-workloads", action="store_true",
                    help="skip the 2D projection and differentiable sub-records")
    ap.add_argument("--batched-only", action="store_true",
                    help="time the batched workload alone (for profiler runs)")
    ap.add_argument("--batched-maps", type=int, default=96,
                    help="maps in the batched workload (smaller for profiler captures)")
    ap.add_argument("--workload", default="clumps_3d",
                    choices=["clumps_3d", "large_hdr", "healpix", "differentiable", "projection_2d"],
                    help="large_hdr: the large-particle projection (2^27 particles, 4096^2), "
                         "FP32C and deterministic against plain FP64 with the error map")
    ap.add_argument("--large-particles", type=int, default=2 ** 27,
                    help="particles of the large-particle workload (smaller for profiler captures)")
    ap.add_argument("--large-npix", type=int, default=4096,
                    help="Npixels of the large-particle workload")
    ap.add_argument("--healpix-particles", type=int, default=2 ** 20,
                    help="particles of the all-sky workload (smaller for profiler captures)")
    ap.add_argument("--batched-tuning", default=None,
                    help="tile_x,tile_y,ctas_per_sm,large_cells instead of autotuning")
    args = ap.parse_args()
    if args.impl == "reference":
        return bench_reference(args)
    return bench_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
