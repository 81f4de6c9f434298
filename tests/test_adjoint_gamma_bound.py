"""The FP32C adjoint's image gradient gam = dL/dW + sum_k q_k dL/dQ_k
(adjoint.cu, adj_fp32_sums) is formed from FP32 (hi, lo) pairs of its
factors with exact products (FMA) and exact sums (TwoSum), then rounded
once.  Its formation error must stay below kGamEps (|dL/dW| + sum_k
|q_k dL/dQ_k|), the term the per-particle error estimate adds for it.

This restates those FP32 steps in numpy (IEEE float32, round to nearest;
the FMA's exact product is formed in float64, where a product of two floats
is exact) and checks the bound, read from the source, against exact
rational arithmetic on cases whose parts cancel down to 1e-9 of their size.
No GPU: the kernel itself is checked against finite differences in
test_gpu_adjoint.py."""
import re
from fractions import Fraction
from pathlib import Path

import numpy as np

f32 = np.float32
SRC = Path(__file__).resolve().parents[1] / "sphtogrid.jl_gb300" / "csrc" / "adjoint.cu"


def _kgameps():
    m = re.search(r"constexpr float kGamEps = ([0-9.eE+-]+)f;", SRC.read_text())
    assert m, "kGamEps not found in adjoint.cu"
    return float(m.group(1))


def _split(v):
    """k_adj_reduce's planes: hi = float(v), lo = float(v - hi)."""
    h = f32(v)
    return h, f32(v - float(h))


def _gamma(gw, q, gq):
    """adj_fp32_sums' gamma_at: returns (s, e) before the final s + e, and mag."""
    s, e = _split(gw)
    mag = abs(s)
    for qk, gk in zip(q, gq):
        qh, ql = _split(qk)
        gh, gl = _split(gk)
        pr = f32(qh * gh)
        pe = f32(float(qh) * float(gh) - float(pr))  # fmaf(qh, gh, -pr)
        t = f32(s + pr)
        bp = f32(t - s)
        se = f32(f32(s - f32(t - bp)) + f32(pr - bp))
        s = t
        e = f32(e + f32(f32(se + pe) + f32(f32(qh * gl) + f32(ql * gh))))
        mag = f32(mag + abs(pr))
    return s, e, mag


def test_image_gradient_formation_within_kgameps():
    eps = _kgameps()
    assert 0.0 < eps < 1e-9
    rng = np.random.default_rng(11)
    worst = 0.0
    for _ in range(3000):
        nq = int(rng.integers(1, 5))
        q = rng.uniform(0.5, 2.0, nq) * 10.0 ** rng.uniform(-3, 3)
        gq = rng.normal(size=nq) * 10.0 ** rng.uniform(-8, 2)
        # dL/dW cancels sum_k q_k dL/dQ_k down to 10^-c of its size
        gw = -float(np.dot(q, gq)) * (1.0 + rng.normal() * 10.0 ** -rng.uniform(0, 9))
        exact = Fraction(gw) + sum(Fraction(float(a)) * Fraction(float(b)) for a, b in zip(q, gq))
        s, e, mag = _gamma(gw, q, gq)
        err = abs(Fraction(float(s)) + Fraction(float(e)) - exact)
        worst = max(worst, float(err) / (eps * float(mag)))
    # the bound holds with a wide margin (about 1% of it is used)
    assert worst < 0.1, worst


def test_image_gradient_without_cancellation_is_float_accurate():
    """Without cancellation the final rounding (2^-24 relative) dominates."""
    rng = np.random.default_rng(12)
    for _ in range(500):
        q = rng.uniform(0.5, 2.0, 2)
        gq = rng.uniform(0.5, 2.0, 2)
        gw = float(rng.uniform(0.5, 2.0))
        exact = gw + float(np.dot(q, gq))
        s, e, _ = _gamma(gw, q, gq)
        assert abs(float(f32(s + e)) - exact) <= 2.0 ** -23 * abs(exact)
