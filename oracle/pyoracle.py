"""Second, pure-Python restatement of the reference's CIC deposition.

TEST INFRASTRUCTURE ONLY (small cases: plain Python loops).  It exists to
cross-check the C oracle: both follow the reference's expression order, and
Python floats are IEEE doubles without FMA contraction, so the two must agree
bit for bit.

Follows src/cic_interpolation/cic_2D.jl:11-244, cic_3D.jl:13-208,
cic_shared.jl:9-121, reduce_image.jl:8-55 and shared/indices.jl of
SPHtoGrid.jl.  Inputs are already centred and filtered; the particle order is
the order of the arrays.  Inputs may be any number type with the arithmetic
operators (the adjoint tests pass dual numbers: forward-mode derivatives of
this restatement).
"""
from __future__ import annotations

import math

PI = 3.14159265358979323846

SIGMA = {  # normalisation for support radius h (2D, 3D)
    "cubic": (40.0 / (7.0 * PI), 8.0 / PI),
    "quintic": (15309.0 / (478.0 * PI), 2187.0 / (40.0 * PI)),
    "wendlandc4": (9.0 / PI, 495.0 / (32.0 * PI)),
    "wendlandc6": (78.0 / (7.0 * PI), 1365.0 / (64.0 * PI)),
    "wendlandc8": (40.0 / (3.0 * PI), 1785.0 / (64.0 * PI)),
}


def W(kernel: str, kdim: int, u: float, h_inv: float) -> float:
    hd = h_inv * h_inv if kdim == 2 else h_inv * h_inv * h_inv
    n = SIGMA[kernel][0 if kdim == 2 else 1] * hd
    if kernel == "cubic":
        if u < 0.5:
            return (1.0 + 6.0 * (u - 1.0) * (u * u)) * n
        if u < 1.0:
            t = 1.0 - u
            return (2.0 * (t * t * t)) * n
        return 0.0
    if kernel == "quintic":
        a, b, c = 1.0 - u, 2.0 / 3.0 - u, 1.0 / 3.0 - u
        a5, b5, c5 = a * a * a * a * a, b * b * b * b * b, c * c * c * c * c
        if u < 1.0 / 3.0:
            return (a5 - 6.0 * b5 + 15.0 * c5) * n
        if u < 2.0 / 3.0:
            return (a5 - 6.0 * b5) * n
        if u < 1.0:
            return a5 * n
        return 0.0
    if u >= 1.0:
        return 0.0
    t = 1.0 - u
    t2 = t * t
    if kernel == "wendlandc4":
        return (t2 * t2 * t2 * (1.0 + 6.0 * u + 35.0 / 3.0 * (u * u))) * n
    if kernel == "wendlandc6":
        t4 = t2 * t2
        return (t4 * t4 * (1.0 + 8.0 * u + 25.0 * (u * u) + 32.0 * (u * u * u))) * n
    t4 = t2 * t2
    t8 = t4 * t4
    u2 = u * u
    return (t8 * t2 * (1.0 + 10.0 * u + 42.0 * u2 + 90.0 * (u2 * u) + 429.0 / 5.0 * (u2 * u2))) * n


def _num(v):
    """Plain floats for numpy scalars; other number types (the dual numbers of
    the adjoint tests) pass through."""
    return v if hasattr(v, "d") else float(v)


def _val(v):
    return v.v if hasattr(v, "d") else v


def _sqrt(v):
    return v.sqrt() if hasattr(v, "sqrt") else math.sqrt(v)


def _range(x, h, P):
    return max(math.floor(_val(x - h)), 0), min(math.floor(_val(x + h)), P - 1)


def _overlap(x, h, i):
    return min(x + h, float(i + 1)) - max(x - h, float(i))


def cic_map(dims, pos, hsml, m, rho, q, w, L, P, kernel, kdim=None, calc_mean=False):
    """Raw accumulator as a list of channels: ``q`` is a list of per-particle
    tuples; returns ``[Q_1, ..., Q_nq, W]`` each a dict ``flat idx -> value``
    (0-based, x slowest) plus the deposit count."""
    kdim = dims if kdim is None else kdim
    nq = len(q[0])
    chans = [dict() for _ in range(nq + 1)]
    deposits = 0
    for p in range(len(m)):
        bq = [_num(v) for v in q[p]]
        allzero = all(v == 0.0 for v in bq)
        if allzero and not calc_mean:
            continue
        h = _num(hsml[p]) * L
        h_inv = 1.0 / h
        if dims == 2:
            area = (2.0 * h) * (2.0 * h)
            rho_pix = _num(rho[p]) * (1.0 / (L * L * L))
            col = _num(m[p]) / rho_pix / area
        else:
            rho_pix = _num(rho[p]) / (L * L * L)
            vol = _num(m[p]) / rho_pix
        c = []
        for d in range(3):
            v = _num(pos[p][d]) * L
            v += 0.5 * float(P)
            c.append(v)
        rngs = [_range(c[d], h, P) for d in range(dims)]
        cells = []
        if dims == 2:
            for i in range(rngs[0][0], rngs[0][1] + 1):
                for j in range(rngs[1][0], rngs[1][1] + 1):
                    cells.append((i, j))
        else:
            for i in range(rngs[0][0], rngs[0][1] + 1):
                for j in range(rngs[1][0], rngs[1][1] + 1):
                    for k in range(rngs[2][0], rngs[2][1] + 1):
                        cells.append((i, j, k))
        deposits += len(cells)
        wk, A = [], []
        s_w, s_a, n_d, n_t = 0.0, 0.0, 0, 0
        for cell in cells:
            dist = [c[d] - float(cell[d]) - 0.5 for d in range(dims)]
            ov = [_overlap(c[d], h, cell[d]) for d in range(dims)]
            if dims == 2:
                u = _sqrt(dist[0] * dist[0] + dist[1] * dist[1]) * h_inv
                a = ov[0] * ov[1]
            else:
                u = _sqrt(dist[0] * dist[0] + dist[1] * dist[1] + dist[2] * dist[2]) * h_inv
                a = ov[0] * ov[1] * ov[2]
            A.append(a)
            s_a += a
            n_t += 1
            if u <= 1.0:
                k_ = W(kernel, kdim, u, h_inv)
                s_w += k_ * a
                n_d += 1
                wk.append(k_)
            else:
                wk.append(0.0)
        if s_w == 0.0:
            n_d = n_t
            wk = [1.0] * len(cells)
            wpp = n_d / s_a if s_a != 0.0 else 1.0
        else:
            wpp = n_d / s_w
        if dims == 2:
            norm = area / n_d * wpp * _num(w[p]) * col
        else:
            norm = vol / n_d * wpp * _num(w[p]) * L
        for t, cell in enumerate(cells):
            idx = cell[0] * P + cell[1] if dims == 2 else cell[0] * P * P + cell[1] * P + cell[2]
            pw = wk[t] * A[t] * norm
            if pw != 0.0:
                chans[nq][idx] = chans[nq].get(idx, 0.0) + pw
                if nq > 1 and allzero:
                    chans[0][idx] = chans[0].get(idx, 0.0) + 0.0 * pw
                else:
                    for ch in range(nq):
                        chans[ch][idx] = chans[ch].get(idx, 0.0) + bq[ch] * pw
    return chans, deposits
