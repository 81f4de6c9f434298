"""Reference gradients for the adjoint tests (test infrastructure).

* ``fd_grad``: FP64 central finite differences of L = sum((out - t)^2) with
  respect to one parameter of one particle.  Only that particle's weights
  change, so the oracle recomputes them alone (``oracle.particle_contrib``)
  and the perturbed reduced map is rebuilt on its footprint from the full raw
  accumulator: the difference is exact up to FP64 rounding.
* ``dual_grad``: forward-mode derivative (dual numbers) of the same loss
  through the pure-Python restatement of the reference (``pyoracle``) -- the
  stand-in for ForwardDiff over the reference, which needs Julia.

Positions must be centred on 0 (parameters with centre [0, 0, 0]) so that the
reference's centring is the identity.
"""
from __future__ import annotations

import math

import numpy as np

PARAMS = ("x", "y", "z", "hsml", "mass", "rho", "weights", "q")


class Dual:
    """a + b eps with eps^2 = 0; comparisons use the value part."""

    __slots__ = ("v", "d")

    def __init__(self, v, d=0.0):
        self.v = float(v)
        self.d = float(d)

    @staticmethod
    def _c(o):
        return o if isinstance(o, Dual) else Dual(o, 0.0)

    def __add__(self, o):
        o = Dual._c(o)
        return Dual(self.v + o.v, self.d + o.d)

    __radd__ = __add__

    def __sub__(self, o):
        o = Dual._c(o)
        return Dual(self.v - o.v, self.d - o.d)

    def __rsub__(self, o):
        return Dual._c(o) - self

    def __mul__(self, o):
        o = Dual._c(o)
        return Dual(self.v * o.v, self.d * o.v + self.v * o.d)

    __rmul__ = __mul__

    def __truediv__(self, o):
        o = Dual._c(o)
        return Dual(self.v / o.v, (self.d * o.v - self.v * o.d) / (o.v * o.v))

    def __rtruediv__(self, o):
        return Dual._c(o) / self

    def __neg__(self):
        return Dual(-self.v, -self.d)

    def sqrt(self):
        r = math.sqrt(self.v)
        return Dual(r, self.d / (2.0 * r) if r > 0 else 0.0)

    def __lt__(self, o):
        return self.v < Dual._c(o).v

    def __le__(self, o):
        return self.v <= Dual._c(o).v

    def __gt__(self, o):
        return self.v > Dual._c(o).v

    def __ge__(self, o):
        return self.v >= Dual._c(o).v

    def __eq__(self, o):
        return self.v == Dual._c(o).v

    def __ne__(self, o):
        return self.v != Dual._c(o).v

    __hash__ = None


def reduce_rows(raw, dims, reduce_image=True):
    """Reduced map on raw rows: raw (PD, nq+1) -> (PD, nq)."""
    Q, W = raw[:, :-1], raw[:, -1:]
    if dims == 2:
        return np.where((W > 0) & reduce_image, Q / np.where(W > 0, W, 1.0), Q)
    return np.where(Q > 0, Q / np.where(Q > 0, W, 1.0), Q)


def rows_to_output(g_rows, dims, P):
    """(PD, nq) on raw rows -> flat column-major output layout."""
    if dims == 2:
        nq = g_rows.shape[1]
        return g_rows.reshape(P, P, nq).flatten(order="F")
    return g_rows[:, 0].copy()


def _perturbed(case, p, name, k, delta):
    pos, hsml, m, rho, q, w = case
    x = [float(pos[d, p]) for d in range(3)]
    vals = dict(hsml=float(hsml[p]), mass=float(m[p]), rho=float(rho[p]), weights=float(w[p]))
    qq = q.reshape(-1, q.shape[-1])[:, p].astype(np.float64).copy()
    if name in ("x", "y", "z"):
        x["xyz".index(name)] += delta
    elif name == "q":
        qq[k] += delta
    else:
        vals[name] += delta
    return x, vals, qq


def fd_grad(oracle, case, par, dims, kernel, kdim, raw, target_rows, p, name, k=0, rel=1e-6,
            reduce_image=True):
    pos, hsml, m, rho, q, w = case
    nq = raw.shape[1] - 1
    base = {"x": hsml[p], "y": hsml[p], "z": hsml[p], "hsml": hsml[p], "mass": m[p],
            "rho": rho[p], "weights": w[p], "q": 1.0}[name]
    eps = rel * abs(float(base)) if name != "q" else rel * max(1.0, abs(float(q.reshape(nq, -1)[k, p])))
    x0, v0, q0 = _perturbed(case, p, name, k, 0.0)
    i0, pw0 = oracle.particle_contrib(dims, par, kernel, kdim, *x0, v0["hsml"], v0["mass"],
                                      v0["rho"], v0["weights"])
    losses = []
    for sgn in (1.0, -1.0):
        x1, v1, q1 = _perturbed(case, p, name, k, sgn * eps)
        i1, pw1 = oracle.particle_contrib(dims, par, kernel, kdim, *x1, v1["hsml"], v1["mass"],
                                          v1["rho"], v1["weights"])
        U = np.union1d(i0, i1)
        sub = raw[U].copy()
        pos0 = np.searchsorted(U, i0)
        pos1 = np.searchsorted(U, i1)
        sub[pos0, -1] -= pw0
        sub[pos1, -1] += pw1
        for c in range(nq):
            sub[pos0, c] -= q0[c] * pw0
            sub[pos1, c] += q1[c] * pw1
        out = reduce_rows(sub, dims, reduce_image)
        losses.append(((out - target_rows[U]) ** 2).sum() - (
            (reduce_rows(raw[U], dims, reduce_image) - target_rows[U]) ** 2).sum())
    return (losses[0] - losses[1]) / (2.0 * eps)


def dual_grad(pyoracle, case, par, dims, kernel, kdim, target_rows, p, name, k=0,
              reduce_image=True):
    """dL/dtheta by forward-mode dual numbers over the Python restatement."""
    pos, hsml, m, rho, q, w = case
    n = pos.shape[1]
    nq = 1 if q.ndim == 1 else q.shape[0]
    qq = q.reshape(nq, n)
    P = int(par.Npixels[0])
    L = par.len2pix
    posl = [[float(pos[d, i]) for d in range(3)] for i in range(n)]
    hs, ms, rs, ws = [list(map(float, a)) for a in (hsml, m, rho, w)]
    ql = [[float(qq[c, i]) for c in range(nq)] for i in range(n)]
    if name in ("x", "y", "z"):
        posl[p]["xyz".index(name)] = Dual(posl[p]["xyz".index(name)], 1.0)
    elif name == "q":
        ql[p][k] = Dual(ql[p][k], 1.0)
    else:
        arr = {"hsml": hs, "mass": ms, "rho": rs, "weights": ws}[name]
        arr[p] = Dual(arr[p], 1.0)
    chans, _ = pyoracle.cic_map(dims, posl, hs, ms, rs, ql, ws, L, P, kernel, kdim)
    loss = Dual(0.0)
    rows = set()
    for ch in chans:
        rows |= set(ch.keys())
    for row in rows:
        W = chans[nq].get(row, 0.0)
        for c in range(nq):
            Q = chans[c].get(row, 0.0)
            if dims == 2:
                o = Q / W if (reduce_image and (W.v if isinstance(W, Dual) else W) > 0) else Q
            else:
                o = Q / W if (Q.v if isinstance(Q, Dual) else Q) > 0 else Q
            diff = o - float(target_rows[row, c])
            loss = loss + diff * diff
    # rows never touched contribute a constant
    return loss.d if isinstance(loss, Dual) else 0.0
