"""Oracle (test infrastructure only): the reference's own test elements,
restated so that the oracle's assembler and solver loops can be pinned to the
reference's golden values (test/TestAssemble.jl, test/TestSweepX0.jl,
test/TestSweepX2.jl).

Turbine, AnchorLine and SdofOscillator follow test/SomeElements.jl:15-94 and
:193-207.  Derivatives use a small forward-mode dual over the element's
seeded variables (the Newton variation of src/SweepX.jl:45-96), so they are
exact like the reference's ∂ℝ numbers.
"""
from __future__ import annotations

import math

import numpy as np


class D:
    """First-order dual number with a vector of partials."""

    __slots__ = ("x", "d")

    def __init__(self, x, d):
        self.x = float(x)
        self.d = np.asarray(d, dtype=np.float64)

    @staticmethod
    def c(x, n):
        return D(x, np.zeros(n))

    def _w(self, o):
        return o if isinstance(o, D) else D(o, np.zeros_like(self.d))

    def __add__(self, o):
        o = self._w(o)
        return D(self.x + o.x, self.d + o.d)

    __radd__ = __add__

    def __sub__(self, o):
        o = self._w(o)
        return D(self.x - o.x, self.d - o.d)

    def __rsub__(self, o):
        return self._w(o) - self

    def __neg__(self):
        return D(-self.x, -self.d)

    def __mul__(self, o):
        o = self._w(o)
        return D(self.x * o.x, self.d * o.x + self.x * o.d)

    __rmul__ = __mul__

    def __truediv__(self, o):
        o = self._w(o)
        q = self.x / o.x
        return D(q, (self.d - q * o.d) / o.x)

    def __rtruediv__(self, o):
        return self._w(o) / self

    def __pow__(self, k):
        return D(self.x**k, k * self.x ** (k - 1) * self.d)


def dsqrt(a):
    s = math.sqrt(a.x)
    return D(s, a.d / (2 * s))


def dsin(a):
    return D(math.sin(a.x), math.cos(a.x) * a.d)


def dcos(a):
    return D(math.cos(a.x), -math.sin(a.x) * a.d)


def dexp10(a):
    v = 10.0**a.x
    return D(v, v * math.log(10.0) * a.d)


def _seed(Xe, sX, mode, c, j_extra=False):
    """Newton-variation seeding for one element: returns ND lists of duals."""
    ND, nX = Xe.shape
    NJ = nX + (1 if mode == 2 else 0)
    out = []
    a = b = None
    if mode == 2:
        a = c["a2"] * Xe[1] + c["a3"] * Xe[2]
        b = c["b2"] * Xe[1] + c["b3"] * Xe[2]
    for d in range(ND):
        row = []
        for i in range(nX):
            g = np.zeros(NJ)
            if d == 0:
                g[i] = sX[i]
            elif mode in (2, 3):
                g[i] = (c["a1"] if d == 1 else c["b1"]) * sX[i]
                if mode == 2:
                    g[nX] = a[i] if d == 1 else b[i]
            row.append(D(Xe[d, i], g))
        out.append(row)
    return out, NJ


class _TestElement:
    @classmethod
    def oracle_residual(cls, g, dis_g, X, U, t, mode, c, sX):
        idx = dis_g.index_X - 1
        nele, nX = idx.shape
        Xe = np.stack([x[idx] for x in X], axis=1)
        Ue = U[0][dis_g.index_U - 1] if dis_g.index_U.size else np.zeros((nele, 0))
        A = np.zeros((nele, dis_g.index_A.shape[1]))
        params = [dict(zip(g.data[0].keys(), vals)) for vals in zip(*[g.cat(k) for k in g.data[0].keys()])]
        NJ = nX + (1 if mode == 2 else 0)
        R = np.zeros((nele, nX))
        J = np.zeros((nele, nX, NJ))
        for e in range(nele):
            Xd, _ = _seed(Xe[e], sX[e], mode, c)
            r = cls.residual(params[e], Xd, Ue[e], A[e], t)
            for i in range(nX):
                ri = r[i] if isinstance(r[i], D) else D.c(r[i], NJ)
                R[e, i] = ri.x * sX[e, i]
                J[e, i] = ri.d * sX[e, i]
        return R, J


class Turbine(_TestElement):
    """test/SomeElements.jl:15-28,54-56"""

    @staticmethod
    def doflist(key):
        return (1, 1, 2, 2), ("X", "X", "A", "A"), ("tx1", "tx2", "Δseadrag", "Δskydrag")

    @staticmethod
    def construct(model, nod, seadrag, sea, skydrag, sky):
        n = nod.shape[0]
        xm = np.stack([model.coord(int(i))[:2] for i in nod[:, 0]])
        return {"xm": xm, "seadrag": np.full(n, seadrag), "skydrag": np.full(n, skydrag),
                "sea": np.array([sea] * n, dtype=object), "sky": np.array([sky] * n, dtype=object)}, ("Turbine",)

    @staticmethod
    def residual(p, X, U, A, t):
        x = [X[0][i] + p["xm"][i] for i in range(2)]
        sea = p["sea"](t, x)
        sky = p["sky"](t, x)
        return [-sea[i] * p["seadrag"] * (1 + A[0]) - sky[i] * p["skydrag"] * (1 + A[1]) for i in range(2)]


_HORNER = [2.82040487827, -24.86027164695, 153.69500343165, -729.52107422849, 2458.11921356871,
           -5856.85610233072, 9769.49700812681, -11141.12651712473, 8260.66447746395, -3582.36704093187,
           687.83550335374]


def _horner(p, x):
    y = 0.0
    for i in reversed(p):
        y = i + x * y
    return y


class AnchorLine(_TestElement):
    """test/SomeElements.jl:60-94: R = ∂L/∂Λ = (Fd, m3)."""

    @staticmethod
    def doflist(key):
        return (1, 1, 1, 2, 2), ("X", "X", "X", "A", "A"), ("tx1", "tx2", "rx3", "ΔL", "Δbuoyancy")

    @staticmethod
    def construct(model, nod, Dxmtop, xmbot, L, buoyancy):
        n = nod.shape[0]
        xmtop = np.stack([model.coord(int(i)) for i in nod[:, 0]])
        return {"xmtop": xmtop, "Dxmtop": np.tile(np.asarray(Dxmtop, float), (n, 1)),
                "xmbot": np.tile(np.asarray(xmbot, float), (n, 1)), "L": np.full(n, L),
                "buoyancy": np.full(n, buoyancy)}, ("AnchorLine",)

    @staticmethod
    def residual(p, X, U, A, t):
        x = X[0]
        L = p["L"] * (1 + A[0])
        buoy = p["buoyancy"] * (1 + A[1])
        Xtop = [x[0] + p["xmtop"][0], x[1] + p["xmtop"][1], 0.0 + p["xmtop"][2]]
        alpha = x[2]
        cs, sn = dcos(alpha), dsin(alpha)
        dx = p["Dxmtop"]
        DXtop = [cs * dx[0] - sn * dx[1], sn * dx[0] + cs * dx[1], 0.0 * cs + dx[2]]
        DXchain = [Xtop[0] + DXtop[0] - p["xmbot"][0], Xtop[1] + DXtop[1] - p["xmbot"][1]]
        xaf = dsqrt(DXchain[0] * DXchain[0] + DXchain[1] * DXchain[1])
        z = Xtop[2] if isinstance(Xtop[2], D) else D.c(Xtop[2], len(xaf.d))
        cr = dexp10(_horner_d((L - xaf) / z)) * z
        Fh = -cr * buoy
        Fd = [DXchain[0] / xaf * Fh, DXchain[1] / xaf * Fh]
        m3 = DXtop[0] * Fd[1] - DXtop[1] * Fd[0]
        return [Fd[0], Fd[1], m3]


def _horner_d(x):
    y = D.c(0.0, len(x.d))
    for i in reversed(_HORNER):
        y = i + x * y
    return y


class SdofOscillator(_TestElement):
    """test/SomeElements.jl:193-207"""

    @staticmethod
    def doflist(key):
        return (1, 1), ("X", "U"), ("tx1", "tu1")

    @staticmethod
    def construct(model, nod, K1=0.0, K2=0.0, C1=0.0, C2=0.0, M1=0.0, M2=0.0):
        n = nod.shape[0]
        return {k: np.full(n, v) for k, v in dict(K1=K1, K2=K2, C1=C1, C2=C2, M1=M1, M2=M2).items()}, ("SdofOscillator",)

    @staticmethod
    def residual(p, X, U, A, t):
        x = X[0][0]
        x1 = X[1][0] if len(X) > 1 else 0.0
        x2 = X[2][0] if len(X) > 2 else 0.0
        u = U[0] if len(U) else 0.0
        return [-u + p["K1"] * x + p["K2"] * x * x + p["C1"] * x1 + p["C2"] * x1 * x1 + p["M1"] * x2 + p["M2"] * x2 * x2]
