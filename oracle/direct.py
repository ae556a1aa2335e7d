"""Oracle (test infrastructure only): CPU restatement of DirectXUA{OX,OU,IA}
(src/DirectXUA.jl), the all-steps-at-once Newton solver of optimisation FEM,
for models of elements that provide a full Lagrangian (no_second_order false).

Reference lines followed:
* AssemblyDirect, one step (src/DirectXUA.jl:18-151): gradient blocks
  L1[α][αder] and Hessian blocks L2[α,β][αder,βder] for α, β ∈ (Λ, X, U, A)
  and the time-derivative orders (1, OX+1, OU+1, IA); L2[Λ,Λ] is empty.  Each
  element's Lagrangian is differentiated twice over its variables laid out
  (Λ, X⁽⁰⁾..X⁽ᴼˣ⁾, U⁽⁰⁾..U⁽ᴼᵘ⁾, A) (revariate{2}, :152-171 and
  DirectXUA_lagrangian_addition!, :122-151): residual elements give
  L = Λ·R (getlagrangian of a residual element), cost elements their cost.
  The per-step assembly is not scaled by the step (assemble! with idmult,
  :331).  A-costs are added once by assembleA! (:67-80 and
  src/Assemble.jl:507-520) and, through the generic element path, once more
  in every step: the method that would skip them in assemble! takes a single
  Acost element (src/Assemble.jl:477), while assemble! passes the vector of a
  type's elements, so it never applies.  The reference's golden values
  (test/TestDirectXUA001.jl) carry that weighting, nstep + 1 A-costs.
* The big system (assemblebig!, :317-356): blocks (Λ, X, U) of every step in
  step order, then one A block; gradient entry αder of step s goes to the
  blocks of steps s+Δs with weight w·Δt^(1−αder), Hessian entries with
  w_α w_β Δt^(2−αder−βder), (Δs, w) the finite-difference kernels of
  src/FiniteDifferences.jl:2-31 (one-sided at the ends, centred inside).
* Newton (solve, :438-513): LU solve of the big system (SuperLU here, UMFPACK
  in the reference), decrement of every step's Λ, X, U derivatives through the
  same kernels and of the shared A (decrementbig!, :357-383), convergence when
  every class's largest squared block decrement is below maxΔ².

Elements with no second order (EulerBeam3D, Bar3D) take another path in the
reference (:85-120: Lλ and the Λ-cross blocks only, no (∂R/∂X)ᵀΛ in Lx);
static_path_without_second_order restates its iterations for beam models
observed by quadratic sensor costs, where the multipliers never settle.

Pinned by test/TestDirectXUA001.jl:33-51 (golden X and A of the static
identification with springs, rtol 1e-4), by the step blocks L1/L2 of
test/TestDirectXUA.jl:93-108 and by the big-system pattern of
test/TestDirectXUA.jl:109-136 (tests/test_direct_oracle.py).
"""
from __future__ import annotations

import math

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla

from muscade_gpu.elements import group_time_values


# --------------------------------------------------------------- second-order duals
class D2:
    """Value, gradient and Hessian over n variables (forward mode, second order)."""

    __slots__ = ("v", "g", "h")

    def __init__(self, v, g, h):
        self.v = float(v)
        self.g = g
        self.h = h

    @staticmethod
    def var(v, i, n):
        g = np.zeros(n)
        g[i] = 1.0
        return D2(v, g, np.zeros((n, n)))

    @staticmethod
    def const(v, n):
        return D2(v, np.zeros(n), np.zeros((n, n)))

    def _w(self, o):
        return o if isinstance(o, D2) else D2.const(o, len(self.g))

    def compose(self, f0, f1, f2):
        """f(self) from f, f′, f″ at self.v"""
        return D2(f0, f1 * self.g, f1 * self.h + f2 * np.outer(self.g, self.g))

    def __add__(self, o):
        o = self._w(o)
        return D2(self.v + o.v, self.g + o.g, self.h + o.h)

    __radd__ = __add__

    def __sub__(self, o):
        o = self._w(o)
        return D2(self.v - o.v, self.g - o.g, self.h - o.h)

    def __rsub__(self, o):
        return self._w(o) - self

    def __neg__(self):
        return D2(-self.v, -self.g, -self.h)

    def __mul__(self, o):
        if not isinstance(o, D2):
            return D2(self.v * o, self.g * o, self.h * o)
        og = np.outer(self.g, o.g)
        return D2(self.v * o.v, self.g * o.v + self.v * o.g, self.h * o.v + self.v * o.h + og + og.T)

    __rmul__ = __mul__

    def __truediv__(self, o):
        if not isinstance(o, D2):
            return self * (1.0 / o)
        return self * o.compose(1.0 / o.v, -1.0 / o.v**2, 2.0 / o.v**3)

    def __rtruediv__(self, o):
        return self._w(o) / self

    def __pow__(self, k):
        if k == 2:
            return self * self
        return self.compose(self.v**k, k * self.v ** (k - 1), k * (k - 1) * self.v ** (k - 2))


def d2sqrt(a):
    s = math.sqrt(a.v)
    return a.compose(s, 0.5 / s, -0.25 / (s * a.v))


def d2exp10(a):
    c = math.log(10.0)
    e = 10.0**a.v
    return a.compose(e, c * e, c * c * e)


# --------------------------------------------------------------- elements
class Spring:
    """Spring{D}: test/SomeElements.jl:164-188.  X: the D translations of its two
    nodes; A: ΞL₀, ΞEI on a third node (rest length L·10^ΞL₀, stiffness EA·10^ΞEI)."""

    @staticmethod
    def doflist(key):
        D = key[1]
        return ((1,) * D + (2,) * D + (3, 3), ("X",) * (2 * D) + ("A", "A"),
                tuple(f"tx{i}" for i in range(1, D + 1)) * 2 + ("ΞL₀", "ΞEI"))

    @staticmethod
    def construct(model, nod, EA, D=2):
        n = nod.shape[0]
        x1 = np.stack([model.coord(int(i))[:D] for i in nod[:, 0]])
        x2 = np.stack([model.coord(int(i))[:D] for i in nod[:, 1]])
        L = np.sqrt(np.sum((x1 - x2) ** 2, axis=1))
        return {"x1": x1, "x2": x2, "EA": np.full(n, float(EA)), "L": L}, ("Spring", D)

    @staticmethod
    def residual(p, X, U, A, t):
        D = len(p["x1"])
        L0 = p["L"] * d2exp10(A[0]) if isinstance(A[0], D2) else p["L"] * 10.0 ** A[0]
        EA = p["EA"] * d2exp10(A[1]) if isinstance(A[1], D2) else p["EA"] * 10.0 ** A[1]
        x1 = [X[0][i] + p["x1"][i] for i in range(D)]
        x2 = [X[0][D + i] + p["x2"][i] for i in range(D)]
        dx = [x1[i] - x2[i] for i in range(D)]
        s2 = dx[0] * dx[0]
        for i in range(1, D):
            s2 = s2 + dx[i] * dx[i]
        L = d2sqrt(s2)
        T = EA * (L - L0) / L0
        F1 = [dx[i] / L * T for i in range(D)]
        return F1 + [-f for f in F1]


class El1:
    """El1 of test/TestDirectXUA.jl:9-20: r = −u + K x + C·10^ΞC x′ + M·10^ΞM x″."""

    @staticmethod
    def doflist(key):
        return (1, 1, 1, 1), ("X", "U", "A", "A"), ("tx1", "u", "ΞC", "ΞM")

    @staticmethod
    def construct(model, nod, K, C, M):
        n = nod.shape[0]
        return {"K": np.full(n, float(K)), "C": np.full(n, float(C)), "M": np.full(n, float(M))}, ("El1",)

    @staticmethod
    def residual(p, X, U, A, t):
        x = X[0][0]
        x1 = X[1][0] if len(X) > 1 else 0.0
        x2 = X[2][0] if len(X) > 2 else 0.0
        return [-U[0][0] + p["K"] * x + p["C"] * d2exp10(A[0]) * x1 + p["M"] * d2exp10(A[1]) * x2]


class SingleDofCost:
    """SingleDofCost (src/BasicElements.jl:198-208 through DofCost :32-50):
    L = cost(x⁽ᵈ⁾, t) on one X- or U-dof."""

    @staticmethod
    def doflist(key):
        return (1,), (key[1],), (key[2],)

    @staticmethod
    def construct(model, nod, cls, field, cost, derivative=0):
        return {"cost": [cost], "n": np.full(nod.shape[0], 1)}, ("SingleDofCost", cls, field, derivative,
                                                                  getattr(cost, "__qualname__", repr(cost)))

    @staticmethod
    def lagrangian(p, key, Lam, X, U, A, t):
        d = key[3]
        v = (X if key[1] == "X" else U)[d][0]
        return p["cost"](v, t)


class SingleUdof:
    """SingleUdof (src/BasicElements.jl:223-248): a U-dof loading the X-dof of
    the same node, L = cost(u, t) − λ u with λ the X-dof's multiplier."""

    @staticmethod
    def doflist(key):
        return (1, 1), ("X", "U"), (key[1], key[2])

    @staticmethod
    def construct(model, nod, Xfield, Ufield, cost):
        return {"cost": [cost], "n": np.full(nod.shape[0], 1)}, ("SingleUdof", Xfield, Ufield,
                                                                  getattr(cost, "__qualname__", repr(cost)))

    @staticmethod
    def lagrangian(p, key, Lam, X, U, A, t):
        u = U[0][0]
        return p["cost"](u, t) - Lam[0] * u


class SingleAcost:
    """SingleAcost (src/BasicElements.jl:130-167 through Acost :77-86): a once-off
    cost on one A-dof, added by assembleA!."""

    @staticmethod
    def doflist(key):
        return (1,), ("A",), (key[1],)

    @staticmethod
    def construct(model, nod, field, cost):
        return {"cost": [cost], "n": np.full(nod.shape[0], 1)}, ("SingleAcost", field,
                                                                 getattr(cost, "__qualname__", repr(cost)))

    @staticmethod
    def acost(p, A):
        return p["cost"](A[0])

    @staticmethod
    def lagrangian(p, key, Lam, X, U, A, t):
        return p["cost"](A[0])


# the cost elements restated here, by element kind: a model built with the
# package's own SingleDofCost / SingleUdof / SingleAcost (same keys and data)
# is evaluated by these restatements, not by the package's classes
COST_ELEMENTS = {"SingleDofCost": SingleDofCost, "SingleUdof": SingleUdof, "SingleAcost": SingleAcost}


def _params(g):
    """Per-element parameter dicts of a group (the fields of its batches in order)."""
    out = []
    for d, nodes in zip(g.data, g.nodes):
        n = nodes.shape[0]
        for e in range(n):
            out.append({k: (v[0] if isinstance(v, list) else v[e]) for k, v in d.items()})
    return out


# --------------------------------------------------------------- one step
class Layout:
    """Variable layout of one element: Λ (nx), X orders, U orders, A (if IA)."""

    def __init__(self, nx, nu, na, OX, OU, IA):
        self.nx, self.nu, self.na = nx, nu, na
        self.nder = {"L": 1, "X": OX + 1, "U": OU + 1, "A": IA}
        self.size = {"L": nx, "X": nx, "U": nu, "A": na}
        self.off = {}
        p = 0
        for a in ("L", "X", "U", "A"):
            for i in range(self.nder[a]):
                self.off[(a, i)] = p
                p += self.size[a]
        self.n = p


CLASSES = ("L", "X", "U", "A")


def _group_kind(g):
    return g.key[0]


def element_lagrangian(g, key, p, Lam, Xe, Ue, Ae, t, lay):
    """D2 Lagrangian of one element over its layout's variables."""
    n = lay.n
    var = lambda a, i, j, val: D2.var(val, lay.off[(a, i)] + j, n)  # noqa: E731
    L = [var("L", 0, j, Lam[j]) for j in range(lay.nx)]
    X = [[var("X", i, j, Xe[i][j]) for j in range(lay.nx)] for i in range(lay.nder["X"])]
    U = [[var("U", i, j, Ue[i][j]) for j in range(lay.nu)] for i in range(lay.nder["U"])]
    if lay.nder["A"]:
        A = [var("A", 0, j, Ae[j]) for j in range(lay.na)]
    else:
        A = [D2.const(a, n) for a in Ae]
    kind = _group_kind(g)
    if kind == "DofLoad":
        R = [D2.const(-float(p["F"]), n)]
    elif kind == "DofConstraint":
        nx = lay.nx - 1
        c = p["coeffs"]
        gap = D2.const(-float(p["off"]), n)
        for i in range(nx):
            gap = gap + c[i] * X[0][i]
        R = [-c[i] * X[0][nx] for i in range(nx)] + [-gap]
    elif kind in COST_ELEMENTS:
        return COST_ELEMENTS[kind].lagrangian(p, key, L, X, U, A, t)
    elif hasattr(g.etype, "residual"):
        R = g.etype.residual(p, X, U, A, t)
    else:
        return g.etype.lagrangian(p, key, L, X, U, A, t)
    out = D2.const(0.0, n)
    for i, r in enumerate(R):
        out = out + L[i] * r
    return out


def assemble_step(model, dis, Lam, X, U, A, t, OX, OU, IA):
    """AssemblyDirect of one step: L1[α][i] (vectors) and L2[(α,β)][(i,j)]
    (dense matrices), α over Λ ('L'), X, U, A; Λ uses the X numbering."""
    n = {"L": model.ndof["X"], "X": model.ndof["X"], "U": model.ndof["U"], "A": model.ndof["A"]}
    nder = {"L": 1, "X": OX + 1, "U": OU + 1, "A": IA}
    L1 = {a: [np.zeros(n[a]) for _ in range(nder[a])] for a in CLASSES}
    L2 = {}
    for a in CLASSES:
        for b in CLASSES:
            if a == b == "L":
                continue
            for i in range(nder[a]):
                for j in range(nder[b]):
                    L2[(a, b, i, j)] = np.zeros((n[a], n[b]))
    for g, dg in zip(model.groups, dis.dis):
        if g.nele == 0:
            continue
        ix, iu, ia = dg.index_X - 1, dg.index_U - 1, dg.index_A - 1
        lay = Layout(ix.shape[1], iu.shape[1] if iu.ndim == 2 else 0, ia.shape[1] if ia.ndim == 2 else 0, OX, OU, IA)
        params = _params(g)
        kind = _group_kind(g)
        tv = None
        if kind == "DofLoad":
            tv = group_time_values(g, "value", t)
        elif kind == "DofConstraint":
            tv = group_time_values(g, "offset", t)
            co = g.cat("coeffs")
        for e in range(g.nele):
            p = params[e]
            if kind == "DofLoad":
                p = {"F": tv[e]}
            elif kind == "DofConstraint":
                p = {"off": tv[e], "coeffs": co[e]}
            Le = element_lagrangian(g, g.key, p, Lam[ix[e]], [x[ix[e]] for x in X],
                                    [u[iu[e]] if lay.nu else np.zeros(0) for u in U],
                                    A[ia[e]] if lay.na else np.zeros(0), t, lay)
            glob = {"L": ix[e], "X": ix[e], "U": iu[e] if lay.nu else np.zeros(0, int),
                    "A": ia[e] if lay.na else np.zeros(0, int)}
            for a in CLASSES:
                for i in range(nder[a]):
                    if lay.size[a] == 0:
                        continue
                    oa = lay.off[(a, i)]
                    np.add.at(L1[a][i], glob[a], Le.g[oa:oa + lay.size[a]])
                    for b in CLASSES:
                        if a == b == "L" or lay.size[b] == 0:
                            continue
                        for j in range(nder[b]):
                            ob = lay.off[(b, j)]
                            blk = Le.h[oa:oa + lay.size[a], ob:ob + lay.size[b]]
                            np.add.at(L2[(a, b, i, j)], (glob[a][:, None], glob[b][None, :]), blk)
    return L1, L2


def assemble_A(model, dis, A):
    """assembleA!: the once-off A-costs, gradient and Hessian over the A-dofs."""
    nA = model.ndof["A"]
    g1, h1 = np.zeros(nA), np.zeros((nA, nA))
    for g, dg in zip(model.groups, dis.dis):
        if _group_kind(g) != "SingleAcost":
            continue
        ia = dg.index_A - 1
        for e, p in enumerate(_params(g)):
            na = ia.shape[1]
            a = [D2.var(A[ia[e, j]], j, na) for j in range(na)]
            c = SingleAcost.acost(p, a)
            np.add.at(g1, ia[e], c.g)
            np.add.at(h1, (ia[e][:, None], ia[e][None, :]), c.h)
    return g1, h1


# --------------------------------------------------------------- all steps
KERNELS = [[[(0, 1.0)]],
           [[(0, -1.0), (1, 1.0)], [(-1, -1.0), (0, 1.0)], [(-1, -0.5), (1, 0.5)]],
           [[(0, 1.0), (1, -2.0), (2, 1.0)], [(-2, 1.0), (-1, -2.0), (0, 1.0)], [(-1, 1.0), (0, -2.0), (1, 1.0)]]]


def finitediff(order, n, s):
    """finitediff (src/FiniteDifferences.jl:8-31), s 1-based."""
    if order > 0 and n < 6:
        raise ValueError("Number of steps must be ≥6")
    if order == 0:
        return KERNELS[0][0]
    return KERNELS[order][0 if s == 1 else 1 if s == n else 2]


class DirectState:
    def __init__(self, t, Lam, X, U):
        self.time, self.Lam, self.X, self.U = t, Lam, X, U


def directxua(model, dis, initialstate, time, OX, OU, IA, maxiter=50, maxdl=1e-5, maxdx=1e-5, maxdu=1e-5,
              maxda=1e-5):
    """solve(DirectXUA{OX,OU,IA}) for one experiment on a uniform time grid.
    Returns (states, A, iterations): states[istep] with .Lam, .X (orders), .U (orders)."""
    time = np.asarray(time, dtype=float)
    nstep = len(time)
    dt = float(time[1] - time[0]) if nstep > 1 else 1.0
    nX, nU, nA = model.ndof["X"], model.ndof["U"], model.ndof["A"]
    nder = {"L": 1, "X": OX + 1, "U": OU + 1, "A": IA}
    size = {"L": nX, "X": nX, "U": nU}

    def orders(vs, nd, k):  # the state's derivatives, zeros for those it lacks
        return [np.array(vs[i], dtype=float) if i < len(vs) else np.zeros(k) for i in range(nd)]

    lam0 = initialstate.L[0] if len(initialstate.L) else np.zeros(nX)
    states = [DirectState(t, np.array(lam0, dtype=float), orders(initialstate.X, OX + 1, nX),
                          orders(initialstate.U, OU + 1, nU)) for t in time]
    A = np.array(initialstate.A, dtype=float)
    # block offsets: (λ, x, u) per step, then A
    bsize = [size[c] for _ in range(nstep) for c in ("L", "X", "U")] + ([nA] if IA else [])
    boff = np.concatenate([[0], np.cumsum(bsize)])
    N = int(boff[-1])
    ablk = 3 * nstep

    def blk(istep, c):  # istep 1-based
        return 3 * (istep - 1) + {"L": 0, "X": 1, "U": 2}[c]

    for it in range(1, maxiter + 1):
        Lv = np.zeros(N)
        Lvv = np.zeros((N, N))
        if IA:
            gA, hA = assemble_A(model, dis, A)
            Lv[boff[ablk]:boff[ablk + 1]] += gA
            Lvv[boff[ablk]:boff[ablk + 1], boff[ablk]:boff[ablk + 1]] += hA
        classes = CLASSES if IA else ("L", "X", "U")
        for s, st in enumerate(states, start=1):
            L1, L2 = assemble_step(model, dis, st.Lam, st.X, st.U, A, st.time, OX, OU, IA)
            for b in classes:
                for bder in range(nder[b]):
                    w_s = dt ** (-bder)
                    for (ds, w) in (finitediff(bder, nstep, s) if b != "A" else [(0, 1.0)]):
                        bb = ablk if b == "A" else blk(s + ds, b)
                        Lv[boff[bb]:boff[bb + 1]] += w * w_s * L1[b][bder]
            for (a, b, i, j), M in L2.items():
                if a not in classes or b not in classes:
                    continue
                w_s = dt ** (-i - j)
                for (dsa, wa) in (finitediff(i, nstep, s) if a != "A" else [(0, 1.0)]):
                    for (dsb, wb) in (finitediff(j, nstep, s) if b != "A" else [(0, 1.0)]):
                        ba = ablk if a == "A" else blk(s + dsa, a)
                        bb = ablk if b == "A" else blk(s + dsb, b)
                        Lvv[boff[ba]:boff[ba + 1], boff[bb]:boff[bb + 1]] += wa * wb * w_s * M
        K = sp.csc_matrix(Lvv)
        try:
            dv = spla.splu(K).solve(Lv)
        except RuntimeError as e:
            raise RuntimeError("Lvv matrix factorization failed") from e
        d2 = {"L": 0.0, "X": 0.0, "U": 0.0, "A": 0.0}
        for s, st in enumerate(states, start=1):
            for b in ("L", "X", "U"):
                for bder in range(nder[b]):
                    w_s = dt ** (-bder)
                    for (ds, w) in finitediff(bder, nstep, s):
                        bb = blk(s + ds, b)
                        D = dv[boff[bb]:boff[bb + 1]]
                        if b == "L":
                            st.Lam = st.Lam - D * w * w_s
                        elif b == "X":
                            st.X[bder] = st.X[bder] - D * w * w_s
                        else:
                            st.U[bder] = st.U[bder] - D * w * w_s
                        if bder == 0:
                            d2[b] = max(d2[b], float(np.sum(D**2)))
        if IA:
            Da = dv[boff[ablk]:boff[ablk + 1]]
            d2["A"] = float(np.sum(Da**2))
            A = A - Da
        lim = {"L": maxdl, "X": maxdx, "U": maxdu, "A": maxda}
        if all(d2[c] <= lim[c] ** 2 for c in ("L", "X", "U", "A")):
            return states, A, it
    raise RuntimeError(f"no convergence after {maxiter} iterations")


# --------------------------------------------------------------- big-system pattern
def big_pattern(model, dis, OX, OU, IA, nstep):
    """makepattern + preparebig (src/DirectXUA.jl:245-300, src/SparseTools.jl:32-120):
    the CSC pattern of the all-steps matrix Lvv and the first entry of every
    block of Lv (1-based, like colptr/rowval and Lvasm).  A block (α, β) of a
    step holds the pairs of element dofs of classes α and β (Λ-dofs are the
    element's X-dofs), whatever the time-derivative orders that reach it."""
    n = {"L": model.ndof["X"], "X": model.ndof["X"], "U": model.ndof["U"], "A": model.ndof["A"]}
    nder = {"L": 1, "X": OX + 1, "U": OU + 1, "A": IA}
    pats = {}
    for a in CLASSES:
        for b in CLASSES:
            pats[(a, b)] = set()
    for g, dg in zip(model.groups, dis.dis):
        dofs = {"X": dg.index_X - 1, "U": dg.index_U - 1, "A": dg.index_A - 1}
        dofs["L"] = dofs["X"]
        for e in range(g.nele):
            for a in CLASSES:
                da = dofs[a][e] if dofs[a].ndim == 2 else ()
                for b in CLASSES:
                    db = dofs[b][e] if dofs[b].ndim == 2 else ()
                    pats[(a, b)].update((int(i), int(j)) for i in da for j in db)
    blocks = {}  # (block row, block col) -> pattern
    bs = {}  # block sizes
    for s in range(1, nstep + 1):
        for a in ("L", "X", "U"):
            for b in ("L", "X", "U"):
                if a == b == "L":
                    continue
                for i in range(nder[a]):
                    for j in range(nder[b]):
                        for (dsa, _) in finitediff(i, nstep, s):
                            for (dsb, _) in finitediff(j, nstep, s):
                                ba = 3 * (s + dsa - 1) + "LXU".index(a)
                                bb = 3 * (s + dsb - 1) + "LXU".index(b)
                                blocks[(ba, bb)] = pats[(a, b)]
                                bs[ba], bs[bb] = n[a], n[b]
    if IA:
        ab = 3 * nstep
        blocks[(ab, ab)] = pats[("A", "A")]
        bs[ab] = n["A"]
        for s in range(1, nstep + 1):
            for a in ("L", "X", "U"):
                blocks[(ab, 3 * (s - 1) + "LXU".index(a))] = pats[("A", a)]
                blocks[(3 * (s - 1) + "LXU".index(a), ab)] = pats[(a, "A")]
    nb = max(bs) + 1
    off = np.concatenate([[0], np.cumsum([bs[i] for i in range(nb)])])
    cols = [[] for _ in range(int(off[-1]))]
    for (ba, bb), P in blocks.items():
        for (i, j) in P:
            cols[off[bb] + j].append(off[ba] + i)
    colptr = [1]
    rowval = []
    for c in cols:
        rowval += [r + 1 for r in sorted(c)]
        colptr.append(len(rowval) + 1)
    return np.array(colptr), np.array(rowval), off[:-1] + 1


# --------------------------------------------------------------- elements without second order
def static_path_without_second_order(model, dis, initialstate, times, sensors, y, niter):
    """The reference's DirectXUA{0,0,0} iterations for residual elements with
    no_second_order (EulerBeam3D: toolbox/BeamElement.jl:106) observed by
    quadratic sensor costs Σ (x[d] − y)²: such elements add Lλ = R and the
    cross blocks Lλx = ∂R/∂X, Lxλ = (∂R/∂X)ᵀ (src/DirectXUA.jl:85-120) but no
    (∂R/∂X)ᵀΛ to Lx, so Lx is the costs' gradient alone.  Returns the largest
    |ΔΛ| and |ΔX| over the steps, per Newton iteration."""
    from . import reference as REF

    prep = REF.Prepared(model, dis)
    n = prep.n
    sens = np.asarray(sensors) - 1
    c0 = REF.newmark_coefficients(0, 1.0, 0.25, 0.5)
    X = [initialstate.X[0].copy() for _ in times]
    Lam = [np.zeros(n) for _ in times]
    out = []
    for _ in range(niter):
        blocks, rhs = [], []
        for k, t in enumerate(times):
            R, nz = REF.assemble(prep, (X[k],), (np.zeros(model.ndof["U"]),), t, "static", c0, A=initialstate.A)
            K = prep.matrix(nz)
            g, h = np.zeros(n), np.zeros(n)
            np.add.at(g, sens, 2.0 * (X[k][sens] - y[k]))
            np.add.at(h, sens, 2.0)
            rhs += [R, g]
            blocks.append(sp.bmat([[None, K], [K.T, sp.diags(h)]], format="csc"))
        dv = spla.splu(sp.block_diag(blocks, format="csc")).solve(np.concatenate(rhs))
        dl = dx = 0.0
        for k in range(len(times)):
            d_l, d_x = dv[2 * k * n:(2 * k + 1) * n], dv[(2 * k + 1) * n:(2 * k + 2) * n]
            Lam[k] -= d_l
            X[k] -= d_x
            dl, dx = max(dl, float(np.linalg.norm(d_l))), max(dx, float(np.linalg.norm(d_x)))
        out.append((dl, dx))
    return out
