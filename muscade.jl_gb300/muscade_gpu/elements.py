"""Element types of the GPU path, restating the reference's constructors and doflists.

Each element class provides
  construct(model, nod, **kwargs) -> (data: dict of per-element arrays, key: tuple)
  doflist(key) -> (inod, class, field)       (ElementAPI `doflist`)
The `key` plays the role of the reference's concrete element type: elements
with equal keys form one element group (ModelDescription.jl:198-208).

* EulerBeam3D          toolbox/BeamElement.jl:6-25 (BeamCrossSection), :109-148
* Bar3D                toolbox/BarElement.jl:36-48, :107-133
* Hold                 src/BasicElements.jl:484-488  (DofConstraint{:X} with gap x)
* DofConstraint        src/BasicElements.jl:406-438  (λclass :X, equal mode, affine gap)
* DofLoad              src/BasicElements.jl:275-284
* SingleDofCost        src/BasicElements.jl:198-208 (through DofCost :32-50)
* SingleUdof           src/BasicElements.jl:239-248
* SingleAcost          src/BasicElements.jl:163-167 (through Acost :77-86)
* QuadraticCost        the cost functor form the GPU path evaluates
"""
from __future__ import annotations

import math

import numpy as np

from .model import MuscadeError

BEAM_NDATA = 69  # EulerBeam3D fields flattened in declaration order
BAR_NDATA = 38  # Bar3D fields flattened in declaration order

BEAM_MAT_FIELDS = ("EA", "EI2", "EI3", "GJ", "mu", "iota1", "w", "Ca1", "Cl1", "Cq1", "Ca2", "Cl2", "Cq2", "Ca3", "Cl3", "Cq3")
BAR_MAT_FIELDS = ("EA", "mu", "w", "Cat", "Clt", "Cqt", "Can", "Cln", "Cqn")


class BeamCrossSection:
    """BeamCrossSection (BeamElement.jl:6-25).  Fields may be scalars or per-element arrays."""

    def __init__(self, EA, EI2, EI3, GJ, mu, iota1, w=0.0, Ca1=0.0, Cl1=0.0, Cq1=0.0, Ca2=0.0, Cl2=0.0, Cq2=0.0,
                 Ca3=0.0, Cl3=0.0, Cq3=0.0):
        loc = locals()
        self.values = {k: loc[k] for k in BEAM_MAT_FIELDS}

    def array(self, n):
        return np.stack([np.broadcast_to(np.asarray(self.values[k], dtype=np.float64), (n,)) for k in BEAM_MAT_FIELDS], axis=1)


class AxisymmetricBarCrossSection:
    """AxisymmetricBarCrossSection (BarElement.jl:36-48)."""

    def __init__(self, EA, mu, w=0.0, Cat=0.0, Clt=0.0, Cqt=0.0, Can=0.0, Cln=0.0, Cqn=0.0):
        loc = locals()
        self.values = {k: loc[k] for k in BAR_MAT_FIELDS}

    def array(self, n):
        return np.stack([np.broadcast_to(np.asarray(self.values[k], dtype=np.float64), (n,)) for k in BAR_MAT_FIELDS], axis=1)


def _coords(model, nod, col):
    return np.stack([model.coord(int(i)) for i in nod[:, col]]).astype(np.float64)


class EulerBeam3D:
    """Corotational 3D Euler beam, 2 nodes, 12 X-dofs (+3 U-dofs when `udof`).

    With `adof`, the element also has one A-dof, field "EIscale", on its last
    node (node 3, or node 4 with `udof`): a factor on both bending stiffnesses
    EI2 and EI3.  The reference's EulerBeam3D has no A-dofs
    (toolbox/BeamElement.jl:109-118); this wrapper gives the stiffness
    identification problem its parameters.  Its value is the factor itself, so
    a State built by initialize() (A = 0) must have A set before solving.
    """

    @staticmethod
    def doflist(key):
        udof = key[1]
        adof = len(key) > 2 and key[2]
        inod = (1, 1, 1, 1, 1, 1, 2, 2, 2, 2, 2, 2) + ((3, 3, 3) if udof else ())
        cls = ("X",) * 12 + (("U",) * 3 if udof else ())
        fld = ("t1", "t2", "t3", "r1", "r2", "r3") * 2 + (("t1", "t2", "t3") if udof else ())
        if adof:
            inod += (4 if udof else 3,)
            cls += ("A",)
            fld += ("EIscale",)
        return inod, cls, fld

    @staticmethod
    def construct(model, nod, mat: BeamCrossSection, orient2=(0.0, 1.0, 0.0), udof=False, adof=False):
        n = nod.shape[0]
        c1 = _coords(model, nod, 0)
        c2 = _coords(model, nod, 1)
        o2 = np.broadcast_to(np.asarray(orient2, dtype=np.float64), (n, 3)).copy()
        ele = beam_fields(c1, c2, o2, mat.array(n))
        key = ("EulerBeam3D", bool(udof), True) if adof else ("EulerBeam3D", bool(udof))
        return {"ele": ele}, key


def beam_fields(c1, c2, orient2, mat):
    """EulerBeam3D constructor (BeamElement.jl:122-148), vectorised over elements."""
    n = c1.shape[0]
    cm = (c1 + c2) / 2
    tgm = c2 - c1
    L = np.sqrt(np.sum(tgm * tgm, axis=1))
    t = tgm / L[:, None]
    o2 = orient2 / np.sqrt(np.sum(orient2 * orient2, axis=1))[:, None]
    nv = o2 - t * np.sum(o2 * t, axis=1)[:, None]
    nn = np.sqrt(np.sum(nv * nv, axis=1))
    if np.any(~(nn > 1e-3)):
        raise MuscadeError("Provide a 'orient' input that is not nearly parallel to the element")
    nv = nv / nn[:, None]
    b = np.cross(t, nv)
    rm = np.concatenate([t, nv, b], axis=1)  # column-major 3x3
    tge = np.zeros((n, 3))
    tge[:, 0] = L
    s30 = math.sqrt(30.0)
    dL = np.stack([L / 2 * (18 - s30) / 36, L / 2 * (18 + s30) / 36, L / 2 * (18 + s30) / 36, L / 2 * (18 - s30) / 36], axis=1)
    s65 = math.sqrt(6 / 5)
    zgp = np.array([-1 / 2 * math.sqrt(3 / 7 + 2 / 7 * s65), -1 / 2 * math.sqrt(3 / 7 - 2 / 7 * s65),
                    +1 / 2 * math.sqrt(3 / 7 - 2 / 7 * s65), +1 / 2 * math.sqrt(3 / 7 + 2 / 7 * s65)])
    znod = np.array([-0.5, 0.5])
    ya = np.broadcast_to(2 * zgp, (n, 4))
    yu = np.broadcast_to(-4 * zgp**3 + 3 * zgp, (n, 4))
    yv = (zgp**2 - 1 / 4)[None, :] * L[:, None]
    ka = np.broadcast_to(2.0, (n, 4)) / L[:, None]
    ku = (-24 * zgp)[None, :] / (L**2)[:, None]
    kv = np.broadcast_to(2.0, (n, 4)) / L[:, None]
    out = np.concatenate([cm, rm, np.broadcast_to(zgp, (n, 4)), np.broadcast_to(znod, (n, 2)), tgm, tge,
                          ya, yu, yv, ka, ku, kv, L[:, None], dL, mat], axis=1)
    assert out.shape[1] == 69
    return np.ascontiguousarray(out)


class Bar3D:
    """3D bar, 2 nodes, 6 X-dofs (+3 U-dofs when `udof`)."""

    @staticmethod
    def doflist(key):
        udof = key[1]
        inod = (1, 1, 1, 2, 2, 2) + ((3, 3, 3) if udof else ())
        cls = ("X",) * 6 + (("U",) * 3 if udof else ())
        fld = ("t1", "t2", "t3") * 2 + (("t1", "t2", "t3") if udof else ())
        return inod, cls, fld

    @staticmethod
    def construct(model, nod, mat: AxisymmetricBarCrossSection, epss=np.finfo(np.float64).eps, udof=False):
        n = nod.shape[0]
        c1 = _coords(model, nod, 0)
        c2 = _coords(model, nod, 1)
        cm = (c1 + c2) / 2
        tgm = c2 - c1
        L0 = np.sqrt(np.sum(tgm * tgm, axis=1))
        Ls = (1 - epss) * L0
        tge = np.zeros((n, 3))
        tge[:, 0] = L0
        s30 = math.sqrt(30.0)
        s65 = math.sqrt(6 / 5)
        wgp = np.stack([L0 / 2 * (18 - s30) / 36, L0 / 2 * (18 + s30) / 36, L0 / 2 * (18 + s30) / 36, L0 / 2 * (18 - s30) / 36], axis=1)
        zgp = np.array([-1 / 2 * math.sqrt(3 / 7 + 2 / 7 * s65), -1 / 2 * math.sqrt(3 / 7 - 2 / 7 * s65),
                        +1 / 2 * math.sqrt(3 / 7 - 2 / 7 * s65), +1 / 2 * math.sqrt(3 / 7 + 2 / 7 * s65)])
        psi1 = -zgp + 1 / 2
        psi2 = zgp + 1 / 2
        out = np.concatenate([cm, tgm, tge, L0[:, None], Ls[:, None], mat.array(n), wgp,
                              np.broadcast_to(zgp, (n, 4)), np.broadcast_to([-0.5, 0.5], (n, 2)),
                              np.broadcast_to(psi1, (n, 4)), np.broadcast_to(psi2, (n, 4))], axis=1)
        assert out.shape[1] == 38
        return {"ele": np.ascontiguousarray(out)}, ("Bar3D", bool(udof))


class DofConstraint:
    """Physical equality constraint on X-dofs with an affine gap g(x,t) = Σ aᵢ xᵢ − c(t).

    The reference's DofConstraint{:X} accepts any gap functor (BasicElements.jl:406-438);
    the GPU path supports the affine gaps that Hold and prescribed motions use.
    `offset(t)` returns c(t) for the elements of the batch (scalar or array).
    """

    @staticmethod
    def doflist(key):
        _, xinod, xfield, linod, lfield, _ = key
        return tuple(xinod) + (linod,), ("X",) * (len(xinod) + 1), tuple(xfield) + (lfield,)

    @staticmethod
    def construct(model, nod, xinod, xfield, lfield, coeffs=None, offset=None, linod=1, name="gap"):
        n = nod.shape[0]
        nx = len(xinod)
        a = np.ones((n, nx)) if coeffs is None else np.broadcast_to(np.asarray(coeffs, dtype=np.float64), (n, nx)).copy()
        return {"coeffs": a, "offset": [offset] * 1, "n": np.full(n, 1)}, ("DofConstraint", tuple(xinod), tuple(xfield), linod, lfield, name)


class Hold:
    """Hold: sets one X-dof to zero through a Lagrange multiplier (BasicElements.jl:484-488)."""

    doflist = DofConstraint.doflist

    @staticmethod
    def construct(model, nod, field, lfield=None):
        lfield = lfield or ("λ" + field)
        data, _ = DofConstraint.construct(model, nod, (1,), (field,), lfield, coeffs=[1.0], offset=None, name="hold")
        return data, ("DofConstraint", (1,), (field,), 1, lfield, "hold")


class DofLoad:
    """DofLoad: R = −F(t) on one X-dof (BasicElements.jl:275-284).

    `value(t)` returns the load of the batch's elements at time t (scalar or array).
    """

    @staticmethod
    def doflist(key):
        return (1,), ("X",), (key[1],)

    @staticmethod
    def construct(model, nod, field, value):
        name = getattr(value, "__qualname__", type(value).__name__)
        return {"value": [value], "n": np.full(nod.shape[0], 1)}, ("DofLoad", field, name)


class QuadraticCost:
    """Cost functor cost(v, t) = weight · (v − target(t))², the form of the cost
    elements' `cost` argument that the GPU path evaluates (the reference takes
    any functor, src/BasicElements.jl:198-208).  `target` is a constant or a
    function of t returning a scalar; for SingleAcost it is a constant and the
    functor is called as cost(a).  Works on floats and on any number type with
    + − * (dual numbers of the oracle)."""

    def __init__(self, weight=1.0, target=0.0):
        self.weight = float(weight)
        self.target = target

    def target_at(self, t):
        return float(self.target(t)) if callable(self.target) else float(self.target)

    def __call__(self, v, t=None, *costargs):
        d = v - self.target_at(t)
        return self.weight * (d * d)


def _cost_batch(nod, cost):
    return {"cost": [cost], "n": np.full(nod.shape[0], 1)}


def _cost_name(cost):
    return getattr(cost, "__qualname__", type(cost).__name__)


class SingleDofCost:
    """SingleDofCost: L = cost(x⁽ᵈ⁾, t) on one dof of class X or U (BasicElements.jl:198-208).
    The GPU path takes class X with a QuadraticCost."""

    @staticmethod
    def doflist(key):
        return (1,), (key[1],), (key[2],)

    @staticmethod
    def construct(model, nod, cls, field, cost, derivative=0, costargs=()):
        if cls not in ("X", "U"):
            raise MuscadeError("'class' must be :X or :U")
        data = _cost_batch(nod, cost)
        data["costargs"] = [tuple(costargs)]
        return data, ("SingleDofCost", cls, field, int(derivative), _cost_name(cost))


class SingleUdof:
    """SingleUdof: a U-dof applied as a load on the X-dof of the same node,
    L = cost(u, t) − λu (BasicElements.jl:239-248)."""

    @staticmethod
    def doflist(key):
        return (1, 1), ("X", "U"), (key[1], key[2])

    @staticmethod
    def construct(model, nod, Xfield, Ufield, cost, costargs=()):
        data = _cost_batch(nod, cost)
        data["costargs"] = [tuple(costargs)]
        return data, ("SingleUdof", Xfield, Ufield, _cost_name(cost))


class SingleAcost:
    """SingleAcost: a once-off cost(a) on one A-dof (BasicElements.jl:163-167)."""

    @staticmethod
    def doflist(key):
        return (1,), ("A",), (key[1],)

    @staticmethod
    def construct(model, nod, field, cost, costargs=()):
        data = _cost_batch(nod, cost)
        data["costargs"] = [tuple(costargs)]
        return data, ("SingleAcost", field, _cost_name(cost))


def quadratic_costs(group):
    """The QuadraticCost of every element of a cost group (batch costs repeated
    over their elements); raises if a batch has another cost functor."""
    out = []
    for nodes, d in zip(group.nodes, group.data):
        cost = d["cost"][0]
        if not isinstance(cost, QuadraticCost) or d.get("costargs", [()])[0]:
            raise MuscadeError(f"{group.key[0]}: the GPU path evaluates QuadraticCost costs without costargs, "
                               f"got {type(cost).__name__}")
        out += [cost] * nodes.shape[0]
    return out


def group_cost_targets(group, t):
    """The cost target y(t) of every element of a SingleDofCost or SingleUdof group."""
    counts = [nodes.shape[0] for nodes in group.nodes]
    vals = np.fromiter((d["cost"][0].target_at(t) for d in group.data), dtype=np.float64, count=len(counts))
    return np.repeat(vals, counts)


def group_time_values(group, name, t):
    """Evaluate a per-batch time function (DofLoad value, DofConstraint offset) for all elements of a group."""
    out = []
    for nodes, d in zip(group.nodes, group.data):
        f = d[name][0]
        n = nodes.shape[0]
        v = np.zeros(n) if f is None else np.broadcast_to(np.asarray(f(t), dtype=np.float64), (n,))
        out.append(v)
    return np.concatenate(out) if out else np.zeros(0)
