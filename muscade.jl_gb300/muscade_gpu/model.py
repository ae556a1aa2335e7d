"""Host-side mirror of the reference's model description and disassembler.

Restates, for the element types the GPU path supports, what the reference's
Julia side computes before `solve` hands work to the device:

* `Model`, `addnode`, `addelement`, `initialize`  -- src/ModelDescription.jl:64-324.
  Dofs are numbered per class (X, U, A) in first-seen order over the calls to
  `addelement` and, within an element, over its `doflist` (ModelDescription.jl:226-249).
  Element types are grouped by their concrete type in first-seen order
  (ModelDescription.jl:198-208).
* `Disassembler` -- src/Assemble.jl:22-99: per element type, the model dof
  indices of each element's X, U and A dofs (1-based, like the reference).
* `State` -- src/Assemble.jl:106-129.

Batched `addelement` calls (a matrix of node ids, ModelDescription.jl:195) are
processed with vectorised numbering that yields exactly the sequential
first-seen order.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field
from typing import Any, Dict, List, Sequence, Tuple

import numpy as np


class MuscadeError(RuntimeError):
    """Raised where the reference raises `muscadeerror` (src/Exceptions.jl:14-24)."""


@dataclass
class DofTyp:
    cls: str
    field: str
    scale: float = 1.0


@dataclass
class ElementGroup:
    """All elements of one concrete element type (model.ele[ieletyp] / model.eleobj[ieletyp])."""

    etype: Any  # element class
    key: tuple  # identity of the concrete type
    nodes: List[np.ndarray] = field(default_factory=list)  # per batch: (nele, nnod) 1-based node ids
    data: List[Dict[str, np.ndarray]] = field(default_factory=list)  # per batch: per-element arrays
    dofid: List[np.ndarray] = field(default_factory=list)  # per batch: (nele, neledof) 1-based idof in class

    @property
    def nele(self) -> int:
        return int(sum(len(n) for n in self.nodes))

    def cat(self, name):
        return np.concatenate([d[name] for d in self.data], axis=0)

    def node_ids(self):
        return np.concatenate(self.nodes, axis=0)

    def dof_ids(self):
        return np.concatenate(self.dofid, axis=0)


class Model:
    """Mirror of `Model` (src/ModelDescription.jl:64-77, constructor :150)."""

    def __init__(self, ID: str = "muscade_model"):
        self.ID = ID
        self.coords: List[np.ndarray] = []
        self.groups: List[ElementGroup] = []
        self.doftyp: List[DofTyp] = []
        self.ndof = {"X": 0, "U": 0, "A": 0}
        # node-dof map: (inod, idoftyp) -> idof (1-based within class); grown as needed
        self._ndmap = np.zeros((0, 0), dtype=np.int64)
        self.dof_node = {"X": [], "U": [], "A": []}  # per class, per idof: node id
        self.dof_typ = {"X": [], "U": [], "A": []}  # per class, per idof: idoftyp (0-based)
        self.scaleL = 1.0
        self.locked = False

    # ---- nodes -------------------------------------------------------------
    @property
    def nnod(self) -> int:
        return len(self.coords)

    def addnode(self, coord):
        """addnode!  ModelDescription.jl:166-173.  Returns a 1-based node id (or ids for a matrix)."""
        self._assert_unlocked()
        c = np.asarray(coord, dtype=np.float64)
        if c.ndim == 1:
            self.coords.append(c.copy())
            self._grow_nodes()
            return self.nnod
        first = self.nnod + 1
        for row in c:
            self.coords.append(row.copy())
        self._grow_nodes()
        return np.arange(first, self.nnod + 1, dtype=np.int64)

    def coord(self, inod: int) -> np.ndarray:
        return self.coords[inod - 1]

    def _grow_nodes(self):
        n, t = self._ndmap.shape
        if self.nnod > n:
            m = np.zeros((max(self.nnod, 2 * n), max(t, 8)), dtype=np.int64)
            m[:n, :t] = self._ndmap
            self._ndmap = m

    def _idoftyp(self, cls: str, fld: str) -> int:
        for i, d in enumerate(self.doftyp):
            if d.cls == cls and d.field == fld:
                return i
        self.doftyp.append(DofTyp(cls, fld))
        n, t = self._ndmap.shape
        if len(self.doftyp) > t:
            m = np.zeros((n, 2 * t), dtype=np.int64)
            m[:, :t] = self._ndmap
            self._ndmap = m
        return len(self.doftyp) - 1

    # ---- elements ----------------------------------------------------------
    def addelement(self, etype, nodid, **kwargs):
        """addelement!  ModelDescription.jl:195-263.

        `nodid` is a vector of node ids (one element) or a matrix (one element
        per row).  Keyword values may be per-element arrays (leading dimension
        = number of elements) for batched construction.  Returns the element
        numbers within the type (1-based), like EleID.iele.
        """
        self._assert_unlocked()
        nod = np.asarray(nodid, dtype=np.int64)
        single = nod.ndim == 1
        if single:
            nod = nod.reshape(1, -1)
        nele, nnod = nod.shape
        data, key = etype.construct(self, nod, **kwargs)
        inod, cls, fld = etype.doflist(key)
        if nnod != max(inod):
            raise MuscadeError(
                f"Connecting element of type {etype.__name__}: Second dimension of inod ({nnod}) must be equal to element's nnod ({max(inod)})"
            )
        # element type (new types appended in first-seen order)
        ig = next((i for i, g in enumerate(self.groups) if g.key == key), None)
        if ig is None:
            self.groups.append(ElementGroup(etype=etype, key=key))
            ig = len(self.groups) - 1
        grp = self.groups[ig]
        iele0 = grp.nele
        # dof types in eledof order (all elements of a batch share the doflist)
        idt = np.array([self._idoftyp(c, f) for c, f in zip(cls, fld)], dtype=np.int64)
        neledof = len(inod)
        # (node, doftyp) keys in (element, eledof) order
        nodes_k = nod[:, np.asarray(inod) - 1]  # (nele, neledof)
        typ_k = np.broadcast_to(idt, (nele, neledof))
        flat_n = nodes_k.reshape(-1)
        flat_t = typ_k.reshape(-1)
        existing = self._ndmap[flat_n - 1, flat_t]
        dofid = existing.copy()
        new = existing == 0
        if np.any(new):
            key_new = flat_n[new] * (len(self.doftyp) + 1) + flat_t[new]
            uniq, first = np.unique(key_new, return_index=True)
            order = np.sort(first)  # first occurrences, in sequential order
            pos_new = np.flatnonzero(new)
            for c in ("X", "U", "A"):
                sel = [p for p in order if self.doftyp[int(flat_t[pos_new[p]])].cls == c]
                if not sel:
                    continue
                sel = np.asarray(sel, dtype=np.int64)
                ids = self.ndof[c] + 1 + np.arange(len(sel), dtype=np.int64)
                self.ndof[c] += len(sel)
                nn = flat_n[pos_new[sel]]
                tt = flat_t[pos_new[sel]]
                self._ndmap[nn - 1, tt] = ids
                self.dof_node[c].extend(nn.tolist())
                self.dof_typ[c].extend(tt.tolist())
            dofid = self._ndmap[flat_n - 1, flat_t]
        grp.nodes.append(nod.copy())
        grp.data.append(data)
        grp.dofid.append(dofid.reshape(nele, neledof))
        ids = np.arange(iele0 + 1, iele0 + nele + 1)
        return int(ids[0]) if single else ids

    def setscale(self, scale=None, scaleL=None):
        """setscale!  ModelDescription.jl:287-299."""
        self._assert_unlocked()
        if scale is not None:
            for d in self.doftyp:
                if d.cls in scale and d.field in scale[d.cls]:
                    d.scale = float(scale[d.cls][d.field])
        if scaleL is not None:
            self.scaleL = float(scaleL)

    def initialize(self, time: float = -math.inf, nXder: int = 1):
        """initialize!  ModelDescription.jl:319-324.  Locks the model."""
        self._assert_unlocked()
        self.locked = True
        dis = Disassembler(self)
        return State(self, dis, time=time, nXder=nXder)

    def _assert_unlocked(self):
        if self.locked:
            raise MuscadeError(f"model {self.ID} is initialized and can no longer be edited")

    def getndof(self, cls: str) -> int:
        return self.ndof[cls]

    def nele(self) -> int:
        return sum(g.nele for g in self.groups)


class EletypDisassembler:
    def __init__(self, index_X, index_U, index_A, scale_X, scale_U, scale_A, scale_L):
        self.index_X = index_X  # (nele, nX) 1-based model idof
        self.index_U = index_U
        self.index_A = index_A
        self.scale_X = scale_X  # (nX,)
        self.scale_U = scale_U
        self.scale_A = scale_A
        self.scale_L = scale_L


class Disassembler:
    """Disassembler(model)  src/Assemble.jl:32-99."""

    def __init__(self, model: Model):
        NX, NU, NA = model.ndof["X"], model.ndof["U"], model.ndof["A"]
        self.scaleX = np.ones(NX)
        self.scaleU = np.ones(NU)
        self.scaleA = np.ones(NA)
        self.scaleL = np.ones(NX)
        self.fieldX = [None] * NX
        self.fieldU = [None] * NU
        self.fieldA = [None] * NA
        self.dis: List[EletypDisassembler] = []
        for g in model.groups:
            inod, cls, fld = g.etype.doflist(g.key)
            cls = np.asarray(cls)
            ids = g.dof_ids()
            idt = [model._idoftyp(c, f) for c, f in zip(cls, fld)]
            sc = np.array([model.doftyp[i].scale for i in idt])
            parts = {}
            for c in ("X", "U", "A"):
                m = cls == c
                parts[c] = (ids[:, m], sc[m])
            eX, eU, eA = parts["X"][0], parts["U"][0], parts["A"][0]
            sX, sU, sA = parts["X"][1], parts["U"][1], parts["A"][1]
            self.dis.append(EletypDisassembler(eX, eU, eA, sX, sU, sA, sX * model.scaleL))
            if eX.size:
                self.scaleX[eX.reshape(-1) - 1] = np.broadcast_to(sX, eX.shape).reshape(-1)
                self.scaleL[eX.reshape(-1) - 1] = np.broadcast_to(sX * model.scaleL, eX.shape).reshape(-1)
            if eU.size:
                self.scaleU[eU.reshape(-1) - 1] = np.broadcast_to(sU, eU.shape).reshape(-1)
            if eA.size:
                self.scaleA[eA.reshape(-1) - 1] = np.broadcast_to(sA, eA.shape).reshape(-1)
            fX = [f for c, f in zip(cls, fld) if c == "X"]
            for j, f in enumerate(fX):
                for i in eX[:, j]:
                    self.fieldX[i - 1] = f
            fU = [f for c, f in zip(cls, fld) if c == "U"]
            for j, f in enumerate(fU):
                for i in eU[:, j]:
                    self.fieldU[i - 1] = f


class State:
    """State  src/Assemble.jl:106-129: time, X (tuple of derivatives), U, A."""

    def __init__(self, model: Model, dis: Disassembler, time: float = -math.inf, nXder: int = 1, nUder: int = 1):
        self.model = model
        self.dis = dis
        self.time = float(time)
        nX, nU, nA = model.ndof["X"], model.ndof["U"], model.ndof["A"]
        self.L = (np.zeros(nX),)
        self.X = tuple(np.zeros(nX) for _ in range(nXder))
        self.U = tuple(np.zeros(nU) for _ in range(nUder))
        self.A = np.zeros(nA)

    def copy(self, nXder: int | None = None) -> "State":
        s = State.__new__(State)
        s.model, s.dis, s.time = self.model, self.dis, self.time
        s.L = tuple(a.copy() for a in self.L)
        nX = len(self.X) if nXder is None else nXder
        xs = [self.X[i].copy() if i < len(self.X) else np.zeros_like(self.X[0]) for i in range(nX)]
        s.X = tuple(xs)
        s.U = tuple(a.copy() for a in self.U)
        s.A = self.A.copy()
        return s

    def getdof(self, field: str, nodID: Sequence[int] | None = None, order: int = 0, cls: str = "X"):
        """Values of the dofs of a field (optionally at given nodes), like getdof (src/Output.jl:21-54)."""
        m = self.model
        idt = next(i for i, d in enumerate(m.doftyp) if d.cls == cls and d.field == field)
        typ = np.asarray(m.dof_typ[cls])
        nod = np.asarray(m.dof_node[cls])
        sel = typ == idt
        if nodID is not None:
            sel &= np.isin(nod, np.asarray(nodID))
        vec = {"X": self.X, "U": self.U}[cls][order] if cls in ("X", "U") else self.A
        return vec[np.flatnonzero(sel)]
