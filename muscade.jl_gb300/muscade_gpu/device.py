"""Device model: the Python side of the C-ABI (include/muscade_gpu.h).

Builds the `mgpu_model_desc` from a `Model` and its `Disassembler` exactly as
the Julia side would (per element type: kind, dof indices `index.X`/`index.U`,
element fields), and wraps the entry points.
"""
from __future__ import annotations

import ctypes
import math

import numpy as np

from . import _lib as L
from .elements import group_cost_targets, group_time_values, quadratic_costs
from .model import MuscadeError


def _kind(g):
    k = g.key[0]
    if k == "SingleDofCost" and g.key[1] != "X":
        return None  # a cost on a U-dof: not on the GPU path
    return {"EulerBeam3D": L.EULERBEAM3D, "Bar3D": L.BAR3D, "DofConstraint": L.DOFCONSTRAINT_X,
            "DofLoad": L.DOFLOAD, "SingleDofCost": L.DOFCOST, "SingleUdof": L.SINGLEUDOF,
            "SingleAcost": L.ACOST}.get(k)


def _cost_data(g, kind):
    """Element fields of a cost group: DOFCOST (w, d), SINGLEUDOF (w), ACOST (w, y)."""
    costs = quadratic_costs(g)
    w = np.array([c.weight for c in costs], dtype=np.float64)
    if kind == L.DOFCOST:
        if g.key[3] not in (0, 1, 2):
            raise DeviceError(1, f"SingleDofCost: derivative must be 0, 1 or 2, got {g.key[3]}")
        return np.stack([w, np.full(len(w), float(g.key[3]))], axis=1)
    if kind == L.SINGLEUDOF:
        return w[:, None]
    if any(callable(c.target) for c in costs):
        raise DeviceError(1, "SingleAcost: the QuadraticCost target must be a constant")
    return np.stack([w, np.array([c.target_at(None) for c in costs])], axis=1)


class DeviceError(MuscadeError):
    def __init__(self, code, msg):
        super().__init__(msg)
        self.code = code
        self.kind = L.ERRORS.get(code, "unknown")


class DeviceModel:
    """One mgpu_ctx for a model (owns device memory and a CUDA stream)."""

    def __init__(self, model, dis, device: int = 0, linsolve: str = "auto"):
        self.lib = L.load()
        self._registered = []
        self._aticket = 0
        self.model, self.dis = model, dis
        self.nX, self.nU = model.ndof["X"], model.ndof["U"]
        self._keep = []
        groups = (L.Group * max(len(model.groups), 1))()
        for ig, (g, dg) in enumerate(zip(model.groups, dis.dis)):
            kind = _kind(g)
            if kind is None:
                raise DeviceError(3, f"element type {g.key[0]} is not supported by the GPU path")
            iX = np.ascontiguousarray(dg.index_X, dtype=np.int64)
            iU = np.ascontiguousarray(dg.index_U, dtype=np.int64)
            if kind in (L.EULERBEAM3D, L.BAR3D):
                ed = np.ascontiguousarray(g.cat("ele"), dtype=np.float64)
            elif kind == L.DOFCONSTRAINT_X:
                ed = np.ascontiguousarray(g.cat("coeffs"), dtype=np.float64)
            elif kind in (L.DOFCOST, L.SINGLEUDOF, L.ACOST):
                ed = np.ascontiguousarray(_cost_data(g, kind), dtype=np.float64)
            else:
                ed = np.zeros((g.nele, 0))
            self._keep += [iX, iU, ed]
            G = groups[ig]
            G.kind, G.nX, G.nU = kind, iX.shape[1], iU.shape[1] if iU.ndim == 2 else 0
            G.ndata = ed.shape[1] if ed.ndim == 2 else 0
            G.nele = g.nele
            G.indexX = L.ptr(iX, ctypes.c_int64) if iX.size else None
            G.indexU = L.ptr(iU, ctypes.c_int64) if G.nU else None
            G.edata = L.ptr(ed) if G.ndata else None
            iA = np.ascontiguousarray(dg.index_A, dtype=np.int64)
            if iA.size:
                if kind not in (L.EULERBEAM3D, L.ACOST) or iA.shape[1] != 1:
                    raise DeviceError(3, f"A-dofs of element type {g.key[0]} are not supported by the GPU path")
                iA = np.ascontiguousarray(iA[:, 0])
                self._keep.append(iA)
                G.indexA = L.ptr(iA, ctypes.c_int64)
        self._groups = groups
        sc = np.ascontiguousarray(dis.scaleX, dtype=np.float64)
        self._keep.append(sc)
        self.nA = model.ndof["A"]
        desc = L.ModelDesc(self.nX, self.nU, len(model.groups), groups, L.ptr(sc), device, self.nA)
        self.ctx = ctypes.c_void_p()
        rc = self.lib.mgpu_create(ctypes.byref(self.ctx), ctypes.byref(desc))
        self._check(rc)
        self.nnz = int(self.lib.mgpu_nnz(self.ctx))
        self.ntval = int(self.lib.mgpu_ntval(self.ctx))
        if linsolve != "auto":
            self.set_linear_solver(linsolve)

    def set_A(self, A):
        """A-dof values (the EI scale factors of EulerBeam3D{adof}); 1 until set."""
        a = np.ascontiguousarray(A, dtype=np.float64)
        if a.shape != (self.nA,):
            raise ValueError(f"A must have {self.nA} values")
        self._check(self.lib.mgpu_set_A(self.ctx, L.ptr(a)))

    def adjoint(self, OX, times, t0, X0, cost_dof=(), cost_w=1.0, cost_y=None, U=None, beta=0.25, gamma=0.5,
                maxiter=50, maxdx=1e-10, maxLl=math.inf, ckpt=0, load_gradient=False, u_gradient=False, tvals=None):
        """Cost and its gradient with respect to the A-dofs (and, with
        load_gradient, to the time values; with u_gradient, to the U-dofs of
        SingleUdof elements) by the discrete adjoint of a converged SweepX{OX}
        sweep; see mgpu_adjoint_sweepx.  The cost is that of the model's cost
        elements plus optional sensors: cost_dof 1-based X-dofs, cost_y[nstep][ncost].
        tvals: the time values of every step (time_values(times)), evaluated
        here when None.  Returns (cost, dCdA, dCdtv, stats), and dCdU after
        them with u_gradient."""
        times = np.ascontiguousarray(times, dtype=np.float64)
        nstep = len(times)
        X0 = [np.asarray(v, dtype=np.float64) for v in X0][: OX + 1]
        x0 = np.ascontiguousarray(np.concatenate(X0)) if X0 else np.zeros(0)
        u = np.ascontiguousarray(U if U is not None else np.zeros(self.nU), dtype=np.float64)
        tv = self.time_values(times) if tvals is None else np.ascontiguousarray(tvals, dtype=np.float64)
        if tv.shape != (nstep, self.ntval):
            raise ValueError(f"tvals must be [{nstep}][{self.ntval}]")
        cd = np.ascontiguousarray(cost_dof, dtype=np.int64).reshape(-1)
        cw = np.ascontiguousarray(np.broadcast_to(cost_w, cd.shape), dtype=np.float64)
        cy = np.ascontiguousarray(np.zeros((nstep, 0)) if cost_y is None else cost_y, dtype=np.float64)
        cy = cy.reshape(nstep, len(cd))
        opts = L.SweepOpts(beta, gamma, maxiter, maxdx, maxLl, 0, 0, 0, 0)
        cost = ctypes.c_double()
        dA = np.zeros(max(self.nA, 1))
        dtv = np.zeros((nstep, self.ntval)) if load_gradient and self.ntval else None
        dU = np.zeros(max(self.nU, 1)) if u_gradient else None
        stats = L.Stats()
        rc = self.lib.mgpu_adjoint_sweepx(self.ctx, OX, nstep, L.ptr(times), float(t0), len(X0), L.ptr(x0), L.ptr(u),
                                          L.ptr(tv), ctypes.byref(opts), len(cd),
                                          L.ptr(cd, ctypes.c_int64) if len(cd) else None,
                                          L.ptr(cw) if len(cd) else None, L.ptr(cy) if len(cd) else None,
                                          int(ckpt), ctypes.byref(cost), L.ptr(dA),
                                          L.ptr(dtv) if dtv is not None else None,
                                          L.ptr(dU) if dU is not None else None, ctypes.byref(stats))
        self._check(rc)
        if u_gradient:
            return cost.value, dA[: self.nA], dtv, stats, dU[: self.nU]
        return cost.value, dA[: self.nA], dtv, stats

    def sensitivity(self, OX, times, t0, X0, sel, cost_dof=(), cost_w=1.0, cost_y=None, U=None, beta=0.25,
                    gamma=0.5, maxiter=50, maxdx=1e-10, maxLl=math.inf, states=False, tvals=None):
        """Forward sensitivities with respect to the A-dofs `sel` (1-based) of a
        converged SweepX{OX} sweep (mgpu_sensitivity_sweepx).  Returns (dCdA[nsel],
        dXdA[nstep][nsel][OX+1][nX] or None, stats); the cost as in adjoint()."""
        times = np.ascontiguousarray(times, dtype=np.float64)
        nstep = len(times)
        X0 = [np.asarray(v, dtype=np.float64) for v in X0][: OX + 1]
        x0 = np.ascontiguousarray(np.concatenate(X0)) if X0 else np.zeros(0)
        u = np.ascontiguousarray(U if U is not None else np.zeros(self.nU), dtype=np.float64)
        tv = self.time_values(times) if tvals is None else np.ascontiguousarray(tvals, dtype=np.float64)
        cd = np.ascontiguousarray(cost_dof, dtype=np.int64).reshape(-1)
        cw = np.ascontiguousarray(np.broadcast_to(cost_w, cd.shape), dtype=np.float64)
        cy = np.ascontiguousarray(np.zeros((nstep, 0)) if cost_y is None else cost_y, dtype=np.float64)
        cy = cy.reshape(nstep, len(cd))
        sl = np.ascontiguousarray(sel, dtype=np.int64).reshape(-1)
        opts = L.SweepOpts(beta, gamma, maxiter, maxdx, maxLl, 0, 0, 0, 0)
        dC = np.zeros(len(sl))
        dX = np.zeros((nstep, len(sl), OX + 1, self.nX)) if states else None
        stats = L.Stats()
        rc = self.lib.mgpu_sensitivity_sweepx(self.ctx, OX, nstep, L.ptr(times), float(t0), len(X0), L.ptr(x0),
                                              L.ptr(u), L.ptr(tv), ctypes.byref(opts), len(cd),
                                              L.ptr(cd, ctypes.c_int64) if len(cd) else None,
                                              L.ptr(cw) if len(cd) else None, L.ptr(cy) if len(cd) else None,
                                              len(sl), L.ptr(sl, ctypes.c_int64), L.ptr(dX) if dX is not None else None,
                                              L.ptr(dC), ctypes.byref(stats))
        self._check(rc)
        return dC, dX, stats

    def autotune(self, mission=L.ASM_STATIC, c=None):
        """Time the element kernels' block sizes and the applicable linear solvers on
        the resident state (see upload_state) and keep the fastest (mgpu_autotune)."""
        nm = L.Newmark(**(c or {})) if c else L.Newmark()
        rep = L.TuneReport()
        self._check(self.lib.mgpu_autotune(self.ctx, mission, ctypes.byref(nm), ctypes.byref(rep)))
        return {"elem_block": rep.elem_block, "linsolve": L.LINSOLVE_NAME[rep.linsolve],
                "ms_elem": dict(zip((64, 128, 256), list(rep.ms_elem))),
                "ms_linsolve": {L.LINSOLVE_NAME[k]: rep.ms_linsolve[k] for k in range(1, 6) if rep.ms_linsolve[k] >= 0}}

    def set_linear_solver(self, kind: str):
        """'auto' | 'f32ir' (row-band FP32 factors + FP64 refinement) | 'f64' (row-band) |
        'block' | 'torn' (partitioned, FP64) | 'torn32' (partitioned, FP32 factors +
        FP64 refinement) | 'sparse' (multifrontal, FP32 factors + FP64 refinement) |
        'sparse64' (multifrontal, FP64); see mgpu_set_linear_solver."""
        self._check(self.lib.mgpu_set_linear_solver(self.ctx, L.LINSOLVE[kind]))

    def launch_count(self):
        """Kernel launches of the assembly, Newton and multifrontal paths so far (mgpu_launch_count)."""
        return int(self.lib.mgpu_launch_count(self.ctx))

    def sparse_info(self):
        """Structure and last solve of the multifrontal solver (mgpu_sparse_info)."""
        rep = L.SparseReport()
        self._check(self.lib.mgpu_sparse_info(self.ctx, ctypes.byref(rep)))
        return {f: getattr(rep, f) for f, _ in L.SparseReport._fields_}

    def linear_solver_info(self):
        info = L.LinsolveInfo()
        self._check(self.lib.mgpu_linear_solver_info(self.ctx, ctypes.byref(info)))
        return {"kind": L.LINSOLVE_NAME[info.kind], "ncomp": info.ncomp, "max_kl": info.max_kl,
                "max_ku": info.max_ku, "last_fallback": info.last_fallback, "last_sweeps": info.last_sweeps}

    # ---------------------------------------------------------------- basics
    def _check(self, rc):
        if rc != L.MGPU_OK:
            msg = self.lib.mgpu_last_error(self.ctx).decode(errors="replace") if self.ctx else "mgpu_create failed"
            raise DeviceError(rc, msg)

    def close(self):
        # destroy first: it waits for the context's streams, so no copy into a
        # page-locked buffer (a pipelined assembly's outputs) is still in flight
        if getattr(self, "ctx", None):
            self.lib.mgpu_destroy(self.ctx)
            self.ctx = None
        for buf in getattr(self, "_registered", []):
            self.lib.mgpu_host_unregister(buf.ctypes.data_as(ctypes.c_void_p))
        self._registered = []

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def pattern(self):
        colptr = np.zeros(self.nX + 1, dtype=np.int64)
        rowval = np.zeros(self.nnz, dtype=np.int64)
        self._check(self.lib.mgpu_get_pattern(self.ctx, L.ptr(colptr, ctypes.c_int64), L.ptr(rowval, ctypes.c_int64)))
        return colptr, rowval

    def asm(self, ig):
        dg = self.dis.dis[ig]
        nele, nX = dg.index_X.shape
        a1 = np.zeros((nele, nX), dtype=np.int64)
        a2 = np.zeros((nele, nX * nX), dtype=np.int64)
        self._check(self.lib.mgpu_get_asm(self.ctx, ig, L.ptr(a1, ctypes.c_int64), L.ptr(a2, ctypes.c_int64)))
        return a1, a2

    def time_values(self, times):
        """The time values of every step, [nstep][ntval] (see tvals)."""
        nstep = len(times)
        return np.ascontiguousarray(np.stack([self.tvals(t) for t in times]) if self.ntval else np.zeros((nstep, 0)))

    def tvals(self, t):
        """Host evaluation of the time functions (DofLoad F(t), constraint offsets
        c(t), cost targets y(t)) in the layout of mgpu_ntval."""
        out = []
        for g in self.model.groups:
            if g.key[0] == "DofLoad":
                out.append(group_time_values(g, "value", t))
            elif g.key[0] == "DofConstraint":
                out.append(group_time_values(g, "offset", t))
            elif g.key[0] in ("SingleDofCost", "SingleUdof"):
                out.append(group_cost_targets(g, t))
        return np.ascontiguousarray(np.concatenate(out) if out else np.zeros(0))

    # ---------------------------------------------------------------- assembly
    def _pinned(self, name, n):
        """A host array kept for the life of the model and page-locked for the device copies."""
        buf = getattr(self, name, None)
        if buf is None or buf.size != n:
            buf = np.zeros(max(n, 1))
            if self.lib.mgpu_host_register(buf.ctypes.data_as(ctypes.c_void_p), buf.nbytes) == L.MGPU_OK:
                self._registered.append(buf)
            setattr(self, name, buf)
        return buf[:n]

    def assemble(self, X, U=None, t=0.0, mission=L.ASM_STATIC, c=None, want=(True, True), reuse=False):
        """One assembly with host buffers (mgpu_assemble).  With reuse, the state
        goes through and the outputs come back in page-locked arrays kept by the
        model: the returned arrays are overwritten by the next reuse call."""
        X = [np.ascontiguousarray(x, dtype=np.float64) for x in X]
        nXder = len(X)
        if reuse:
            x = self._pinned("_xin", nXder * self.nX)
            np.concatenate(X, out=x)
        else:
            x = np.ascontiguousarray(np.concatenate(X))
        u = np.ascontiguousarray(U if U is not None else np.zeros(self.nU), dtype=np.float64)
        tv = self.tvals(t)
        nm = L.Newmark(**(c or {})) if c else L.Newmark()
        if reuse:
            Ll = self._pinned("_Lout", self.nX) if want[0] else None
            nz = self._pinned("_nzout", self.nnz) if want[1] else None
        else:
            Ll = np.zeros(self.nX) if want[0] else None
            nz = np.zeros(self.nnz) if want[1] else None
        rc = self.lib.mgpu_assemble(self.ctx, mission, nXder, L.ptr(x), L.ptr(u), float(t), L.ptr(tv),
                                    ctypes.byref(nm), L.ptr(Ll), L.ptr(nz))
        self._check(rc)
        return Ll, nz

    def assemble_async(self, X, U=None, t=0.0, mission=L.ASM_STATIC, c=None, want=(True, True)):
        """Pipelined assembly (mgpu_assemble_async): enqueues one assembly and
        returns (ticket, Lλ, nzval) without waiting.  The arrays are page-locked
        buffers of the ticket's slot (two slots, alternating), valid after
        assemble_wait(ticket) and overwritten two calls later."""
        X = [np.ascontiguousarray(x, dtype=np.float64) for x in X]
        x = X[0] if len(X) == 1 else np.concatenate(X)
        u = np.ascontiguousarray(U if U is not None else np.zeros(self.nU), dtype=np.float64)
        tv = self.tvals(t)
        nm = L.Newmark(**(c or {})) if c else L.Newmark()
        slot = self._aticket & 1
        Ll = self._pinned(f"_aLout{slot}", self.nX) if want[0] else None
        nz = self._pinned(f"_anzout{slot}", self.nnz) if want[1] else None
        tk = ctypes.c_int64()
        rc = self.lib.mgpu_assemble_async(self.ctx, mission, len(X), L.ptr(x), L.ptr(u), float(t), L.ptr(tv),
                                          ctypes.byref(nm), L.ptr(Ll), L.ptr(nz), ctypes.byref(tk))
        self._check(rc)
        self._aticket = tk.value + 1
        return tk.value, Ll, nz

    def assemble_wait(self, ticket):
        """Waits for the outputs of a pipelined assembly (one of the last two tickets)."""
        self._check(self.lib.mgpu_assemble_wait(self.ctx, int(ticket)))

    def element_eval(self, ig, X, U=None, t=0.0, p=(1.0, 0.0, 0.0)):
        """diffed_residual-like evaluation of all elements of group ig.
        X: (nele, nXder, nX).  Returns R (nele,nX), dR (nele,nX,nX) [i,j], dRdU (nele,nX,3) or None."""
        X = np.ascontiguousarray(X, dtype=np.float64)
        nele, nXder, nX = X.shape
        R = np.zeros((nele, nX))
        dR = np.zeros((nele, nX * nX))
        Uc = None if U is None else np.ascontiguousarray(U, dtype=np.float64)
        H = np.zeros((nele, nX * 3)) if U is not None else None
        rc = self.lib.mgpu_element_eval(self.ctx, ig, nXder, L.ptr(X), L.ptr(Uc), float(t), p[0], p[1], p[2],
                                        L.ptr(R), L.ptr(dR), L.ptr(H))
        self._check(rc)
        dR = dR.reshape(nele, nX, nX).transpose(0, 2, 1)  # column-major per element -> [i, j]
        if H is not None:
            H = H.reshape(nele, 3, nX).transpose(0, 2, 1)
        return R, dR, H

    def element_lagrangian(self, ig, Lam, X, U=None, A=None, t=0.0):
        """diffed_lagrangian{2}-like evaluation of the elements of group ig
        (loads, constraints and cost elements; mgpu_element_lagrangian).
        Lam (nele,nX), X (nele,nXder,nX), U (nele,nU), A (nele,nA).  Returns L (nele,),
        dL (nele,np), d2L (nele,np,np) over (Λ, X⁽⁰⁾.., U, A)."""
        g = self.model.groups[ig]
        dg = self.dis.dis[ig]
        nele = g.nele
        nX = dg.index_X.shape[1]
        nU = dg.index_U.shape[1] if dg.index_U.ndim == 2 else 0
        nA = dg.index_A.shape[1] if dg.index_A.ndim == 2 else 0
        X = np.ascontiguousarray(X, dtype=np.float64).reshape(nele, -1, nX) if nX else np.zeros((nele, 1, 0))
        nXder = X.shape[1]
        lam = np.ascontiguousarray(Lam, dtype=np.float64).reshape(nele, nX)
        Uc = np.ascontiguousarray(U if U is not None else np.zeros((nele, nU)), dtype=np.float64).reshape(nele, nU)
        Ac = np.ascontiguousarray(A if A is not None else np.zeros((nele, nA)), dtype=np.float64).reshape(nele, nA)
        tvall = self.tvals(t)
        tv = None
        off = 0
        for h in self.model.groups[:ig]:
            if h.key[0] in ("DofLoad", "DofConstraint", "SingleDofCost", "SingleUdof"):
                off += h.nele
        if g.key[0] in ("DofLoad", "DofConstraint", "SingleDofCost", "SingleUdof"):
            tv = np.ascontiguousarray(tvall[off:off + nele])
        npar = nX * (1 + nXder) + nU + nA
        Lv = np.zeros(nele)
        dL = np.zeros((nele, npar))
        d2L = np.zeros((nele, npar, npar))
        rc = self.lib.mgpu_element_lagrangian(self.ctx, ig, nXder, L.ptr(lam), L.ptr(X), L.ptr(Uc), L.ptr(Ac),
                                              L.ptr(tv) if tv is not None else None, L.ptr(Lv), L.ptr(dL), L.ptr(d2L))
        self._check(rc)
        return Lv, dL, d2L

    BEAM_RESULTS = ("eps", "rsm", "x", "kappa", "fi", "mi")

    def beam_results(self, ig, X):
        """getresult of an EulerBeam3D group at states X[nstate][nX] (mgpu_beam_results):
        a dict of arrays eps (nstate, nele), rsm (nstate, nele, 3, 3), and per Gauss
        point x, kappa, mi (nstate, nele, 4, 3) and fi (nstate, nele, 4)."""
        X = np.ascontiguousarray(np.atleast_2d(X), dtype=np.float64)
        nstate = X.shape[0]
        nele = self.model.groups[ig].nele
        out = np.zeros((nstate, nele, 50))
        self._check(self.lib.mgpu_beam_results(self.ctx, ig, nstate, L.ptr(X), L.ptr(out)))
        gp = out[:, :, 10:].reshape(nstate, nele, 4, 10)
        return {"eps": out[:, :, 0], "rsm": out[:, :, 1:10].reshape(nstate, nele, 3, 3).transpose(0, 1, 3, 2),
                "x": gp[..., 0:3], "kappa": gp[..., 3:6], "fi": gp[..., 6], "mi": gp[..., 7:10]}

    def upload_state(self, X, U=None, t=0.0):
        x = np.ascontiguousarray(np.concatenate([np.asarray(v, dtype=np.float64) for v in X]))
        u = np.ascontiguousarray(U if U is not None else np.zeros(self.nU), dtype=np.float64)
        tv = self.tvals(t)
        self._check(self.lib.mgpu_upload_state(self.ctx, len(X), L.ptr(x), L.ptr(u), L.ptr(tv)))

    def time_assemble(self, mission=L.ASM_STATIC, t=0.0, c=None, reps=10, flush_l2=True):
        """Mean device times (ms) of `reps` resident assemblies: total, per element type, scatter."""
        nm = L.Newmark(**(c or {})) if c else L.Newmark()
        tt, ts = ctypes.c_double(), ctypes.c_double()
        tg = np.zeros(max(len(self.model.groups), 1))
        self._check(self.lib.mgpu_time_assemble(self.ctx, mission, float(t), ctypes.byref(nm), reps, int(flush_l2),
                                                ctypes.byref(tt), L.ptr(tg), ctypes.byref(ts)))
        return tt.value, tg[: len(self.model.groups)], ts.value

    # ---------------------------------------------------------------- solver
    def sweepx(self, OX, times, t0, X0, U=None, beta=0.25, gamma=0.5, maxiter=50, maxdx=1e-5, maxLl=math.inf,
               fixed_iter=0, per_component=False, graph=True, device_loop=False):
        """Whole SweepX{OX} on the device.  fixed_iter > 0 runs exactly that many
        Newton iterations per step (replayed from a captured CUDA graph unless
        graph=False); per_component applies the convergence test to each
        connected component (independent models) on its own; device_loop runs
        the load steps and Newton iterations of a SweepX{0} as one graph launch
        with device-side loops (see mgpu_sweep_opts.device_loop)."""
        times = np.ascontiguousarray(times, dtype=np.float64)
        nstep = len(times)
        X0 = [np.asarray(v, dtype=np.float64) for v in X0][: OX + 1]
        x0 = np.ascontiguousarray(np.concatenate(X0)) if X0 else np.zeros(0)
        u = np.ascontiguousarray(U if U is not None else np.zeros(self.nU), dtype=np.float64)
        tv = np.ascontiguousarray(np.stack([self.tvals(t) for t in times]) if self.ntval else np.zeros((nstep, 0)))
        opts = L.SweepOpts(beta, gamma, maxiter, maxdx, maxLl, fixed_iter, int(bool(per_component)),
                           int(not graph), int(bool(device_loop)))
        states = np.zeros((nstep, OX + 1, self.nX))
        stats = L.Stats()
        rc = self.lib.mgpu_sweepx(self.ctx, OX, nstep, L.ptr(times), float(t0), len(X0), L.ptr(x0), L.ptr(u),
                                  L.ptr(tv), ctypes.byref(opts), L.ptr(states), ctypes.byref(stats))
        return rc, states, stats
