"""Oracle (test infrastructure only): CPU restatement of the reference's
assembly and solvers for the SweepX path.

* asm maps and CSC pattern: asmvec!/asmmat!  src/Assemble.jl:340-448
  (pairs (j,i) in element-type, element, column, row order; lexicographic
  sortperm; colptr/rowval; asm2[i+nX(j-1), iele] = nnz index)
* assembly: assemble!/addin!{:step|:iter}  src/Assemble.jl:470-608,
  src/SweepX.jl:39-96  (scatter with add_value!/add_∂!, accumulating in
  element order)
* SweepX{0} / SweepX{2} Newton loops: src/SweepX.jl:179-226 with the
  Newmark coefficients and decrement of :3-15 and :98-132.  The reference
  factorises with UMFPACK; the oracle uses SuperLU (scipy.sparse.linalg.splu),
  which yields the same Δx to rounding.

Element evaluations come from oracle.lib (C++ nested duals) for EulerBeam3D
and Bar3D, and from closed forms here for DofConstraint (affine gap) and
DofLoad, and from oracle.testelements for the reference's test elements.
"""
from __future__ import annotations

import math

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla

from . import lib as O


# --------------------------------------------------------------- pattern
def asm_pattern(index_list, n):
    """asmmat! for the all-X dof group.  index_list: per element type, (nele, nX) 1-based.

    Returns colptr (1-based), rowval (1-based), asm1 list, asm2 list (nele, nX*nX) 1-based.
    """
    J, I = [], []
    for idx in index_list:
        nele, nX = idx.shape
        # for iele, jeledof, ieledof  (ieledof fastest)
        jj = np.repeat(idx, nX, axis=1)          # (nele, nX*nX): j varies slowly
        ii = np.tile(idx, (1, nX))               # i varies fastest
        J.append(jj.reshape(-1))
        I.append(ii.reshape(-1))
    J = np.concatenate(J) if J else np.zeros(0, np.int64)
    I = np.concatenate(I) if I else np.zeros(0, np.int64)
    order = np.lexsort((I, J))  # sortperm of (j,i) tuples
    Js, Is = J[order], I[order]
    new = np.ones(len(Js), dtype=bool)
    new[1:] = (Js[1:] != Js[:-1]) | (Is[1:] != Is[:-1])
    inz = np.cumsum(new)  # 1-based nnz of each sorted pair
    K = np.empty(len(Js), dtype=np.int64)
    K[order] = inz
    nnz = int(inz[-1]) if len(inz) else 0
    rowval = Is[new]
    colcount = np.bincount(Js[new], minlength=n + 1)[1:]
    colptr = np.concatenate([[1], 1 + np.cumsum(colcount)])
    asm2, asm1, p = [], [], 0
    for idx in index_list:
        nele, nX = idx.shape
        asm2.append(K[p:p + nele * nX * nX].reshape(nele, nX * nX))
        asm1.append(idx.copy())
        p += nele * nX * nX
    return colptr, rowval, asm1, asm2, nnz


# --------------------------------------------------------------- elements
def group_time_values(group, name, t):
    """Evaluate the user time functions (DofLoad value, constraint offset) of a group at t."""
    out = []
    for nodes, d in zip(group.nodes, group.data):
        f = d[name][0]
        n = nodes.shape[0]
        out.append(np.zeros(n) if f is None else np.broadcast_to(np.asarray(f(t), dtype=np.float64), (n,)))
    return np.concatenate(out) if out else np.zeros(0)


def group_kind(g):
    return g.key[0]


def eval_group(model, g, dis_g, X, U, t, mode, c, scaleX=None, A=None):
    """Residual (scaled) and partials of all elements of a group, in the
    seeding mode of oracle_api.cpp (1: SweepX{0}, 2: Newmark step, 3: iter).
    X: tuple of state vectors (X, X', X'').  Returns R (nele,nX), J (nele,nX,NJ)."""
    idx = dis_g.index_X - 1
    nele, nX = idx.shape
    ND = len(X)
    Xe = np.stack([x[idx] for x in X], axis=1)  # (nele, ND, nX)
    sX = np.broadcast_to(dis_g.scale_X, (nele, nX)).copy()
    kind = group_kind(g)
    if kind in ("EulerBeam3D", "Bar3D"):
        ele = g.cat("ele")
        if kind == "EulerBeam3D" and dis_g.index_A.size:
            # EI-scale A-dof: factor on EI2, EI3 (fields 54, 55 of the 69-field record)
            a = np.asarray(A)[dis_g.index_A[:, 0] - 1]
            ele = ele.copy()
            ele[:, 54] *= a
            ele[:, 55] *= a
        Ue = U[0][dis_g.index_U - 1] if dis_g.index_U.size else None
        a = b = None
        if mode == 2:
            a = c["a2"] * Xe[:, 1, :] + c["a3"] * Xe[:, 2, :]
            b = c["b2"] * Xe[:, 1, :] + c["b3"] * Xe[:, 2, :]
        fn = O.beam_eval if kind == "EulerBeam3D" else (lambda *ar, **kw: O.bar_eval(*ar, t=t, **kw))
        return fn(ele, Xe, Ue, mode=mode, a1=c.get("a1", 0.0), b1=c.get("b1", 0.0), scaleX=sX, a=a, b=b)
    NJ = nX + 1 if mode == 2 else nX
    R = np.zeros((nele, nX))
    Jm = np.zeros((nele, nX, NJ))
    if kind == "DofConstraint":
        coeffs = g.cat("coeffs")
        off = group_time_values(g, "offset", t)
        x0 = Xe[:, 0, :]
        lam = x0[:, -1]
        gap = np.sum(coeffs * x0[:, :-1], axis=1) - off
        nx = nX - 1
        R[:, :nx] = -coeffs * lam[:, None]
        R[:, nx] = -gap
        Jm[:, :nx, nx] = -coeffs * sX[:, [nx]]
        Jm[:, nx, :nx] = -coeffs * sX[:, :nx]
    elif kind == "DofLoad":
        R[:, 0] = -group_time_values(g, "value", t)
    elif kind == "SingleDofCost":
        pass  # R = ∂L/∂Λ = 0 (getresidual of a Lagrangian element, src/Assemble.jl:661-677)
    elif kind == "SingleUdof":
        R[:, 0] = -U[0][dis_g.index_U[:, 0] - 1]  # L = cost(u,t) − λu  ⇒  R = −u
    elif hasattr(g.etype, "oracle_residual"):
        return g.etype.oracle_residual(g, dis_g, X, U, t, mode, c, sX)
    else:
        raise NotImplementedError(kind)
    # scale rows like Lλ .* scale.X (seeds already carry column scales)
    return R * sX, Jm * sX[:, :, None]


class Prepared:
    """prepare(AssemblySweepX{OX}) src/SweepX.jl:24-33."""

    def __init__(self, model, dis):
        self.model, self.dis = model, dis
        self.n = model.ndof["X"]
        self.colptr, self.rowval, self.asm1, self.asm2, self.nnz = asm_pattern([d.index_X for d in dis.dis], self.n)

    def matrix(self, nzval):
        return sp.csc_matrix((nzval, self.rowval - 1, self.colptr - 1), shape=(self.n, self.n))


def assemble(prep, X, U, t, mission, c, A=None):
    """assemble!{mission}: returns Lλ and nzval.  mission: 'static', 'step', 'iter'.
    A: the A-dof values (EI-scale beams)."""
    model, dis = prep.model, prep.dis
    Ll = np.zeros(prep.n)
    nz = np.zeros(prep.nnz)
    mode = {"static": 1, "step": 2, "iter": 3}[mission]
    for g, dg, a1, a2 in zip(model.groups, dis.dis, prep.asm1, prep.asm2):
        if g.nele == 0 or dg.index_X.shape[1] == 0:
            continue  # no X-dofs (SingleAcost): nothing in SweepX's Lλ, Lλx
        R, J = eval_group(model, g, dg, X, U, t, mode, c, A=A)
        nele, nX = R.shape
        # add_value!(Lλ), add_∂!{1,:minus}(Lλ, ..., (Nx+1,)) for the Newmark step,
        # add_∂!{1}(Lλx) with entry i+nX*j <- J[i, j]: serial, in element order
        O.scatter(a1, a2, R, J, Ll, nz, minus_col=nX if mode == 2 else -1)
    return Ll, nz


def newmark_coefficients(OX, dt, beta, gamma):
    """Newmarkβcoefficients  src/SweepX.jl:12-14."""
    if OX == 0:
        return dict(a1=0.0, a2=0.0, a3=0.0, b1=0.0, b2=0.0, b3=0.0)
    return dict(a1=gamma / (beta * dt), a2=gamma / beta, a3=(gamma / (2 * beta) - 1) * dt, b1=1 / (beta * dt**2),
                b2=1 / (beta * dt), b3=1 / (2 * beta))


class NoConvergence(RuntimeError):
    pass


def sweepx(model, dis, initialstate, time, OX=0, beta=0.25, gamma=0.5, maxiter=50, maxdx=1e-5, maxLl=math.inf,
           tvals_override=None, fixed_iter=0):
    """solve(SweepX{OX}) src/SweepX.jl:179-226.  Returns list of (time, X tuple).

    fixed_iter > 0 runs exactly that many Newton iterations per step and
    accepts the state without a convergence test (no counterpart in the
    reference: the fixed-cost time stepping of the device solver)."""
    prep = Prepared(model, dis)
    n = prep.n
    nder = OX + 1
    X = [initialstate.X[i].copy() if i < len(initialstate.X) else np.zeros(n) for i in range(nder)]
    U = tuple(u.copy() for u in initialstate.U)
    A = initialstate.A.copy()
    sX = dis.scaleX
    told = initialstate.time
    out = []
    for step, t in enumerate(time, start=1):
        dt = t - told
        told = t
        if OX > 0 and not dt > 0:
            raise ValueError(f"Time step length not strictly positive at step={step:3d}")
        c = newmark_coefficients(OX, dt, beta, gamma)
        for it in range(1, (fixed_iter if fixed_iter > 0 else maxiter) + 1):
            first = it == 1
            mission = "static" if OX == 0 else ("step" if first else "iter")
            Ll, nz = assemble(prep, tuple(X), U, t, mission, c, A=A)
            Kmat = prep.matrix(nz)
            try:
                lu = spla.splu(Kmat.tocsc())
                dx = lu.solve(Ll)
            except RuntimeError as e:
                raise RuntimeError(f"matrix factorization failed at step={step}, iiter={it}") from e
            dx2, Ll2 = float(np.sum(dx**2)), float(np.sum(Ll**2))
            if OX == 2:
                if first:
                    a = c["a2"] * X[1] / sX + c["a3"] * X[2] / sX
                    b = c["b2"] * X[1] / sX + c["b3"] * X[2] / sX
                    d1 = c["a1"] * dx + a
                    d2 = c["b1"] * dx + b
                else:
                    d1 = c["a1"] * dx
                    d2 = c["b1"] * dx
                X[1] = X[1] - d1 * sX
                X[2] = X[2] - d2 * sX
            X[0] = X[0] - dx * sX
            if fixed_iter > 0:
                if it == fixed_iter:
                    out.append((t, tuple(x.copy() for x in X)))
                continue
            if dx2 <= maxdx**2 and Ll2 <= maxLl**2:
                out.append((t, tuple(x.copy() for x in X)))
                break
            if it == maxiter:
                raise NoConvergence(f"no convergence of step {step:3d} after {it:3d} iterations")
    return out


def sweep_cost(model, dis, traj, t0, OX, U, A):
    """The cost of a SweepX trajectory as the device adjoint defines it: the
    cost elements' Lagrangians summed over the steps, weighted by Δtₙ (OX = 2)
    or 1 (OX = 0), plus the once-off A-costs.  Each element's cost functor is
    called as the reference calls it: cost(x⁽ᵈ⁾, t) for SingleDofCost
    (src/BasicElements.jl:198-208), cost(u, t) for SingleUdof (:239-248; the
    −λu term is not a cost), cost(a) for SingleAcost (:163-167).
    traj: list of (t, X tuple) as returned by sweepx."""
    C = 0.0
    tprev = t0
    for t, X in traj:
        w = (t - tprev) if OX == 2 else 1.0
        tprev = t
        c = 0.0
        for g, dg in zip(model.groups, dis.dis):
            kind = g.key[0]
            if kind not in ("SingleDofCost", "SingleUdof"):
                continue
            e0 = 0
            for nodes, d in zip(g.nodes, g.data):
                cost = d["cost"][0]
                args = d.get("costargs", [()])[0]
                for e in range(e0, e0 + nodes.shape[0]):
                    if kind == "SingleDofCost":
                        v = X[g.key[3]][dg.index_X[e, 0] - 1]
                    else:
                        v = U[0][dg.index_U[e, 0] - 1]
                    c += cost(v, t, *args)
                e0 += nodes.shape[0]
        C += w * c
    for g, dg in zip(model.groups, dis.dis):
        if g.key[0] != "SingleAcost":
            continue
        e0 = 0
        for nodes, d in zip(g.nodes, g.data):
            cost = d["cost"][0]
            args = d.get("costargs", [()])[0]
            for e in range(e0, e0 + nodes.shape[0]):
                C += cost(A[dg.index_A[e, 0] - 1], *args)
            e0 += nodes.shape[0]
    return C
