"""Oracle (test infrastructure only): the static identification problem of
the device's discrete adjoint, solved all steps at once like DirectXUA: for
models of residual elements (EulerBeam3D with the EI-scale A-dof, Hold,
DofLoad) observed by SingleDofCost-type sensor costs, static (OX=0, no
U-dofs), loads given and A held.

It is the stationarity of Σₙ Δt (Λₙ·Rₙ + costₙ) over (Λ, X) with the complete
Lagrangian: Lλ = R, Lx = (∂R/∂X)ᵀΛ + ∇cost, Lλx = ∂R/∂X, Lxx = ∇²cost (the
beam's residual has no second-order term in the Newton system), solved by one
sparse LU per Newton iteration with the block layout of the reference's big
system (blocks (λ, x) of every step in step order, assemblebig!,
src/DirectXUA.jl:317-356, decremented block by block like decrementbig!,
:357-383).  The cost gradient with respect to A is the A-block of Lv at the
converged (Λ, X): Σₙ Δt Λₙ·∂Rₙ/∂A.  The EI-scale beam residual is affine in
its A-dof (the bending moments are linear in EI₂, EI₃), so
∂R_e/∂a_e = R_e(a_e = 1) − R_e(a_e = 0) exactly.

Two differences from the reference's DirectXUA, which oracle/direct.py
restates and pins to the reference's own tests: there the steps of a static
problem carry weight 1 (assemble! with idmult, src/DirectXUA.jl:331; the
factor Δt here is a uniform scaling of the step terms, which leaves Λ and X
unchanged and scales dC/dA by Δt), and elements without second order, like
EulerBeam3D, add only Lλ and the Λ-cross blocks (:85-120), not (∂R/∂X)ᵀΛ to
Lx.  This restatement is pinned by central differences of the oracle's
SweepX{0} cost (tests/test_directxua.py).
"""
from __future__ import annotations

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla

from . import reference as REF


def _sensor_terms(x, sensors, w, y):
    """Value, gradient and (diagonal) Hessian of Σ_s w (x[d_s] − y_s)²."""
    d = np.asarray(sensors) - 1
    r = x[d] - y
    g = np.zeros_like(x)
    h = np.zeros_like(x)
    np.add.at(g, d, 2.0 * w * r)
    np.add.at(h, d, 2.0 * w)
    return float(np.sum(w * r * r)), g, h


def _dR_dA(prep, X, U, t, A):
    """∂R/∂A per A-dof: for each EI-scale beam group the element residual
    difference R_e(a=1) − R_e(a=0), scattered as (A index, X index, value)."""
    model, dis = prep.model, prep.dis
    rows, cols, vals = [], [], []
    c0 = REF.newmark_coefficients(0, 1.0, 0.25, 0.5)
    for g, dg in zip(model.groups, dis.dis):
        if g.nele == 0 or REF.group_kind(g) != "EulerBeam3D" or not dg.index_A.size:
            continue
        ia = dg.index_A[:, 0] - 1
        one, zero = np.array(A, dtype=float), np.array(A, dtype=float)
        one[ia] = 1.0
        zero[ia] = 0.0
        R1, _ = REF.eval_group(model, g, dg, (X,), U, t, 1, c0, A=one)
        R0, _ = REF.eval_group(model, g, dg, (X,), U, t, 1, c0, A=zero)
        D = R1 - R0  # (nele, 12)
        idx = dg.index_X - 1
        for e in range(g.nele):
            rows.append(np.full(idx.shape[1], ia[e]))
            cols.append(idx[e])
            vals.append(D[e])
    nA = len(A)
    if not rows:
        return sp.csr_matrix((nA, prep.n))
    return sp.csr_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))), shape=(nA, prep.n))


def directxua_static(model, dis, initialstate, times, sensors, w, y, maxiter=50, maxdx=1e-9, maxdl=1e-9):
    """The all-steps solve with A held: returns (C, dC/dA, states) where
    C = Σₙ Δt Σ_s w (xₙ[d_s] − yₙ,ₛ)² at the converged states, dC/dA the A-block
    of Lv, states the converged X (nstep × nX).  The time grid must be uniform
    (the reference takes a range); Δt = times[1] − times[0]."""
    times = np.asarray(times, dtype=float)
    nstep = len(times)
    dt = float(times[1] - times[0]) if nstep > 1 else float(times[0] - initialstate.time)
    prep = REF.Prepared(model, dis)
    n = prep.n
    U = tuple(u.copy() for u in initialstate.U)
    A = initialstate.A.copy()
    c0 = REF.newmark_coefficients(0, 1.0, 0.25, 0.5)
    X = [initialstate.X[0].copy() for _ in range(nstep)]
    Lam = [np.zeros(n) for _ in range(nstep)]
    for it in range(1, maxiter + 1):
        blocks, rhs = [], []
        for k, t in enumerate(times):
            R, nz = REF.assemble(prep, (X[k],), U, t, "static", c0, A=A)
            K = prep.matrix(nz)
            _, gC, hC = _sensor_terms(X[k], sensors, w, y[k])
            # Lv of step k: [Lλ; Lx] = Δt [R; Kᵀλ + ∇C];  Lvv = Δt [[0, K]; [Kᵀ, ∇²C]]
            rhs.append(dt * R)
            rhs.append(dt * (K.T @ Lam[k] + gC))
            blocks.append(sp.bmat([[None, dt * K], [dt * K.T, sp.diags(dt * hC)]], format="csc"))
        Lvv = sp.block_diag(blocks, format="csc")
        Lv = np.concatenate(rhs)
        try:
            dv = spla.splu(Lvv).solve(Lv)
        except RuntimeError as e:
            raise RuntimeError(f"matrix factorization failed at iiter={it}") from e
        dl2 = dx2 = 0.0
        for k in range(nstep):
            dl = dv[2 * k * n:(2 * k + 1) * n]
            dx = dv[(2 * k + 1) * n:(2 * k + 2) * n]
            Lam[k] -= dl
            X[k] -= dx
            dl2 = max(dl2, float(np.sum(dl**2)))
            dx2 = max(dx2, float(np.sum(dx**2)))
        if dx2 <= maxdx**2 and dl2 <= maxdl**2:
            break
        if it == maxiter:
            raise REF.NoConvergence(f"DirectXUA: no convergence after {it} iterations")
    C = 0.0
    gA = np.zeros(len(A))
    for k, t in enumerate(times):
        Ck, _, _ = _sensor_terms(X[k], sensors, w, y[k])
        C += dt * Ck
        gA += dt * (_dR_dA(prep, X[k], U, t, A) @ Lam[k])
    return C, gA, np.stack(X)
