"""Adjoint sensitivities on the device against central finite differences.

The cost is a sum of squared sensor misfits (SingleDofCost-type terms,
src/BasicElements.jl:198-208) over a SweepX trajectory; its gradient with
respect to the EI-scale A-dofs and to the load values comes from
mgpu_adjoint_sweepx and is compared with central differences of the same
device forward sweep (bar: 1e-6 relative to the largest checked component).
"""
import math

import numpy as np
import pytest

from muscade_gpu import workloads as W
from muscade_gpu.device import DeviceModel
from oracle import reference as REF

pytestmark = pytest.mark.gpu

MAXDX = 1e-7
TOL_FD = 1e-6


def _problem(nel=30, nstep=20, seed=2029):
    d = W.adjoint_beam(nel=nel, nstep=nstep, seed=seed)
    m = d["model"]
    st = m.initialize(time=0.0)
    dm = DeviceModel(m, st.dis)
    dm.set_A(d["A_true"])
    rc, states, _ = dm.sweepx(2, d["times"], st.time, list(st.X), maxdx=MAXDX)
    assert rc == 0
    y, sd = W.synthetic_measurements(states, d["sensors"])
    d.update(st=st, dm=dm, y=y, w=1.0 / sd**2)
    return d


def _cost(d, A, OX=2):
    dm, st = d["dm"], d["st"]
    dm.set_A(A)
    rc, states, _ = dm.sweepx(OX, d["times"], st.time, list(st.X), maxdx=MAXDX)
    assert rc == 0
    r = states[:, 0, d["sensors"] - 1] - d["y"]
    wt = np.diff(np.concatenate([[st.time], d["times"]])) if OX == 2 else np.ones(len(d["times"]))
    return float(np.sum(wt * np.sum(d["w"] * r * r, axis=1)))


def test_ei_scaled_beams_match_oracle():
    d = W.adjoint_beam(nel=12, nstep=6)
    m = d["model"]
    st = m.initialize(time=0.0)
    st.A[:] = d["A_true"]
    from muscade_gpu import SweepXGPU, solve

    out = solve(SweepXGPU[2], st, d["times"], maxdx=1e-9)
    ref = REF.sweepx(m, st.dis, st, d["times"], OX=2, maxdx=1e-9)
    for s, (t, Xr) in zip(out, ref):
        for k in range(3):
            sel = np.array([not str(f).startswith("λ") for f in st.dis.fieldX])
            scale = max(np.max(np.abs(Xr[k][sel])), 1e-300)
            assert np.max(np.abs(s.X[k][sel] - Xr[k][sel])) <= 1e-9 * scale


def test_newmark_adjoint_matches_central_differences():
    d = _problem()
    dm, st = d["dm"], d["st"]
    A0 = np.ones(dm.nA)
    dm.set_A(A0)
    C, gA, gF, stats = dm.adjoint(2, d["times"], st.time, list(st.X), d["sensors"], d["w"], d["y"], maxdx=MAXDX,
                                  ckpt=0, load_gradient=True)
    assert C == pytest.approx(_cost(d, A0), rel=1e-12)
    rng = np.random.default_rng(3)
    idx = rng.choice(dm.nA, 6, replace=False)
    h = 1e-4
    fd = []
    for i in idx:
        Ap, Am = A0.copy(), A0.copy()
        Ap[i] += h
        Am[i] -= h
        fd.append((_cost(d, Ap) - _cost(d, Am)) / (2 * h))
    fd = np.array(fd)
    assert np.max(np.abs(gA[idx] - fd)) <= TOL_FD * np.max(np.abs(fd)), (gA[idx], fd)
    # load values: perturb one entry of the load table (the DofLoad functions read it);
    # gF follows the tvals layout, where the Hold offsets come first
    dm.set_A(A0)
    tbl = d["loads"]
    off = sum(g.nele for g in d["model"].groups if g.key[0] == "DofConstraint")
    checks = [(3, 5), (10, 12), (19, 20)]
    fdF, adF = [], []
    for k, j in checks:
        hF = 1e-2
        tbl[k, j] += hF
        cp = _cost(d, A0)
        tbl[k, j] -= 2 * hF
        cm = _cost(d, A0)
        tbl[k, j] += hF
        fdF.append((cp - cm) / (2 * hF))
        adF.append(gF[k, off + j])
    fdF, adF = np.array(fdF), np.array(adF)
    assert np.max(np.abs(adF - fdF)) <= TOL_FD * np.max(np.abs(fdF)), (adF, fdF)
    dm.close()


def test_checkpoint_interval_does_not_change_the_gradient():
    d = _problem(nel=16, nstep=12)
    dm, st = d["dm"], d["st"]
    dm.set_A(np.ones(dm.nA))
    res = [dm.adjoint(2, d["times"], st.time, list(st.X), d["sensors"], d["w"], d["y"], maxdx=MAXDX, ckpt=c)
           for c in (1, 0, 5, 12)]
    for C, g, _, _ in res[1:]:
        assert C == res[0][0] and np.array_equal(g, res[0][1])
    dm.close()


def test_static_adjoint_matches_central_differences():
    d = W.adjoint_beam(nel=20, nstep=4, load_std=1e5)
    m = d["model"]
    st = m.initialize()
    dm = DeviceModel(m, st.dis)
    dm.set_A(d["A_true"])
    rc, states, _ = dm.sweepx(0, d["times"], st.time, list(st.X), maxdx=MAXDX)
    assert rc == 0
    y, sd = W.synthetic_measurements(states, d["sensors"])
    d.update(st=st, dm=dm, y=y, w=1.0 / sd**2)
    A0 = np.ones(dm.nA)
    dm.set_A(A0)
    C, gA, _, _ = dm.adjoint(0, d["times"], st.time, list(st.X), d["sensors"], d["w"], y, maxdx=MAXDX)
    assert C == pytest.approx(_cost(d, A0, OX=0), rel=1e-12)
    idx = np.array([0, 7, 13, 19])
    h = 1e-4
    fd = []
    for i in idx:
        Ap, Am = A0.copy(), A0.copy()
        Ap[i] += h
        Am[i] -= h
        fd.append((_cost(d, Ap, OX=0) - _cost(d, Am, OX=0)) / (2 * h))
    fd = np.array(fd)
    assert np.max(np.abs(gA[idx] - fd)) <= TOL_FD * np.max(np.abs(fd)), (gA[idx], fd)
    dm.close()


def test_static_adjoint_matches_directxua():
    """The device static adjoint against the all-steps restatement
    (oracle/directxua.py): both are the stationarity conditions of
    Σ cost + Λ·R with the loads given and A held, so the gradients agree to
    rounding.  The restatement weighs every step by Δt, the static adjoint by 1."""
    from oracle import directxua as DX
    from test_directxua import MAXDX as MAXDX_DX
    from test_directxua import _problem as dx_problem

    d = dx_problem()
    m, st = d["model"], d["st"]
    A0 = np.ones(len(st.A))
    s = st.copy()
    s.A = A0.copy()
    C_dx, g_dx, X_dx = DX.directxua_static(m, s.dis, s, d["times"], d["sensors"], d["w"], d["y"], maxdx=MAXDX_DX,
                                          maxdl=np.inf)
    dm = DeviceModel(m, st.dis)
    dm.set_A(A0)
    C, gA, _, _ = dm.adjoint(0, d["times"], s.time, list(s.X), d["sensors"], d["w"], d["y"], maxdx=MAXDX_DX)
    dm.close()
    assert d["dt"] * C == pytest.approx(C_dx, rel=1e-9)
    assert np.max(np.abs(d["dt"] * gA - g_dx)) <= 1e-8 * np.max(np.abs(g_dx))
