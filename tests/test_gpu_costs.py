"""Cost and A-dof element groups on the device (GPU): SingleDofCost,
SingleUdof and SingleAcost with quadratic costs
(src/BasicElements.jl:32-50,77-86,163-167,198-208,239-248).

* Element Lagrangians, gradients and Hessians over (Λ, X, X′, X″, U, A), the
  per-element terms DirectXUA adds into its step blocks: equal to the oracle's
  second-order-dual restatement (oracle/direct.py) to 1e-14.
* SweepX{2} of a beam with sensors, A-costs and SingleUdof loads: states within
  1e-9 of the oracle's sweep (the U-dof value is a load, the costs add R = 0).
* The adjoint with its cost taken from the element groups: the cost equals the
  oracle's cost of the oracle's trajectory, and dC/dA, dC/dU and dC/dy agree
  with central differences of the oracle's cost (bar 1e-6 relative).
"""
import numpy as np
import pytest

from muscade_gpu import _lib
from muscade_gpu import workloads as W
from muscade_gpu.device import DeviceError, DeviceModel
from muscade_gpu.elements import (DofConstraint, DofLoad, Hold, QuadraticCost, SingleAcost, SingleDofCost, SingleUdof,
                                  group_time_values)
from muscade_gpu.model import Model
from oracle import direct as D
from oracle import lib as O
from oracle import reference as REF

pytestmark = pytest.mark.gpu
MAXDX = 1e-5  # above the multipliers' rounding floor (about 5e-7 N for these beams)
TOL_FD = 1e-6


@pytest.fixture(scope="module", autouse=True)
def built():
    _lib.build()
    O.build()


def test_element_lagrangians_match_the_restatement():
    m = Model("lagrangians")
    n = m.addnode(np.array([[0.0, 0, 0], [1, 0, 0], [2, 0, 0], [0, 1, 0]]))
    m.addelement(DofLoad, n[:2, None], field="t1", value=lambda t: np.array([3.0 * t, -2.0]))
    m.addelement(Hold, n[:3, None], field="t2")
    m.addelement(DofConstraint, np.array([[n[0], n[1]]]), xinod=(1, 2), xfield=("t1", "t1"), lfield="λgap",
                 coeffs=[1.0, -2.0], offset=lambda t: 0.1 * t)
    m.addelement(SingleDofCost, n[:2, None], cls="X", field="t3", cost=QuadraticCost(2.5, lambda t: 0.2 * t))
    m.addelement(SingleDofCost, [n[1]], cls="X", field="r1", cost=QuadraticCost(0.5, 1.0), derivative=2)
    m.addelement(SingleUdof, n[1:3, None], Xfield="t3", Ufield="ut3", cost=QuadraticCost(4.0, -0.3))
    m.addelement(SingleAcost, [n[3]], field="EIscale", cost=QuadraticCost(7.0, 1.1))
    st = m.initialize()
    dm = DeviceModel(m, st.dis)
    rng = np.random.default_rng(11)
    t = 0.7
    for ig, (g, dg) in enumerate(zip(m.groups, st.dis.dis)):
        nele, nX = dg.index_X.shape
        nU = dg.index_U.shape[1] if dg.index_U.ndim == 2 else 0
        nA = dg.index_A.shape[1] if dg.index_A.ndim == 2 else 0
        lam = rng.normal(size=(nele, nX))
        X = rng.normal(size=(nele, 3, nX))
        U = rng.normal(size=(nele, nU))
        A = rng.normal(size=(nele, nA))
        Lv, dL, d2L = dm.element_lagrangian(ig, lam, X, U, A, t=t)
        lay = D.Layout(nX, nU, nA, 2, 0, 1)
        params = D._params(g)
        kind = g.key[0]
        for e in range(nele):
            p = params[e]
            if kind == "DofLoad":
                p = {"F": group_time_values(g, "value", t)[e]}
            elif kind == "DofConstraint":
                p = {"off": group_time_values(g, "offset", t)[e], "coeffs": g.cat("coeffs")[e]}
            Le = D.element_lagrangian(g, g.key, p, lam[e], [X[e, i] for i in range(3)], [U[e]], A[e], t, lay)
            scale = max(1.0, np.max(np.abs(Le.g)), np.max(np.abs(Le.h)))
            assert abs(Lv[e] - Le.v) <= 1e-14 * max(1.0, abs(Le.v)), (kind, e)
            assert np.max(np.abs(dL[e] - Le.g)) <= 1e-14 * scale, (kind, e)
            assert np.max(np.abs(d2L[e] - Le.h)) <= 1e-14 * scale, (kind, e)
    dm.close()


def _identification(nel=12, nstep=10, a_weight=1.0, seed=2029):
    """A beam of the identification workload with its sensors and A-costs as
    elements, a velocity sensor, and SingleUdof loads at three nodes."""
    d0 = W.adjoint_beam(nel=nel, nstep=nstep, seed=seed)
    rng = np.random.default_rng(17)
    y = rng.normal(size=(nstep, len(d0["sensors"]))) * 1e-7
    d = W.adjoint_beam(nel=nel, nstep=nstep, seed=seed, measurements=(y, 1e-6), a_weight=a_weight)
    m = d["model"]
    nodes = d["nodes"]
    m.addelement(SingleDofCost, [nodes[nel // 2]], cls="X", field="t2", derivative=1,
                 cost=QuadraticCost(1e8, lambda t: 1e-6 * t))
    m.addelement(SingleUdof, nodes[[2, nel // 2, nel - 2]][:, None], Xfield="t2", Ufield="ut2",
                 cost=QuadraticCost(1e-7, 5.0))
    st = m.initialize(time=0.0)
    st.A[:] = d["A_true"]
    st.U[0][:] = [40.0, -25.0, 10.0]
    d.update(st=st, y=y)
    return d


def _oracle_cost(d, A=None, U=None, OX=2):
    m, st = d["model"], d["st"]
    s = st.copy()
    if A is not None:
        s.A[:] = A
    if U is not None:
        s.U = (np.asarray(U, dtype=float),)
    traj = REF.sweepx(m, s.dis, s, d["times"], OX=OX, maxdx=MAXDX)
    return REF.sweep_cost(m, s.dis, traj, s.time, OX, s.U, s.A), traj


def test_sweepx_with_cost_and_udof_elements_matches_oracle():
    d = _identification()
    m, st = d["model"], d["st"]
    dm = DeviceModel(m, st.dis)
    dm.set_A(st.A)
    rc, states, _ = dm.sweepx(2, d["times"], st.time, list(st.X), U=st.U[0], maxdx=MAXDX)
    dm.close()
    assert rc == 0
    _, ref = _oracle_cost(d)
    lam = np.array([str(f).startswith("λ") for f in st.dis.fieldX])
    for k in range(3):
        dev = max(np.max(np.abs(states[i, k][~lam] - X[k][~lam])) for i, (_, X) in enumerate(ref))
        scale = max(np.max(np.abs(X[k][~lam])) for _, X in ref)
        assert dev <= 1e-9 * scale, (k, dev, scale)


def test_adjoint_of_element_costs_matches_oracle_differences():
    d = _identification()
    m, st = d["model"], d["st"]
    dm = DeviceModel(m, st.dis)
    A0 = st.A.copy()
    dm.set_A(A0)
    u0 = st.U[0].copy()
    C, gA, gtv, stats, gU = dm.adjoint(2, d["times"], st.time, list(st.X), U=u0, maxdx=MAXDX, load_gradient=True,
                                       u_gradient=True)
    dm.close()
    Cr, _ = _oracle_cost(d)
    assert C == pytest.approx(Cr, rel=1e-8)
    rng = np.random.default_rng(4)
    idx = rng.choice(len(A0), 3, replace=False)
    h = 1e-4
    fd = []
    for i in idx:
        Ap, Am = A0.copy(), A0.copy()
        Ap[i] += h
        Am[i] -= h
        fd.append((_oracle_cost(d, A=Ap)[0] - _oracle_cost(d, A=Am)[0]) / (2 * h))
    fd = np.array(fd)
    assert np.max(np.abs(gA[idx] - fd)) <= TOL_FD * np.max(np.abs(fd)), (gA[idx], fd)
    hu = 0.5
    fdu = []
    for j in range(len(u0)):
        up, um = u0.copy(), u0.copy()
        up[j] += hu
        um[j] -= hu
        fdu.append((_oracle_cost(d, U=up)[0] - _oracle_cost(d, U=um)[0]) / (2 * hu))
    fdu = np.array(fdu)
    assert np.max(np.abs(gU - fdu)) <= TOL_FD * np.max(np.abs(fdu)), (gU, fdu)
    # a sensor target: the cost is quadratic in it and the states do not depend on it
    keys = [g.key[0] for g in m.groups]
    off = 0
    for g in m.groups:
        if g.key[0] == "SingleDofCost":
            break
        if g.key[0] in ("DofLoad", "DofConstraint", "SingleUdof"):
            off += g.nele
    g0 = m.groups[keys.index("SingleDofCost")]
    rec = g0.data[0]["cost"][0].target
    k, hy = 4, 1e-8
    rec.values[k] += hy
    cp = _oracle_cost(d)[0]
    rec.values[k] -= 2 * hy
    cm = _oracle_cost(d)[0]
    rec.values[k] += hy
    assert gtv[k, off] == pytest.approx((cp - cm) / (2 * hy), rel=1e-6)


def test_element_costs_equal_sensor_arrays():
    """The same sensors as elements or as the sensor arrays: the same cost and
    gradient (summation order aside)."""
    d0 = W.adjoint_beam(nel=16, nstep=8)
    y = np.random.default_rng(2).normal(size=(8, len(d0["sensors"]))) * 1e-7
    sd = 1e-6
    dc = W.adjoint_beam(nel=16, nstep=8, measurements=(y, sd))
    out = []
    for d, arrays in ((d0, True), (dc, False)):
        st = d["model"].initialize(time=0.0)
        dm = DeviceModel(d["model"], st.dis)
        dm.set_A(d["A_true"])
        if arrays:
            r = dm.adjoint(2, d["times"], st.time, list(st.X), d["sensors"], 1.0 / sd**2, y, maxdx=MAXDX)
        else:
            r = dm.adjoint(2, d["times"], st.time, list(st.X), maxdx=MAXDX)
        dm.close()
        out.append(r)
    assert out[1][0] == pytest.approx(out[0][0], rel=1e-12)
    assert np.max(np.abs(out[1][1] - out[0][1])) <= 1e-11 * np.max(np.abs(out[0][1]))


def test_static_adjoint_of_element_costs():
    d = _identification(nel=10, nstep=3)
    m, st = d["model"], d["st"]
    # the velocity sensor needs OX = 2
    dm = DeviceModel(m, st.dis)
    dm.set_A(st.A)
    with pytest.raises(DeviceError) as e:
        dm.adjoint(0, d["times"], st.time, list(st.X), U=st.U[0], maxdx=MAXDX)
    assert e.value.kind == "argument"
    dm.close()
    d0 = W.adjoint_beam(nel=10, nstep=3, load_std=1e5)
    y = np.random.default_rng(8).normal(size=(3, len(d0["sensors"]))) * 1e-5
    d = W.adjoint_beam(nel=10, nstep=3, load_std=1e5, measurements=(y, 1e-5), a_weight=3.0)
    m = d["model"]
    st = m.initialize()
    st.A[:] = d["A_true"]
    d["st"] = st
    dm = DeviceModel(m, st.dis)
    dm.set_A(st.A)
    C, gA, _, _ = dm.adjoint(0, d["times"], st.time, list(st.X), maxdx=MAXDX)
    dm.close()
    assert C == pytest.approx(_oracle_cost(d, OX=0)[0], rel=1e-8)
    h = 1e-4
    for i in (1, 6):
        Ap, Am = st.A.copy(), st.A.copy()
        Ap[i] += h
        Am[i] -= h
        fd = (_oracle_cost(d, A=Ap, OX=0)[0] - _oracle_cost(d, A=Am, OX=0)[0]) / (2 * h)
        assert gA[i] == pytest.approx(fd, rel=TOL_FD)
