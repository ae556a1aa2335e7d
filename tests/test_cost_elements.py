"""Cost and A-dof elements on the host side (CPU): SingleDofCost, SingleUdof
and SingleAcost (src/BasicElements.jl:32-50,77-86,163-167,198-208,239-248)
built through addelement, their dofs, the oracle's SweepX residuals of
Lagrangian elements (R = ∂L/∂Λ, src/Assemble.jl:661-677), the oracle's cost
of a trajectory, and the DirectXUA restatement evaluating the package's cost
elements by its own restatements.
"""
import numpy as np
import pytest

from muscade_gpu import workloads as W
from muscade_gpu.elements import DofLoad, Hold, QuadraticCost, SingleAcost, SingleDofCost, SingleUdof
from muscade_gpu.model import Model, MuscadeError
from oracle import direct as D
from oracle import reference as REF


def _cantilever_with(extra):
    m, times = W.cantilever(nel=8)
    extra(m)
    return m, times


def test_dofs_and_groups():
    m, _ = W.cantilever(nel=4)
    tip = m.nnod
    m.addelement(SingleUdof, [tip], Xfield="t3", Ufield="ut3", cost=QuadraticCost(2.0, 0.0))
    m.addelement(SingleDofCost, [tip], cls="X", field="t3", cost=QuadraticCost(1.0, lambda t: 0.1 * t))
    m.addelement(SingleDofCost, [tip], cls="X", field="t2", cost=QuadraticCost(1.0, 0.0), derivative=2)
    a = m.addnode([0.0, 0.0, 1.0])
    m.addelement(SingleAcost, [a], field="EIscale", cost=QuadraticCost(3.0, 1.0))
    st = m.initialize()
    assert m.ndof["U"] == 1 and m.ndof["A"] == 1
    keys = [g.key[0] for g in m.groups]
    assert keys.count("SingleDofCost") == 2  # one concrete type per field and derivative
    dg = st.dis.dis[keys.index("SingleUdof")]
    assert dg.index_X.shape == (1, 1) and dg.index_U.shape == (1, 1)
    assert st.dis.dis[keys.index("SingleAcost")].index_X.shape == (1, 0)
    with pytest.raises(MuscadeError):
        W.cantilever(nel=2)[0].addelement(SingleDofCost, [1], cls="A", field="t1", cost=QuadraticCost())


def test_singleudof_is_a_load_and_costs_leave_sweepx_unchanged():
    """SweepX holds U from the initial state: a SingleUdof with u applies the
    load −u like a DofLoad of value u, and cost elements add R = 0."""
    u = 5.0

    def with_udof(m):
        m.addelement(SingleUdof, [m.nnod], Xfield="t2", Ufield="ut2", cost=QuadraticCost(1.0, 0.0))
        m.addelement(SingleDofCost, [m.nnod], cls="X", field="t3", cost=QuadraticCost(5.0, 1.0))
        m.addelement(SingleAcost, [m.addnode([0.0, 1.0, 0.0])], field="EIscale", cost=QuadraticCost(1.0, 1.0))

    def with_load(m):
        m.addelement(DofLoad, [m.nnod], field="t2", value=lambda t: u)

    mu, times = _cantilever_with(with_udof)
    su = mu.initialize()
    su.U[0][:] = u
    ml, _ = _cantilever_with(with_load)
    sl = ml.initialize()
    ru = REF.sweepx(mu, su.dis, su, times[:4], OX=0, maxdx=1e-10)
    rl = REF.sweepx(ml, sl.dis, sl, times[:4], OX=0, maxdx=1e-10)
    for (_, Xu), (_, Xl) in zip(ru, rl):
        assert np.array_equal(Xu[0], Xl[0])


def test_sweep_cost_of_a_trajectory():
    d = W.adjoint_beam(nel=10, nstep=6)
    rng = np.random.default_rng(5)
    y = rng.normal(size=(6, len(d["sensors"]))) * 1e-4
    d = W.adjoint_beam(nel=10, nstep=6, measurements=(y, 1e-3), a_weight=4.0)
    m = d["model"]
    st = m.initialize(time=0.0)
    st.A[:] = d["A_true"]
    traj = [(t, (rng.normal(size=m.ndof["X"]), rng.normal(size=m.ndof["X"]), rng.normal(size=m.ndof["X"])))
            for t in d["times"]]
    C = REF.sweep_cost(m, st.dis, traj, 0.0, 2, st.U, st.A)
    dt = np.diff(np.concatenate([[0.0], d["times"]]))
    X0 = np.stack([X[0] for _, X in traj])
    ref = float(np.sum(dt * np.sum((X0[:, d["sensors"] - 1] - y) ** 2, axis=1)) / 1e-6)
    ref += 4.0 * float(np.sum((d["A_true"] - 1.0) ** 2))
    assert C == pytest.approx(ref, rel=1e-12)


def test_direct_restatement_evaluates_package_cost_elements():
    """The DirectXUA restatement's step blocks for a model of the package's
    cost elements: ∂L/∂x⁽ᵈ⁾ = 2w(x⁽ᵈ⁾ − y), ∂²L = 2w; SingleUdof ∂L/∂Λ = −u,
    ∂L/∂u = 2w(u − y) − Λ, ∂²L/∂Λ∂u = −1; the A-costs once per step."""
    m = Model("costs")
    tip = m.addnode([1.0, 0.0, 0.0])
    m.addelement(Hold, [tip], field="t1")
    m.addelement(SingleDofCost, [tip], cls="X", field="t3", cost=QuadraticCost(2.0, 0.5), derivative=1)
    m.addelement(SingleUdof, [tip], Xfield="t2", Ufield="ut2", cost=QuadraticCost(3.0, 0.25))
    a = m.addnode([0.0, 0.0, 2.0])
    m.addelement(SingleAcost, [a], field="EIscale", cost=QuadraticCost(7.0, 1.0))
    st = m.initialize()
    nX = m.ndof["X"]
    rng = np.random.default_rng(9)
    Lam = rng.normal(size=nX)
    X = [rng.normal(size=nX) for _ in range(3)]
    U = [np.array([0.8])]
    A = np.array([1.3])
    L1, L2 = D.assemble_step(m, st.dis, Lam, X, U, A, 0.0, 2, 0, 1)
    keys = [g.key[0] for g in m.groups]
    ix = st.dis.dis[keys.index("SingleDofCost")].index_X[0, 0] - 1
    iu = st.dis.dis[keys.index("SingleUdof")].index_X[0, 0] - 1
    assert L1["X"][1][ix] == pytest.approx(2 * 2.0 * (X[1][ix] - 0.5), rel=1e-14)
    assert L2[("X", "X", 1, 1)][ix, ix] == pytest.approx(4.0, rel=1e-14)
    assert L1["U"][0][0] == pytest.approx(2 * 3.0 * (0.8 - 0.25) - Lam[iu], rel=1e-14)
    assert L2[("L", "U", 0, 0)][iu, 0] == -1.0 and L2[("U", "L", 0, 0)][0, iu] == -1.0
    assert L1["A"][0][0] == pytest.approx(2 * 7.0 * 0.3, rel=1e-14)
    g1, h1 = D.assemble_A(m, st.dis, A)
    assert g1[0] == pytest.approx(2 * 7.0 * 0.3, rel=1e-14) and h1[0, 0] == 14.0
