"""The oracle's restatement of DirectXUA (oracle/direct.py) against the
reference's own DirectXUA tests, restated here:

* test/TestDirectXUA001.jl:33-51 -- static identification (DirectXUA{0,0,1})
  of a point held by two 2D springs that share their A-dofs (rest length and
  stiffness exponents), loaded by DofLoads, observed by SingleDofCosts and
  regularised by SingleAcosts, over 11 steps of 0.1: the state of step 2 and
  A, at the reference's rtol 1e-4 (Julia's ≈: norm of the difference).
* test/TestDirectXUA.jl:56-108 -- the step blocks L1/L2 of AssemblyDirect{2,0,1}
  for El1 oscillators coupled by a 1D spring, with SingleUdof loads,
  SingleDofCost measurements and tiny SingleAcosts, at the zero state of step
  6 (t = 6).  The golden numbers are those of the reference test file.
"""
import math

import numpy as np
import pytest

from conftest import julia_isapprox
from muscade_gpu.elements import DofLoad, Hold
from muscade_gpu.model import Model
from oracle import direct as DX


def test_directxua001_static_identification():
    m = Model("TestModel")
    n1 = m.addnode([0.0, 0.0])
    n2 = m.addnode([10.0, 0.0])
    n3 = m.addnode([0.0, 10.0])
    n4 = m.addnode(np.zeros(0))  # A-node of the springs
    m.addelement(DX.Spring, [n1, n2, n4], EA=10.0)
    m.addelement(DX.Spring, [n1, n3, n4], EA=10.0)

    def load(t):
        return 0.1 * t

    m.addelement(DofLoad, [n1], field="tx1", value=load)
    m.addelement(DofLoad, [n1], field="tx2", value=load)
    for nod, f in ((n2, "tx1"), (n2, "tx2"), (n3, "tx1"), (n3, "tx2")):
        m.addelement(Hold, [nod], field=f)

    def position_meas(x, t):
        return 0.5 * ((x - 0.12 * t) / 0.01) ** 2

    def acost(a):
        return 0.5 * (a / 0.1) ** 2

    m.addelement(DX.SingleDofCost, [n1], cls="X", field="tx1", cost=position_meas)
    m.addelement(DX.SingleDofCost, [n1], cls="X", field="tx2", cost=position_meas)
    m.addelement(DX.SingleAcost, [n4], field="ΞL₀", cost=acost)
    m.addelement(DX.SingleAcost, [n4], field="ΞEI", cost=acost)
    st = m.initialize()
    # solve(SweepX{0}; time=[0.]) leaves this model at zero (no load at t = 0,
    # springs at rest), so the DirectXUA starts from the initial state
    states, A, _ = DX.directxua(m, st.dis, st, np.arange(11) * 0.1, OX=0, OU=0, IA=1, maxiter=50)
    gold_X = [0.0154897, 0.0154897, 0.0, 0.0, 0.0, 0.0, -0.0100155, 1.55379e-5, 1.55379e-5, -0.0100155]
    gold_A = [-0.000195471, -0.0400374]
    assert julia_isapprox(states[1].X[0], gold_X, rtol=1e-4)
    assert julia_isapprox(A, gold_A, rtol=1e-4)


def _el1_model():
    m = Model("TrueModel")
    n1 = m.addnode([0.0])
    n2 = m.addnode([1.0])
    n3 = m.addnode(np.zeros(0))  # A-node of the spring
    m.addelement(DX.El1, [n1], K=1.0, C=0.05, M=1.0)
    m.addelement(DX.El1, [n2], K=0.0, C=0.0, M=1.0)
    m.addelement(DX.Spring, [n1, n2, n3], EA=1.1, D=1)

    def fa(a):
        return a * a * 1e-14

    def fu(u, t):
        return u * u

    def l1(x, t):
        return (x - 0.1 * math.sin(t)) ** 2

    def l2(x, t):
        return (x - 0.1 * math.cos(t)) ** 2

    for nod, f in ((n3, "ΞL₀"), (n3, "ΞEI"), (n1, "ΞC"), (n1, "ΞM"), (n2, "ΞC"), (n2, "ΞM")):
        m.addelement(DX.SingleAcost, [nod], field=f, cost=fa)
    m.addelement(DX.SingleUdof, [n1], Xfield="tx1", Ufield="utx1", cost=fu)
    m.addelement(DX.SingleUdof, [n2], Xfield="tx1", Ufield="utx1", cost=fu)
    m.addelement(DX.SingleDofCost, [n1], cls="X", field="tx1", cost=l1)
    m.addelement(DX.SingleDofCost, [n2], cls="X", field="tx1", cost=l2)
    return m


def test_direct_step_blocks():
    m = _el1_model()
    st = m.initialize()
    assert m.ndof == {"X": 2, "U": 4, "A": 6}
    nX, nU, nA = 2, 4, 6
    OX, OU, IA = 2, 0, 1
    X = [np.zeros(nX) for _ in range(OX + 1)]
    U = [np.zeros(nU)]
    L1, L2 = DX.assemble_step(m, st.dis, np.zeros(nX), X, U, np.zeros(nA), 6.0, OX, OU, IA)
    close = lambda a, b: julia_isapprox(np.asarray(a, float), np.asarray(b, float))  # noqa: E731
    # L1[α][αder]
    assert close(L1["L"][0], [0.0, 0.0])
    assert close(L1["X"][0], [0.055883099639785175, -0.1920340573300732])
    assert close(L1["X"][1], [0.0, 0.0]) and close(L1["X"][2], [0.0, 0.0])
    assert close(L1["U"][0], np.zeros(4)) and close(L1["A"][0], np.zeros(6))
    # L2[α,β][αder,βder] (dense here, sparse in the reference)
    assert close(L2[("X", "X", 0, 0)], [[2.0, 0.0], [0.0, 2.0]])
    assert close(L2[("X", "X", 0, 1)], np.zeros((2, 2))) and close(L2[("X", "X", 0, 2)], np.zeros((2, 2)))
    assert close(L2[("X", "L", 0, 0)], [[2.1, -1.1], [-1.1, 1.1]])
    assert close(L2[("X", "L", 1, 0)], [[0.05, 0.0], [0.0, 0.0]])
    assert close(L2[("X", "L", 2, 0)], [[1.0, 0.0], [0.0, 1.0]])
    assert close(L2[("U", "U", 0, 0)], np.diag([0.0, 0.0, 2.0, 2.0]))
    assert close(L2[("U", "A", 0, 0)], np.zeros((4, 6)))
    assert close(L2[("A", "A", 0, 0)], np.diag([2e-14] * 6))


def test_big_system_pattern():
    """preparebig of test/TestDirectXUA.jl:109-136 (6 steps, OX=2, OU=0, IA=1):
    size, the first 50 column pointers and 60 row indices of Lvv, and the
    first entry of every block of Lv."""
    m = _el1_model()
    st = m.initialize()
    colptr, rowval, lvasm = DX.big_pattern(m, st.dis, OX=2, OU=0, IA=1, nstep=6)
    assert len(colptr) - 1 == 54
    assert list(colptr[:50]) == [1, 13, 25, 43, 61, 68, 75, 80, 85, 97, 109, 133, 157, 164, 171, 176, 181, 193, 205, 235,
                                 265, 272, 279, 284, 289, 301, 313, 343, 373, 380, 387, 392, 397, 409, 421, 445, 469,
                                 476, 483, 488, 493, 505, 517, 535, 553, 560, 567, 572, 577, 597]
    assert list(rowval[:60]) == [3, 4, 5, 7, 11, 12, 19, 20, 49, 50, 53, 54, 3, 4, 6, 8, 11, 12, 19, 20, 51, 52, 53, 54,
                                 1, 2, 3, 4, 5, 7, 9, 10, 11, 12, 13, 15, 19, 20, 49, 50, 53, 54, 1, 2, 3, 4, 6, 8, 9,
                                 10, 11, 12, 14, 16, 19, 20, 51, 52, 53, 54]
    assert list(lvasm) == [1, 3, 5, 9, 11, 13, 17, 19, 21, 25, 27, 29, 33, 35, 37, 41, 43, 45, 49]


def test_reference_path_without_second_order_does_not_settle_the_multipliers():
    """EulerBeam3D declares no second order; the reference's DirectXUA then
    leaves (∂R/∂X)ᵀΛ out of Lx (src/DirectXUA.jl:85-120).  On a static beam
    identification the states converge while every iteration decrements Λ by
    the same K⁻ᵀ∇cost, so the default convergence test on ΔΛ (1e-5) is never
    met.  This is why the device differentiates SweepX itself (the discrete
    adjoint) rather than reproducing DirectXUA for beams."""
    from muscade_gpu import workloads as W
    from oracle import reference as REF

    d = W.adjoint_beam(nel=10, nstep=4, seed=2029, load_std=1e5)
    m = d["model"]
    st = m.initialize()
    st.A[:] = 1.0
    ref = REF.sweepx(m, st.dis, st, d["times"], OX=0, maxdx=1e-5)
    y = np.stack([X[0][d["sensors"] - 1] for _, X in ref]) + 1e-3
    it = DX.static_path_without_second_order(m, st.dis, st, d["times"], d["sensors"], y, 8)
    dls = np.array([dl for dl, _ in it])
    assert it[-1][1] < 1e-5  # the states have converged
    assert np.all(dls > 1e-5) and np.max(np.abs(dls[2:] - dls[-1])) <= 1e-9 * dls[-1]  # a constant ΔΛ
