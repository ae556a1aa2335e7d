"""DirectXUA restatement (oracle/directxua.py) on the CPU: its A-block
gradient against central differences of the oracle's SweepX{0} cost, and
its converged states against SweepX{0} (static, loads given, A held)."""
import numpy as np
import pytest

from muscade_gpu import workloads as W
from oracle import directxua as DX
from oracle import reference as REF

# absolute, like the reference: X holds the Hold reactions (about 1e5 N), whose
# rounding stalls Newton near 1e-6; one iteration past 1e-5 is converged to rounding
MAXDX = 1e-5


def _problem(nel=10, nstep=4, seed=2029):
    d = W.adjoint_beam(nel=nel, nstep=nstep, seed=seed, load_std=1e5)
    m = d["model"]
    st = m.initialize()
    st.A[:] = d["A_true"]
    ref = REF.sweepx(m, st.dis, st, d["times"], OX=0, maxdx=MAXDX)
    states = np.stack([np.stack(X) for _, X in ref])
    y, sd = W.synthetic_measurements(states, d["sensors"])
    d.update(st=st, y=y, w=1.0 / sd**2, dt=float(d["times"][1] - d["times"][0]))
    return d


def _sweep_cost(d, A):
    m, st = d["model"], d["st"]
    s = st.copy()
    s.A = np.array(A, dtype=float)
    ref = REF.sweepx(m, s.dis, s, d["times"], OX=0, maxdx=MAXDX)
    X = np.stack([X[0] for _, X in ref])
    r = X[:, d["sensors"] - 1] - d["y"]
    return d["dt"] * float(np.sum(d["w"] * r * r)), X


def test_directxua_gradient_matches_central_differences():
    d = _problem()
    m, st = d["model"], d["st"]
    A0 = np.ones(len(st.A))
    s = st.copy()
    s.A = A0.copy()
    # Λ is exact one iteration after X has converged (the λ rows of the Newton
    # system are K Δx = R), so the X criterion alone decides
    C, gA, X = DX.directxua_static(m, s.dis, s, d["times"], d["sensors"], d["w"], d["y"], maxdx=MAXDX,
                                   maxdl=np.inf)
    C_sweep, X_sweep = _sweep_cost(d, A0)
    assert C == pytest.approx(C_sweep, rel=1e-9)
    assert np.max(np.abs(X - X_sweep)) <= 1e-9 * np.max(np.abs(X_sweep))
    idx = np.array([0, 3, 6, 9])
    h = 1e-4
    fd = []
    for i in idx:
        Ap, Am = A0.copy(), A0.copy()
        Ap[i] += h
        Am[i] -= h
        fd.append((_sweep_cost(d, Ap)[0] - _sweep_cost(d, Am)[0]) / (2 * h))
    fd = np.array(fd)
    assert np.max(np.abs(gA[idx] - fd)) <= 1e-6 * np.max(np.abs(fd)), (gA[idx], fd)
