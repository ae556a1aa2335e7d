"""Forward sensitivities on the device (GPU), the forward-mode counterpart of
the adjoint (SweepXA's sensitivity system, src/SweepXA.jl:49-221, on the
Newmark discretisation of SweepX).

* The cost gradient at a few A-dofs from the forward sensitivities equals the
  adjoint's gradient there (both are exact derivatives of the same discrete
  sweep): 1e-8 relative, Newmark and static, with cost elements (sensors, a
  velocity sensor, A-costs) and sensor arrays together.
* The state sensitivities dX/dA equal central differences of the device's
  forward sweep: 1e-5 relative to their largest value (h = 1e-5).
"""
import numpy as np
import pytest

from muscade_gpu import _lib
from muscade_gpu import workloads as W
from muscade_gpu.device import DeviceModel
from muscade_gpu.elements import QuadraticCost, SingleDofCost

pytestmark = pytest.mark.gpu
MAXDX = 1e-5  # above the multipliers' rounding floor


@pytest.fixture(scope="module", autouse=True)
def built():
    _lib.build()


def _model(nel=12, nstep=10, velocity=True, load_std=1e3):
    d0 = W.adjoint_beam(nel=nel, nstep=nstep, load_std=load_std)
    rng = np.random.default_rng(21)
    y = rng.normal(size=(nstep, len(d0["sensors"]))) * 1e-7
    d = W.adjoint_beam(nel=nel, nstep=nstep, load_std=load_std, measurements=(y, 1e-6), a_weight=2.0)
    if velocity:
        d["model"].addelement(SingleDofCost, [d["nodes"][nel // 2]], cls="X", field="t2", derivative=1,
                              cost=QuadraticCost(1e8, lambda t: 1e-6 * t))
    # extra sensor arrays on two dofs
    d["arr_dof"] = np.array([d0["sensors"][0], d0["sensors"][-1]])
    d["arr_y"] = rng.normal(size=(nstep, 2)) * 1e-7
    return d


@pytest.mark.parametrize("OX", [2, 0])
def test_forward_sensitivities_equal_the_adjoint_gradient(OX):
    d = _model(velocity=OX == 2, load_std=1e3 if OX == 2 else 1e5)
    m = d["model"]
    st = m.initialize(time=0.0) if OX == 2 else m.initialize()
    dm = DeviceModel(m, st.dis)
    dm.set_A(d["A_true"])
    kw = dict(cost_dof=d["arr_dof"], cost_w=1e12, cost_y=d["arr_y"], maxdx=MAXDX)
    C, gA, _, _ = dm.adjoint(OX, d["times"], st.time, list(st.X), **kw)
    sel = np.array([2, 5, 11])
    dC, _, stats = dm.sensitivity(OX, d["times"], st.time, list(st.X), sel, **kw)
    dm.close()
    assert stats.nstep_done == len(d["times"])
    ref = gA[sel - 1]
    print(f"OX={OX}: forward {dC}, adjoint {ref}")
    assert np.max(np.abs(dC - ref)) <= 1e-8 * np.max(np.abs(ref)), (dC, ref)


def test_state_sensitivities_match_central_differences():
    d = _model(nstep=6)
    m = d["model"]
    st = m.initialize(time=0.0)
    dm = DeviceModel(m, st.dis)
    A0 = np.asarray(d["A_true"], dtype=float)
    dm.set_A(A0)
    theta = 4
    _, dX, _ = dm.sensitivity(2, d["times"], st.time, list(st.X), [theta], maxdx=MAXDX, states=True)
    h = 1e-5
    out = []
    for sgn in (1, -1):
        A = A0.copy()
        A[theta - 1] += sgn * h
        dm.set_A(A)
        rc, S, _ = dm.sweepx(2, d["times"], st.time, list(st.X), maxdx=MAXDX)
        assert rc == 0
        out.append(S)
    dm.close()
    fd = (out[0] - out[1]) / (2 * h)  # [nstep][3][nX]
    lam = np.array([str(f).startswith("λ") for f in st.dis.fieldX])
    for k in range(3):
        a = dX[:, 0, k][:, ~lam]
        b = fd[:, k][:, ~lam]
        err = np.max(np.abs(a - b)) / np.max(np.abs(b))
        print(f"derivative {k}: max rel err {err:.2e}")
        assert err <= 1e-5, (k, err)
