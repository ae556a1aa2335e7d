"""Element results on the device (GPU): getresult (src/Output.jl:131-181) of
the values EulerBeam3D's residual makes requestable (toolbox/BeamElement.jl:
151-189) -- ε, rₛₘ, and per Gauss point x, κ, fᵢ = EA ε, mᵢ = (GJ κ₁, EI₃ κ₂,
EI₂ κ₃) -- for every element and state, against the oracle's kinematics and
resultants: 1e-12 relative to each quantity's largest value, or to its natural
scale where that is larger (ε is the difference of a length ratio from 1, so
its rounding is absolute: scale 1 for ε and EA for fᵢ; the curvatures and
moments inherit the rounding of the local displacements, scale |κᵤ|·L and
EI·|κᵤ|·L).  The EI scale of an A-dof multiplies the bending moments.
"""
import numpy as np
import pytest

from muscade_gpu import _lib
from muscade_gpu import workloads as W
from muscade_gpu.device import DeviceModel
from oracle import lib as O

from test_gpu_parity import random_beams

pytestmark = pytest.mark.gpu
TOL = 1e-12


@pytest.fixture(scope="module", autouse=True)
def built():
    _lib.build()
    O.build()


def _compare(dev, ref, ele):
    n = ref.shape[0]
    names = {"eps": ref[:, 0], "rsm": ref[:, 1:10]}
    gp = ref[:, 10:].reshape(n, 4, 10)
    names.update(x=gp[..., 0:3], kappa=gp[..., 3:6], fi=gp[..., 6], mi=gp[..., 7:10])
    kuL = float(np.max(np.abs(ele[:, 40:44]) * ele[:, 48:49]))
    EI = float(np.max(ele[:, 54:57]))
    natural = {"eps": 1.0, "fi": float(np.max(ele[:, 53])), "kappa": kuL, "mi": EI * kuL}
    out = {}
    for k, r in names.items():
        d = dev[k]
        if k == "rsm":
            d = d.transpose(0, 2, 1).reshape(n, 9)
        scale = max(np.max(np.abs(r)), natural.get(k, 0.0), 1e-300)
        out[k] = float(np.max(np.abs(d.reshape(r.shape) - r)) / scale)
    return out


def test_beam_results_match_oracle():
    m, X, _ = random_beams(300, seed=41)
    st = m.initialize()
    dm = DeviceModel(m, st.dis)
    dg = st.dis.dis[0]
    nstate = 3
    rng = np.random.default_rng(5)
    states = np.zeros((nstate, m.ndof["X"]))
    for k in range(nstate):
        Xk = X[:, 0, :] * (1.0 + 0.3 * k) + rng.normal(size=X[:, 0, :].shape) * 1e-3
        states[k, dg.index_X - 1] = Xk  # each beam has its own nodes
    res = dm.beam_results(0, states)
    dm.close()
    ele = m.groups[0].cat("ele")
    for k in range(nstate):
        ref = O.beam_results(ele, states[k][dg.index_X - 1])
        errs = _compare({q: v[k] for q, v in res.items()}, ref, ele)
        print(f"state {k}: {errs}")
        assert all(e <= TOL for e in errs.values()), errs


def test_beam_results_with_ei_scale():
    d = W.adjoint_beam(nel=20, nstep=2)
    m = d["model"]
    st = m.initialize(time=0.0)
    dm = DeviceModel(m, st.dis)
    dm.set_A(d["A_true"])
    rc, states, _ = dm.sweepx(2, d["times"], st.time, list(st.X), maxdx=1e-5)
    assert rc == 0
    res = dm.beam_results(0, states[:, 0, :])
    dm.close()
    dg = st.dis.dis[0]
    ele = m.groups[0].cat("ele").copy()
    a = d["A_true"][dg.index_A[:, 0] - 1]
    ele[:, 54] *= a
    ele[:, 55] *= a
    for k in range(states.shape[0]):
        ref = O.beam_results(ele, states[k, 0][dg.index_X - 1])
        errs = _compare({q: v[k] for q, v in res.items()}, ref, ele)
        assert all(e <= TOL for e in errs.values()), errs
