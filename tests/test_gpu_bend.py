"""The 45° cantilever bend of examples/StaticBeamAnalysis.jl:10-36 on the GPU:
SweepX{0} over the three load steps (300, 450 and 600 N out of plane), its
states against the oracle's SweepX at 1e-9 of each dof class's largest value,
and the tip coordinates against the two published solutions the example quotes
(:131-134) within 0.1 m — a multi-element EulerBeam3D solve pinned by values
from outside this code.
"""
import numpy as np
import pytest

from muscade_gpu import _lib
from muscade_gpu import workloads as W
from muscade_gpu.device import DeviceModel
from oracle import reference as REF

pytestmark = pytest.mark.gpu
TOL_STATE = 1e-9


@pytest.fixture(scope="module", autouse=True)
def built():
    _lib.build()


def tip_coords(model, dis, X, tip):
    nod = np.asarray(model.dof_node["X"])
    fx = list(dis.fieldX)
    idx = [next(i for i in range(len(fx)) if fx[i] == f and nod[i] == tip) for f in ("t1", "t2", "t3")]
    return np.asarray(model.coord(tip)) + np.asarray(X)[idx]


@pytest.mark.parametrize("device_loop", [False, True])
def test_bend45_matches_oracle_and_literature(golden, device_loop):
    model, times, tip = W.bend45()
    st = model.initialize()
    ref = REF.sweepx(model, st.dis, st, times, OX=0, maxdx=1e-9)
    dm = DeviceModel(model, st.dis)
    rc, states, stats = dm.sweepx(0, times, st.time, list(st.X), maxdx=1e-9, device_loop=device_loop)
    dm.close()
    assert rc == 0 and stats.nstep_done == len(times)
    lam = np.array([str(f).startswith("λ") for f in st.dis.fieldX])
    for sel in (~lam, lam):
        dev = max(np.max(np.abs(states[k, 0][sel] - Xr[0][sel])) for k, (_, Xr) in enumerate(ref))
        scale = max(np.max(np.abs(Xr[0][sel])) for _, Xr in ref)
        assert dev <= TOL_STATE * scale, (dev, scale)
    tips = np.asarray([tip_coords(model, st.dis, states[k, 0], tip) for k in range(1, len(times))])
    print(f"bend tip coordinates at 300/450/600 N: {np.round(tips, 3).tolist()}")
    for key in ("bend_tip_longva", "bend_tip_crisfield"):
        assert np.max(np.abs(tips - np.asarray(golden[key]["value"]))) <= 0.1, key
