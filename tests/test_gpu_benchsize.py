"""Parity at the sizes the benchmark runs (GPU).

* The 60×60×20 lattice frame of the headline assembly (210,000 EulerBeam3D,
  21,600 Hold, 205,200 DofLoad; 453,600 dofs, 17,776,800 nonzeros): CSC
  pattern and asm maps bit-exact against the oracle's asmmat!, and one static
  assembly at the benchmark's state, Lλ and Lλx.nzval within 1e-12 of the
  largest entry of the oracle's (nested-dual elements, serial add_∂! scatter).
* Risers of the Newmark workload's shape (250 EulerBeam3D over 1000 m each,
  Δt = 0.05 s, exactly 3 Newton iterations per step, steps replayed from a
  captured CUDA graph) over 50 steps: states within 1e-9 of the oracle's
  SweepX{2} run with the same fixed iteration count, relative to each dof
  class's largest value over the trajectory.
"""
import numpy as np
import pytest

from muscade_gpu import _lib
from muscade_gpu import workloads as W
from muscade_gpu.device import DeviceModel
from oracle import lib as O
from oracle import reference as REF

pytestmark = pytest.mark.gpu
TOL_ASM = 1e-12
TOL_STATE = 1e-9


@pytest.fixture(scope="module", autouse=True)
def built():
    _lib.build()
    O.build()


def lattice_state(model, seed=2027):
    """The benchmark's state: X ~ N(0, 1e-3²) on every dof (bench.py state_for)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    return [rng.normal(size=model.ndof["X"]) * 1e-3]


def test_full_lattice_pattern_and_assembly_match_oracle():
    m, times = W.lattice(60, 60, 20)
    st = m.initialize()
    assert m.groups[0].nele == 210000 and m.ndof["X"] == 453600
    dm = DeviceModel(m, st.dis)
    prep = REF.Prepared(m, st.dis)
    assert dm.nnz == prep.nnz == 17776800
    colptr, rowval = dm.pattern()
    assert np.array_equal(colptr, prep.colptr) and np.array_equal(rowval, prep.rowval)
    for ig in range(len(m.groups)):
        a1, a2 = dm.asm(ig)
        assert np.array_equal(a1, prep.asm1[ig]) and np.array_equal(a2, prep.asm2[ig]), ig
    X = lattice_state(m)
    t = float(times[0])
    Ll, nz = dm.assemble(X, t=t)
    dm.close()
    Lr, nr = REF.assemble(prep, tuple(X), (np.zeros(0),), t, "static", REF.newmark_coefficients(0, 1.0, 0.25, 0.5))
    eL = np.max(np.abs(Ll - Lr)) / np.max(np.abs(Lr))
    eK = np.max(np.abs(nz - nr)) / np.max(np.abs(nr))
    print(f"lattice 60x60x20: Ll rel err {eL:.2e}, nzval rel err {eK:.2e}")
    assert eL <= TOL_ASM and eK <= TOL_ASM, (eL, eK)


def test_risers_at_benchmark_shape_match_oracle():
    m, times = W.risers(nriser=3, nel=250)
    st = m.initialize(time=0.0)
    T = np.asarray(times[:50])
    dm = DeviceModel(m, st.dis)
    rc, states, stats = dm.sweepx(2, T, st.time, list(st.X), fixed_iter=3, graph=True)
    dm.close()
    assert rc == 0 and stats.nstep_done == 50 and stats.niter_total == 150
    ref = REF.sweepx(m, st.dis, st, T, OX=2, fixed_iter=3)
    lam = np.array([str(f).startswith("λ") for f in st.dis.fieldX])
    errs = {}
    for d in range(3):
        for name, sel in (("dofs", ~lam), ("multipliers", lam)):
            if d > 0 and name == "multipliers":
                continue  # no element reads the multipliers' time derivatives
            dev = max(np.max(np.abs(states[k, d][sel] - Xr[d][sel])) for k, (_, Xr) in enumerate(ref))
            scale = max(np.max(np.abs(Xr[d][sel])) for _, Xr in ref)
            errs[(name, d)] = dev / scale
    print("risers 3x250, 50 steps:", {f"{k[0]}/{k[1]}": f"{v:.1e}" for k, v in errs.items()})
    assert all(e <= TOL_STATE for e in errs.values()), errs
