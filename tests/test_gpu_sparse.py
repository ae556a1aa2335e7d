"""The multifrontal device solver (GPU): SweepX{0} of lattice frames whose
bands are too wide for the banded kernels, against the oracle's SweepX (SuperLU
in place of the reference's UMFPACK, src/SweepX.jl:207-210).

Tolerance: converged states within 1e-9 of the oracle's, relative to the
largest value of each dof class (node dofs, multipliers) over the trajectory.
"""
import numpy as np
import pytest

from muscade_gpu import _lib
from muscade_gpu import workloads as W
from muscade_gpu.device import DeviceError, DeviceModel
from oracle import lib as O
from oracle import reference as REF

pytestmark = pytest.mark.gpu
TOL_STATE = 1e-9


@pytest.fixture(scope="module", autouse=True)
def built():
    _lib.build()
    O.build()


def state_errors(states, ref, fieldX):
    lam = np.array([str(f).startswith("λ") for f in fieldX])
    assert len(states) == len(ref)
    out = {}
    for name, sel in (("dofs", ~lam), ("multipliers", lam)):
        if not sel.any():
            continue
        dev = max(np.max(np.abs(states[k, 0][sel] - Xr[0][sel])) for k, (_, Xr) in enumerate(ref))
        scale = max(np.max(np.abs(Xr[0][sel])) for _, Xr in ref)
        out[name] = dev / scale
    return out


@pytest.fixture(scope="module")
def lattice():
    m, times = W.lattice(12, 12, 6)
    st = m.initialize()
    ref = REF.sweepx(m, st.dis, st, times, OX=0, maxdx=1e-8, maxLl=1e-3)
    return m, st, times, ref


@pytest.mark.parametrize("linsolve", ["auto", "sparse64"])
def test_lattice_sweepx0_matches_oracle(lattice, linsolve):
    m, st, times, ref = lattice
    dm = DeviceModel(m, st.dis, linsolve=linsolve)
    rc, states, stats = dm.sweepx(0, times, st.time, list(st.X), maxdx=1e-8, maxLl=1e-3)
    info, sp = dm.linear_solver_info(), dm.sparse_info()
    dm.close()
    assert rc == 0 and stats.nstep_done == len(times)
    assert info["kind"] == ("sparse" if linsolve == "auto" else "sparse64")
    assert sp["nfront"] > 1 and sp["max_pivots"] <= sp["max_front"] and sp["last_sweeps"] >= 1
    errs = state_errors(states, ref, st.dis.fieldX)
    print(f"lattice 12x12x6 ({linsolve}): {errs}, fronts {sp['nfront']}, largest {sp['max_front']}, "
          f"FP64 {sp['fp64']}, sweeps {sp['last_sweeps']}, perturbed pivots {sp['last_perturbed']}")
    assert all(e <= TOL_STATE for e in errs.values()), errs


def test_multifrontal_and_banded_solvers_agree():
    """A lattice narrow enough for the banded block kernels: the multifrontal
    trajectory equals theirs to the state tolerance, and repeats bitwise."""
    m, times = W.lattice(6, 5, 4)
    st = m.initialize()
    out = {}
    for kind in ("block", "sparse", "sparse"):
        dm = DeviceModel(m, st.dis, linsolve=kind)
        rc, states, _ = dm.sweepx(0, times[:3], st.time, list(st.X), maxdx=1e-8, maxLl=1e-3)
        dm.close()
        assert rc == 0
        if kind in out:
            assert np.array_equal(out[kind], states)  # deterministic
        out[kind] = states
    ref = [(0.0, (out["block"][k, 0],)) for k in range(len(out["block"]))]
    errs = state_errors(out["sparse"], ref, st.dis.fieldX)
    assert all(e <= TOL_STATE for e in errs.values()), errs


@pytest.mark.parametrize("threshold", ["64", "1"])
def test_blocked_substitutions_match_oracle(lattice, monkeypatch, threshold):
    """Fronts with many pivots take the blocked substitutions (one launch per
    column block over a grid of row tiles); lowering the threshold sends most
    (64) or all (1) fronts of the 12×12×6 lattice through them."""
    m, st, times, ref = lattice
    monkeypatch.setenv("MGPU_SPARSE_BLOCKED_PIVOTS", threshold)
    out = {}
    for kind in ("sparse", "sparse64"):
        dm = DeviceModel(m, st.dis, linsolve=kind)
        rc, states, stats = dm.sweepx(0, times, st.time, list(st.X), maxdx=1e-8, maxLl=1e-3)
        sp = dm.sparse_info()
        dm.close()
        assert rc == 0 and stats.nstep_done == len(times)
        errs = state_errors(states, ref, st.dis.fieldX)
        print(f"blocked from {threshold} pivots ({kind}): {errs}, sweeps {sp['last_sweeps']}")
        assert all(e <= TOL_STATE for e in errs.values()), errs
        out[kind] = states
    monkeypatch.delenv("MGPU_SPARSE_BLOCKED_PIVOTS")
    dm = DeviceModel(m, st.dis, linsolve="sparse64")
    rc, states, _ = dm.sweepx(0, times, st.time, list(st.X), maxdx=1e-8, maxLl=1e-3)
    dm.close()
    ref64 = [(0.0, (states[k, 0],)) for k in range(len(states))]
    errs = state_errors(out["sparse64"], ref64, st.dis.fieldX)
    assert all(e <= 1e-12 for e in errs.values()), errs  # FP64 blocked vs one-block: rounding only


def test_fixed_iterations_without_graph_replay(lattice):
    m, st, times, _ = lattice
    dm = DeviceModel(m, st.dis)
    rc, states, stats = dm.sweepx(0, times[:2], st.time, list(st.X), fixed_iter=4)
    dm.close()
    assert rc == 0 and stats.niter_total == 8
    ref = REF.sweepx(m, st.dis, st, times[:2], OX=0, fixed_iter=4)
    errs = state_errors(states, ref, st.dis.fieldX)
    assert all(e <= TOL_STATE for e in errs.values()), errs


def test_per_component_convergence_is_rejected(lattice):
    m, st, times, _ = lattice
    dm = DeviceModel(m, st.dis)
    with pytest.raises(DeviceError) as e:
        dm._check(dm.sweepx(0, times[:1], st.time, list(st.X), per_component=True)[0])
    dm.close()
    assert e.value.kind == "unsupported"


@pytest.mark.parametrize("grid", [(12, 12, 6), (20, 20, 8)])
def test_super_panel_factorisation(monkeypatch, grid):
    """The FP32 factors by super-panels of 256 pivots (left-looking inside,
    one trailing update per super-panel) against those by 64-column blocks:
    both refine to the FP64 solution without falling back to FP64 factors,
    and their iterates agree to the state tolerance."""
    m, times = W.lattice(*grid)
    st = m.initialize()
    out, info = {}, {}
    for sup in ("1", "0"):
        monkeypatch.setenv("MGPU_SPARSE_SUPER", sup)
        dm = DeviceModel(m, st.dis, linsolve="sparse")
        rc, states, _ = dm.sweepx(0, times[:2], st.time, list(st.X), fixed_iter=3)
        info[sup] = dm.sparse_info()
        dm.close()
        assert rc == 0
        out[sup] = states
    monkeypatch.delenv("MGPU_SPARSE_SUPER")
    print(f"super-panels {grid}: pivots {info['1']['max_pivots']}, sweeps {info['1']['last_sweeps']} "
          f"(per block {info['0']['last_sweeps']})")
    assert info["1"]["max_pivots"] > 256  # more than one super-panel in the largest front
    assert info["1"]["last_fallback"] == 0 and info["0"]["last_fallback"] == 0
    assert info["1"]["last_sweeps"] <= info["0"]["last_sweeps"] + 2
    ref = [(0.0, (out["0"][k, 0],)) for k in range(len(out["0"]))]
    errs = state_errors(out["1"], ref, st.dis.fieldX)
    assert all(e <= TOL_STATE for e in errs.values()), errs


@pytest.mark.parametrize("kind", ["sparse", "sparse64"])
def test_chained_substitutions_match_launch_per_block(lattice, monkeypatch, kind):
    """The chained substitutions (one launch per height and direction, tiles
    published through flags) repeat the arithmetic of the launch-per-column-
    block kernels in the same order: the trajectories are bitwise equal, with
    every front of 1 pivot or more on the blocked path."""
    m, st, times, ref = lattice
    monkeypatch.setenv("MGPU_SPARSE_BLOCKED_PIVOTS", "1")
    out = {}
    for chained in ("1", "0"):
        monkeypatch.setenv("MGPU_SPARSE_CHAINED", chained)
        dm = DeviceModel(m, st.dis, linsolve=kind)
        rc, states, _ = dm.sweepx(0, times[:2], st.time, list(st.X), maxdx=1e-8, maxLl=1e-3)
        dm.close()
        assert rc == 0
        out[chained] = states
    assert np.array_equal(out["1"], out["0"])
    errs = state_errors(out["1"], ref[:2], st.dis.fieldX)
    assert all(e <= TOL_STATE for e in errs.values()), errs


def test_tensor_core_trailing_update(monkeypatch):
    """The super-panels' trailing blocks on the tensor cores (tcgen05 TF32 ×3,
    MGPU_SPARSE_TC=1) against the FP32 SIMT kernel: no fallback to FP64
    factors, iterates within the state tolerance of each other."""
    m, times = W.lattice(20, 20, 8)
    st = m.initialize()
    out, info = {}, {}
    for tc in ("1", "0"):
        monkeypatch.setenv("MGPU_SPARSE_TC", tc)
        dm = DeviceModel(m, st.dis, linsolve="sparse")
        rc, states, _ = dm.sweepx(0, times[:2], st.time, list(st.X), fixed_iter=3)
        info[tc] = dm.sparse_info()
        dm.close()
        assert rc == 0
        out[tc] = states
    monkeypatch.delenv("MGPU_SPARSE_TC")
    print(f"tensor-core trailing update: sweeps {info['1']['last_sweeps']} (SIMT {info['0']['last_sweeps']}), "
          f"factor {info['1']['last_factor_ms']:.2f} ms (SIMT {info['0']['last_factor_ms']:.2f} ms)")
    assert info["1"]["last_fallback"] == 0
    ref = [(0.0, (out["0"][k, 0],)) for k in range(len(out["0"]))]
    errs = state_errors(out["1"], ref, st.dis.fieldX)
    assert all(e <= TOL_STATE for e in errs.values()), errs
