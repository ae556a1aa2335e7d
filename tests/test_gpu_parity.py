"""Parity of the CUDA path with the oracle (GPU).

Tolerances (written where used):
  * element residuals and tangents: max |gpu − oracle| ≤ 1e-12 · max |oracle|
    per element array (norm-relative, FP64), static and Newmark, for every
    element whose two Rodrigues⁻¹ arguments x = (tr m − 1)/2 (the relative
    rotation r₂r₁ᵀ and the mid-frame rₛₘ) keep 1 − x² ≥ 1e-2.  Closer to
    x = ±1 the reference's own formulas are ill-conditioned: near x = −1 (a
    frame near a half turn) scac(x) = sinc1(acos x) → 0 divides spin⁻¹(m),
    and near x = 1 the Newmark tangent's third-order terms scac‴ =
    sinc1‴t₁³ + 3sinc1″t₁t₂ + sinc1′t₃ with t₁ = −1/√(1−x²) cancel terms of
    order 1e4 to order 1e-2 just above the Taylor branch; there any other
    sin/cos/acos or FMA rounding changes the last digits.  Those elements
    are evaluated and their largest deviation printed, not asserted;
  * CSC pattern and asm maps: bit-exact;
  * assembled Lλ and Lλx.nzval: ≤ 1e-12 relative to the largest entry;
  * converged states: ≤ 1e-9 relative (‖Δ‖∞ / ‖x‖∞).
"""
import math

import numpy as np
import pytest

from muscade_gpu import _lib
from muscade_gpu import workloads as W
from muscade_gpu.device import DeviceError, DeviceModel
from muscade_gpu.elements import AxisymmetricBarCrossSection, Bar3D, BeamCrossSection, DofLoad, EulerBeam3D, Hold
from muscade_gpu.model import Model
from oracle import lib as O
from oracle import reference as REF

pytestmark = pytest.mark.gpu
TOL_ELE = 1e-12
TOL_ASM = 1e-12
SCAC_MARGIN = 1e-2  # elements with 1 − x² below this at either Rodrigues⁻¹ are reported, not asserted
TOL_STATE = 1e-9


@pytest.fixture(scope="module", autouse=True)
def built():
    _lib.build()
    O.build()


def relerr(a, b):
    return np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300)


def random_beams(n, seed, udof=False, rot=0.5):
    rng = np.random.default_rng(seed)
    m = Model()
    c1 = rng.normal(size=(n, 3))
    c2 = c1 + rng.normal(size=(n, 3)) * 2
    ids1 = m.addnode(c1)
    ids2 = m.addnode(c2)
    mat = BeamCrossSection(EA=1e3 * rng.uniform(1, 2, n), EI2=3 * rng.uniform(1, 2, n), EI3=2 * rng.uniform(1, 2, n),
                           GJ=4 * rng.uniform(1, 2, n), mu=1.3, iota1=2.1, w=0.7, Ca1=0.3, Cl1=0.2, Cq1=0.1, Ca2=0.5,
                           Cl2=0.4, Cq2=0.3, Ca3=0.6, Cl3=0.7, Cq3=0.8)
    o2 = rng.normal(size=(n, 3))
    if udof:
        ids3 = m.addnode(np.zeros((n, 3)))
        m.addelement(EulerBeam3D, np.stack([ids1, ids2, ids3], axis=1), mat=mat, orient2=o2, udof=True)
    else:
        m.addelement(EulerBeam3D, np.stack([ids1, ids2], axis=1), mat=mat, orient2=o2)
    # nodal rotations up to ~1.5 rad, relative rotation across an element ≲ 0.3 rad
    # (away from the half-turn where Rodrigues⁻¹ is singular in the reference too)
    X = rng.normal(size=(n, 3, 12)) * 0.1
    X[:, 0, 3:6] = rng.normal(size=(n, 3)) * rot
    X[:, 0, 9:12] = X[:, 0, 3:6] + rng.normal(size=(n, 3)) * 0.1
    X[: n // 5, 0, 3:6] = 0.0  # exactly unrotated node 1 (norm3 zero branch)
    X[:, 1:, :] = rng.normal(size=(n, 2, 12)) * 0.5
    U = rng.normal(size=(n, 3)) if udof else None
    return m, X, U


def _spin(v):
    return np.array([[0.0, -v[2], v[1]], [v[2], 0.0, -v[0]], [-v[1], v[0], 0.0]])


def _rodrigues(v):
    """Rodrigues (toolbox/Rotations.jl): I + sinc1(θ)S + ½sinc1(θ/2)²S²."""
    th = np.linalg.norm(v)
    S = _spin(v)
    return np.eye(3) + np.sinc(th / np.pi) * S + 0.5 * np.sinc(th / 2 / np.pi) ** 2 * (S @ S)


def _rodrigues_inv(m):
    x = (np.trace(m) - 1.0) / 2.0
    w = 0.5 * np.array([m[2, 1] - m[1, 2], m[0, 2] - m[2, 0], m[1, 0] - m[0, 1]])
    return w / np.sinc(np.arccos(np.clip(x, -1.0, 1.0)) / np.pi), x


def scac_margin(ele, X):
    """min over the beam's two Rodrigues⁻¹ (corotated, toolbox/BeamElement.jl:193-208)
    of 1 − x², x = (tr m − 1)/2: m = r₂r₁ᵀ and m = rₛₘ = Rod(½Δv) r₁ rₘ."""
    out = np.zeros(len(X))
    for e in range(len(X)):
        r1, r2 = _rodrigues(X[e, 0, 3:6]), _rodrigues(X[e, 0, 9:12])
        w, xr = _rodrigues_inv(r2 @ r1.T)
        rm = ele[e, 3:12].reshape(3, 3, order="F")
        _, xs = _rodrigues_inv(_rodrigues(0.5 * w) @ r1 @ rm)
        out[e] = min(1.0 - xr * xr, 1.0 - xs * xs)
    return out


@pytest.mark.parametrize("udof", [False, True])
def test_beam_element_parity(udof):
    m, X, U = random_beams(256, 11 + udof, udof=udof)
    dm = DeviceModel(m, m.initialize().dis)
    ele = m.groups[0].cat("ele")
    ordinary = scac_margin(ele, X) >= SCAC_MARGIN
    assert ordinary.sum() >= 0.7 * len(X)  # the assertion covers most of the random elements
    worst = {"ordinary": 0.0, "near x=±1": 0.0}

    def check(got, ref, e, what):
        err = relerr(got, ref)
        key = "ordinary" if ordinary[e] else "near x=±1"
        worst[key] = max(worst[key], err)
        if ordinary[e]:
            assert err <= TOL_ELE, (what, e, err)

    # static (SweepX{0} form): K = ∂R/∂X₀
    d = O.diffed("beam", ele, X[:, :1, :], U)
    R, K, H = dm.element_eval(0, X[:, :1, :], U)
    for e in range(len(X)):
        check(R[e], d["R"][e], e, "R static")
        check(K[e], d["K"][e], e, "K static")
        if udof:
            check(H[e], d["H"][e], e, "dR/dU")
    # Newmark: K, C, M from unit perturbations of (X, X', X'')
    d = O.diffed("beam", ele, X, U)
    for p, name in (((1, 0, 0), "K"), ((0, 1, 0), "C"), ((0, 0, 1), "M")):
        R, J, _ = dm.element_eval(0, X, U, p=p)
        for e in range(len(X)):
            check(R[e], d["R"][e], e, "R Newmark")
            check(J[e], d[name][e], e, name)
    dm.close()
    print(f"beam element parity (udof={udof}): {int(ordinary.sum())} ordinary elements, largest deviation "
          f"{worst['ordinary']:.1e}; {int((~ordinary).sum())} near a Rodrigues⁻¹ singularity or branch, largest "
          f"deviation {worst['near x=±1']:.1e}")


def test_bar_element_parity():
    rng = np.random.default_rng(5)
    n = 32
    m = Model()
    c1 = rng.normal(size=(n, 3))
    ids1 = m.addnode(c1)
    ids2 = m.addnode(c1 + rng.normal(size=(n, 3)))
    mat = AxisymmetricBarCrossSection(EA=10.0, mu=1.0, w=2.0, Cat=0.2, Clt=0.3, Cqt=0.4, Can=0.5, Cln=0.6, Cqn=0.7)
    m.addelement(Bar3D, np.stack([ids1, ids2], axis=1), mat=mat)
    dm = DeviceModel(m, m.initialize().dis)
    X = rng.normal(size=(n, 3, 6)) * 0.3
    d = O.diffed("bar", m.groups[0].cat("ele"), X, t=-7.0)
    for p, name in (((1, 0, 0), "K"), ((0, 1, 0), "C"), ((0, 0, 1), "M")):
        R, J, _ = dm.element_eval(0, X, t=-7.0, p=p)
        for e in range(n):
            assert relerr(R[e], d["R"][e]) <= TOL_ELE
            assert relerr(J[e], d[name][e]) <= TOL_ELE, (name, e)
    dm.close()


def _models():
    yield "cantilever", W.cantilever()[0]
    yield "lattice", W.lattice(7, 6, 4)[0]
    yield "risers", W.risers(nriser=3, nel=12)[0]


@pytest.mark.parametrize("name,model", list(_models()))
def test_pattern_and_asm_bit_exact(name, model):
    dis = model.initialize().dis
    dm = DeviceModel(model, dis)
    prep = REF.Prepared(model, dis)
    colptr, rowval = dm.pattern()
    assert dm.nnz == prep.nnz
    assert np.array_equal(colptr, prep.colptr) and np.array_equal(rowval, prep.rowval)
    for ig in range(len(model.groups)):
        a1, a2 = dm.asm(ig)
        assert np.array_equal(a1, prep.asm1[ig]) and np.array_equal(a2, prep.asm2[ig])
    dm.close()


def _state(model, seed, nder, amp=0.05):
    rng = np.random.default_rng(seed)
    n = model.ndof["X"]
    return [rng.normal(size=n) * amp for _ in range(nder)]


@pytest.mark.parametrize("name,model", list(_models()))
def test_assembly_parity(name, model):
    st = model.initialize()
    dm = DeviceModel(model, st.dis)
    prep = REF.Prepared(model, st.dis)
    U = (np.zeros(model.ndof["U"]),)
    X = _state(model, 7, 1)
    Ll, nz = dm.assemble(X, t=0.4)
    Lr, nr = REF.assemble(prep, tuple(X), U, 0.4, "static", REF.newmark_coefficients(0, 1, 0.25, 0.5))
    assert relerr(Ll, Lr) <= TOL_ASM and relerr(nz, nr) <= TOL_ASM
    # determinism: bitwise identical on repeat, and through the page-locked reused buffers
    Ll2, nz2 = dm.assemble(X, t=0.4)
    assert np.array_equal(Ll, Ll2) and np.array_equal(nz, nz2)
    Ll3, nz3 = dm.assemble(X, t=0.4, reuse=True)
    assert np.array_equal(Ll, Ll3) and np.array_equal(nz, nz3)
    # Newmark forms
    X3 = _state(model, 8, 3)
    c = REF.newmark_coefficients(2, 0.05, 0.25, 0.5)
    for mission, mref in ((_lib.ASM_STEP, "step"), (_lib.ASM_ITER, "iter")):
        Ll, nz = dm.assemble(X3, t=0.35, mission=mission, c=c)
        Lr, nr = REF.assemble(prep, tuple(X3), U, 0.35, mref, c)
        assert relerr(Ll, Lr) <= TOL_ASM, mref
        assert relerr(nz, nr) <= TOL_ASM, mref
    dm.close()


def _state_errors(gpu_states, ref, nder, fieldX):
    """Largest deviation from the oracle over the trajectory, per dof class and
    derivative order, relative to that class's largest value over the trajectory.

    A per-step scale would be meaningless at the start of a ramped motion: the
    displacements are then ~1e-5 m on node coordinates of ~1e3 m, so both codes
    only resolve them to ~1e-13 m, and the Newmark update multiplies that
    rounding by 1/(βΔt²) in the accelerations.  The time derivatives of the
    Lagrange multipliers are left out: the Newmark decrement updates them like
    any X-dof (src/SweepX.jl:98-116) but no element reads them, so they only
    carry the multipliers' rounding amplified by γ/(βΔt) and 1/(βΔt²).
    """
    lam = np.array([str(f).startswith("λ") for f in fieldX])
    assert len(gpu_states) == len(ref)
    out = {}
    for d in range(nder):
        for name, sel in (("dofs", ~lam), ("multipliers", lam)):
            if not sel.any() or (d > 0 and name == "multipliers"):
                continue
            dev = max(np.max(np.abs(s.X[d][sel] - Xr[d][sel])) for s, (t, Xr) in zip(gpu_states, ref))
            scale = max(max(np.max(np.abs(Xr[d][sel])) for t, Xr in ref), 1e-300)
            out[(name, d)] = dev / scale
    return out


def _compare_states(gpu_states, ref, nder, fieldX):
    errs = _state_errors(gpu_states, ref, nder, fieldX)
    assert all(e <= TOL_STATE for e in errs.values()), errs


@pytest.mark.parametrize("linsolve", ["f32ir", "f64", "block"])
def test_sweepx0_cantilever_matches_oracle(linsolve):
    from muscade_gpu import SweepXGPU, solve

    m, times = W.cantilever()
    st = m.initialize()
    out = solve(SweepXGPU[0], st, times, maxdx=1e-9, maxLl=1e-5, linsolve=linsolve)
    ref = REF.sweepx(m, st.dis, st, times, OX=0, maxdx=1e-9, maxLl=1e-5)
    _compare_states(out, ref, 1, st.dis.fieldX)
    tip = out[-1].X[0][120:123]
    assert tip[2] > 5.0  # large-rotation equilibrium: the tip has risen well above a linear answer's scale


def test_sweepx0_lattice_matches_oracle():
    from muscade_gpu import SweepXGPU, solve

    m, times = W.lattice(8, 7, 5)
    st = m.initialize()
    out = solve(SweepXGPU[0], st, times[:2], maxdx=1e-8, maxLl=1e-3)
    ref = REF.sweepx(m, st.dis, st, times[:2], OX=0, maxdx=1e-8, maxLl=1e-3)
    _compare_states(out, ref, 1, st.dis.fieldX)


@pytest.mark.parametrize("linsolve", ["f32ir", "f64", "block"])
def test_sweepx2_risers_match_oracle(linsolve):
    from muscade_gpu import SweepXGPU, solve

    m, times = W.risers(nriser=2, nel=20)
    st = m.initialize(time=0.0)
    T = times[:20]
    out = solve(SweepXGPU[2], st, T, maxiter=20, maxdx=1e-5, maxLl=math.inf, linsolve=linsolve)
    ref = REF.sweepx(m, st.dis, st, T, OX=2, maxiter=20, maxdx=1e-5, maxLl=math.inf)
    _compare_states(out, ref, 3, st.dis.fieldX)


def _sweep(model, st, OX, times, linsolve, **kw):
    dm = DeviceModel(model, st.dis, linsolve=linsolve)
    rc, states, stats = dm.sweepx(OX, times, st.time, list(st.X), **kw)
    info = dm.linear_solver_info()
    dm.close()
    assert rc == 0
    return states, info


def test_row_band_fp64_is_bitwise_the_block_solver():
    """Same gbtf2/gbtrs arithmetic in two layouts: identical Newton trajectories."""
    m, times = W.risers(nriser=3, nel=16)
    st = m.initialize(time=0.0)
    a, ia = _sweep(m, st, 2, times[:8], "f64", maxiter=20, maxdx=1e-5)
    b, ib = _sweep(m, st, 2, times[:8], "block", maxiter=20, maxdx=1e-5)
    assert ia["kind"] == "f64" and ib["kind"] == "block" and ia["ncomp"] == 3
    assert np.array_equal(a, b)


def test_fp32_refinement_reaches_fp64_accuracy():
    """Risers: FP32 factors refined in FP64 give the FP64 trajectory to rounding, no fallback."""
    m, times = W.risers(nriser=3, nel=16)
    st = m.initialize(time=0.0)
    a, ia = _sweep(m, st, 2, times[:8], "f32ir", maxiter=20, maxdx=1e-5)
    b, _ = _sweep(m, st, 2, times[:8], "f64", maxiter=20, maxdx=1e-5)
    assert ia["kind"] == "f32ir" and ia["last_fallback"] == 0 and 1 <= ia["last_sweeps"] <= 8
    as_states = [[None, (a[k, 0], a[k, 1], a[k, 2])] for k in range(len(a))]
    gpu = [type("S", (), {"X": X})() for _, X in as_states]
    ref = [(0.0, (b[k, 0], b[k, 1], b[k, 2])) for k in range(len(b))]
    errs = _state_errors(gpu, ref, 3, st.dis.fieldX)
    assert all(e <= TOL_STATE for e in errs.values()), errs


def test_fp32_refinement_falls_back_to_fp64_when_ill_conditioned():
    """A 400-element cantilever (condition number ~1e12) defeats FP32 refinement:
    the component is refactorised in FP64 and the result is the FP64 one
    (three Newton iterations per step on both paths, small load)."""
    m, _ = W.cantilever(nel=400, length=200.0, load=1e-3)
    st = m.initialize()
    times = np.array([0.1, 0.2])
    a, ia = _sweep(m, st, 0, times, "f32ir", fixed_iter=3)
    b, _ = _sweep(m, st, 0, times, "f64", fixed_iter=3)
    assert ia["last_fallback"] == 1
    assert np.array_equal(a, b)


def test_graph_replay_matches_kernel_by_kernel_launches():
    """Fixed-iteration Newmark steps replayed from one captured CUDA graph give
    the states of the same kernels launched one by one."""
    m, times = W.risers(nriser=3, nel=16)
    st = m.initialize(time=0.0)
    dm = DeviceModel(m, st.dis)
    rc1, a, s1 = dm.sweepx(2, times[:12], st.time, list(st.X), fixed_iter=3, graph=True)
    rc2, b, s2 = dm.sweepx(2, times[:12], st.time, list(st.X), fixed_iter=3, graph=False)
    dm.close()
    assert rc1 == 0 and rc2 == 0 and s1.nstep_done == s2.nstep_done == 12 and s1.niter_total == 36
    assert np.array_equal(a, b)


def test_batched_models_follow_their_own_iterations():
    """Independent models in one context with per-component convergence give,
    bitwise, the states each model reaches when solved alone."""
    params = W.batched_params(6, nel_range=(10, 30), seed=11)
    mb, offs, times = W.build_batched(params)
    sb = mb.initialize()
    dm = DeviceModel(mb, sb.dis)
    rc, xb, stats = dm.sweepx(0, times, sb.time, list(sb.X), maxdx=1e-9, maxLl=1e-5, per_component=True)
    info = dm.linear_solver_info()
    dm.close()
    assert rc == 0 and info["ncomp"] == 6
    for p, off in zip(params, offs):
        mi, _, _ = W.build_batched([p])
        si = mi.initialize()
        dmi = DeviceModel(mi, si.dis)
        rci, xi, _ = dmi.sweepx(0, times, si.time, list(si.X), maxdx=1e-9, maxLl=1e-5)
        dmi.close()
        assert rci == 0
        nodes = np.arange(1, mi.nnod + 1)
        di, db = W.node_dofs(mi, nodes), W.node_dofs(mb, nodes + off)
        assert np.array_equal(di >= 0, db >= 0)
        sel = di >= 0
        assert np.array_equal(xi[:, 0, di[sel]], xb[:, 0, db[sel]]), p


def test_sweepx0_portal_frame_matches_oracle():
    from muscade_gpu import SweepXGPU, solve

    p = next(q for q in W.batched_params(20, nel_range=(12, 24), seed=5) if q["kind"] == "portal")
    m, _, times = W.build_batched([p])
    st = m.initialize()
    out = solve(SweepXGPU[0], st, times, maxdx=1e-9, maxLl=1e-5)
    ref = REF.sweepx(m, st.dis, st, times, OX=0, maxdx=1e-9, maxLl=1e-5)
    _compare_states(out, ref, 1, st.dis.fieldX)


def _rel_dev(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def test_partitioned_solver_matches_row_band_solver():
    """Long risers (n = 606 per component) cut into interiors and separators:
    the trajectory of the row-band solver within rounding (the pivoting is
    restricted to the blocks, so not bitwise)."""
    m, times = W.risers(nriser=3, nel=100)
    st = m.initialize(time=0.0)
    a, ia = _sweep(m, st, 2, times[:10], "torn", fixed_iter=3)
    b, ib = _sweep(m, st, 2, times[:10], "f64", fixed_iter=3)
    assert ia["kind"] == "torn" and ib["kind"] == "f64"
    lam = np.array([str(f).startswith("λ") for f in st.dis.fieldX])
    # the state tolerance: accelerations carry 1/(βΔt²) times the rounding of the positions
    for d in range(3):
        assert _rel_dev(a[:, d][:, ~lam], b[:, d][:, ~lam]) <= TOL_STATE, d
    assert _rel_dev(a[:, 0][:, lam], b[:, 0][:, lam]) <= TOL_STATE


def test_partitioned_fp32_refined_matches_fp64():
    """FP32 partitioned factors inside FP64 refinement: the FP64 trajectory to
    the state tolerance, no fallback on the (well-conditioned) risers."""
    m, times = W.risers(nriser=3, nel=100)
    st = m.initialize(time=0.0)
    a, ia = _sweep(m, st, 2, times[:10], "torn32", fixed_iter=3)
    b, _ = _sweep(m, st, 2, times[:10], "torn", fixed_iter=3)
    assert ia["kind"] == "torn32" and ia["last_fallback"] == 0
    lam = np.array([str(f).startswith("λ") for f in st.dis.fieldX])
    for d in range(3):
        assert _rel_dev(a[:, d][:, ~lam], b[:, d][:, ~lam]) <= TOL_STATE, d


def test_partitioned_fp32_falls_back_on_an_ill_conditioned_chain():
    """A static 600-element cantilever is beyond FP32 refinement: its component
    is solved again in FP64 and the result is the FP64 one."""
    m, _ = W.cantilever(nel=600, length=300.0, load=1e-4)
    st = m.initialize()
    times = np.array([0.5, 1.0])
    a, ia = _sweep(m, st, 0, times, "torn32", fixed_iter=2)
    b, _ = _sweep(m, st, 0, times, "torn", fixed_iter=2)
    assert ia["last_fallback"] == 1
    assert np.array_equal(a, b)


def test_fused_partitioned_solve_is_bitwise_the_level_by_level_one(monkeypatch):
    """Components of few interiors are solved by one block each (interiors,
    cyclic reduction and back-substitution behind block barriers); the
    arithmetic is that of the one-launch-per-level kernels, bit for bit, for
    Lλx and for its transpose."""
    m, times = W.risers(nriser=3, nel=100)
    st = m.initialize(time=0.0)
    a, _ = _sweep(m, st, 2, times[:6], "torn", fixed_iter=3)
    d = W.adjoint_beam(nel=120, nstep=6)
    ma = d["model"]
    sa = ma.initialize(time=0.0)
    y = np.zeros((6, len(d["sensors"])))

    def adj():
        dm = DeviceModel(ma, sa.dis, linsolve="torn")
        r = dm.adjoint(2, d["times"], sa.time, list(sa.X), d["sensors"], 1.0, y, maxdx=1e-7)
        dm.close()
        return r

    ga = adj()
    monkeypatch.setenv("MGPU_TORN_FUSED", "0")
    b, _ = _sweep(m, st, 2, times[:6], "torn", fixed_iter=3)
    gb = adj()
    assert np.array_equal(a, b)
    assert ga[0] == gb[0] and np.array_equal(ga[1], gb[1])


def test_fused_partitioned_fp32_falls_back_on_an_ill_conditioned_chain():
    """The fused FP32 refinement flags a component it cannot refine (a slender
    cantilever, about 20 interiors); its FP64 solve is the FP64 one."""
    m, _ = W.cantilever(nel=200, length=300.0, load=1e-4)
    st = m.initialize()
    times = np.array([0.5, 1.0])
    a, ia = _sweep(m, st, 0, times, "torn32", fixed_iter=2)
    b, _ = _sweep(m, st, 0, times, "torn", fixed_iter=2)
    assert ia["last_fallback"] == 1
    assert np.array_equal(a, b)


def test_partitioned_solver_static_cantilever_matches_oracle():
    from muscade_gpu import SweepXGPU, solve

    m, _ = W.cantilever(nel=120, length=10.0, load=1e2)
    st = m.initialize()
    times = np.array([0.5, 1.0])
    out = solve(SweepXGPU[0], st, times, maxdx=1e-8, maxiter=30, linsolve="torn")
    ref = REF.sweepx(m, st.dis, st, times, OX=0, maxdx=1e-8, maxiter=30)
    _compare_states(out, ref, 1, st.dis.fieldX)


def test_partitioned_transposed_solve_gives_the_adjoint():
    d = W.adjoint_beam(nel=120, nstep=8)
    m = d["model"]
    st = m.initialize(time=0.0)
    y = np.zeros((8, len(d["sensors"])))
    res = {}
    for kind in ("torn", "torn32", "f64"):
        dm = DeviceModel(m, st.dis, linsolve=kind)
        res[kind] = dm.adjoint(2, d["times"], st.time, list(st.X), d["sensors"], 1.0, y, maxdx=1e-7)
        assert dm.linear_solver_info()["kind"] == kind
        dm.close()
    for kind in ("torn", "torn32"):
        assert res[kind][0] == pytest.approx(res["f64"][0], rel=1e-10)
        assert _rel_dev(res[kind][1], res["f64"][1]) <= 1e-9


def test_autotune_keeps_a_faster_configuration_with_the_same_results():
    m, times = W.risers(nriser=3, nel=100)
    st = m.initialize(time=0.0)
    ref, _ = _sweep(m, st, 2, times[:6], "auto", fixed_iter=3)
    dm = DeviceModel(m, st.dis)
    dm.upload_state([st.X[0], np.zeros(m.ndof["X"]), np.zeros(m.ndof["X"])], t=times[0])
    c = REF.newmark_coefficients(2, 0.05, 0.25, 0.5)
    rep = dm.autotune(_lib.ASM_ITER, {k: c[k] for k in ("a1", "a2", "a3", "b1", "b2", "b3")})
    assert rep["elem_block"] in (64, 128, 256) and set(rep["ms_elem"]) == {64, 128, 256}
    assert rep["linsolve"] in rep["ms_linsolve"] and {"f64", "torn", "torn32", "block"} <= set(rep["ms_linsolve"])
    assert rep["ms_linsolve"][rep["linsolve"]] == min(rep["ms_linsolve"].values())
    rc, a, _ = dm.sweepx(2, times[:6], st.time, list(st.X), fixed_iter=3)
    dm.close()
    assert rc == 0
    lam = np.array([str(f).startswith("λ") for f in st.dis.fieldX])
    for d in range(3):
        assert _rel_dev(a[:, d][:, ~lam], ref[:, d][:, ~lam]) <= TOL_STATE, d


def test_pipelined_assembly_is_bitwise_the_synchronous_one():
    """mgpu_assemble_async/wait: five steps of different states and times with
    two in flight (both slots reused) give the synchronous call's Lλ and nzval
    bit for bit, static and Newmark; a NaN is reported at the wait."""
    m, _ = W.lattice(6, 5, 4)
    st = m.initialize()
    dm = DeviceModel(m, st.dis)
    c = REF.newmark_coefficients(2, 0.05, 0.25, 0.5)
    cases = [(_state(m, 20 + k, 1), 0.2 * (k + 1), _lib.ASM_STATIC, None) for k in range(3)]
    cases += [(_state(m, 30 + k, 3), 0.3 + 0.05 * k, mis, c) for k, mis in enumerate((_lib.ASM_STEP, _lib.ASM_ITER))]
    ref = [tuple(a.copy() for a in dm.assemble(X, t=t, mission=mis, c=cc)) for X, t, mis, cc in cases]
    got, pending = [], []
    for X, t, mis, cc in cases:
        tk, Ll, nz = dm.assemble_async(X, t=t, mission=mis, c=cc)
        pending.append((tk, Ll, nz))
        if len(pending) == 2:
            tk0, Ll0, nz0 = pending.pop(0)
            dm.assemble_wait(tk0)
            got.append((Ll0.copy(), nz0.copy()))
    tk0, Ll0, nz0 = pending.pop(0)
    dm.assemble_wait(tk0)
    got.append((Ll0.copy(), nz0.copy()))
    for (La, na), (Lb, nb) in zip(got, ref):
        assert np.array_equal(La, Lb) and np.array_equal(na, nb)
    x = np.zeros(m.ndof["X"])
    x[7] = np.nan
    tk, _, _ = dm.assemble_async([x], t=0.1)
    with pytest.raises(DeviceError) as e:
        dm.assemble_wait(tk)
    assert e.value.kind == "nan" and "returned NaN" in str(e.value)
    dm.close()


def test_nan_is_reported_like_the_reference():
    m, _ = W.cantilever()
    st = m.initialize()
    dm = DeviceModel(m, st.dis)
    x = np.zeros(m.ndof["X"])
    x[7] = np.nan
    with pytest.raises(DeviceError) as e:
        dm.assemble([x])
    assert e.value.kind == "nan" and "returned NaN" in str(e.value)
    dm.close()


def test_singular_matrix_is_reported():
    from muscade_gpu import SweepXGPU, solve

    m = Model()
    a = m.addnode([0.0, 0.0, 0.0])
    m.addelement(DofLoad, [a], field="t3", value=lambda t: 1.0)  # a dof without stiffness: Lλx = [0]
    st = m.initialize()
    with pytest.raises(DeviceError) as e:
        solve(SweepXGPU[0], st, [1.0])
    assert e.value.kind == "singular" and "matrix factorization failed at step=1, iiter=1" in str(e.value)
