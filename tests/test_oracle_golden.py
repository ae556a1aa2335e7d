"""The oracle against the reference's own golden values (CPU).

Each test restates one of the reference's unit tests: the same inputs and the
same expected numbers (copied from test/*.jl by tests/golden/extract_golden.py
where they are numeric, restated as the closed forms the test writes where
they are analytic) and Julia's `≈` semantics (norm-wise, rtol = √eps).
"""
import math

import numpy as np
import pytest

from conftest import julia_isapprox as approx
from oracle import lib as O
from oracle import reference as REF
from oracle import testelements as TE
from muscade_gpu.model import Model


# ------------------------------------------------------------------ rotations
def test_sinc1_and_derivatives(golden):  # test/TestRotations.jl:6-13
    th = golden["sinc1_theta"]["value"]
    for k in range(5):
        got = [O.sinc1k(k, x) for x in th]
        assert approx(got, golden[f"sinc1_d{k}"]["value"]), k


def test_scac_nested_derivatives(golden):  # test/TestRotations.jl:31-64
    xs = golden["scac_x"]["value"]
    got = np.array([O.scac_derivs(x) for x in xs])
    for k in range(5):
        assert approx(got[:, k], golden[f"scac_d{k}"]["value"]), k


@pytest.mark.parametrize("v", [[0.1, 0.2, 0.3], [1e-7, 2e-7, 1e-8], [0.0, 0.0, 0.0]])
def test_rodrigues_roundtrip(v):  # test/TestRotations.jl:89-111
    w, J = O.rodrigues_roundtrip(v)
    assert approx(w, v)
    assert approx(J, np.eye(3))


# ------------------------------------------------------------------ beam
def _beam(c2, EA, EI2, EI3, GJ, mu, iota1, **kw):
    mat = np.array([EA, EI2, EI3, GJ, mu, iota1, kw.get("w", 0.0), kw.get("Ca1", 0.0), kw.get("Cl1", 0.0),
                    kw.get("Cq1", 0.0), kw.get("Ca2", 0.0), kw.get("Cl2", 0.0), kw.get("Cq2", 0.0),
                    kw.get("Ca3", 0.0), kw.get("Cl3", 0.0), kw.get("Cq3", 0.0)])
    return O.beam_construct([0.0, 0.0, 0.0], c2, [0.0, 1.0, 0.0], mat)


def test_beam_constructor(golden):  # test/TestBeamElement.jl:15-31
    f = _beam([4.0, 3.0, 0.0], 10.0, 3.0, 3.0, 4.0, 1.0, 1.0)[0]
    L = 5.0
    assert approx(f[0:3], golden["beam_cm"]["value"])
    rm = np.array(golden["beam_rm"]["value"])
    assert approx(f[3:12].reshape(3, 3, order="F"), rm)
    assert approx(f[12:16], golden["beam_zgp"]["value"])
    assert approx(f[16:18], golden["beam_znod"]["value"])
    assert approx(f[18:21], golden["beam_tgm"]["value"])
    assert approx(f[21:24], golden["beam_tge"]["value"])
    assert approx(f[24:28], golden["beam_ya"]["value"])
    assert approx(f[28:32], golden["beam_yu"]["value"])
    assert approx(f[32:36], np.array(golden["beam_yv"]["value"]) * L)
    assert approx(f[36:40], np.array(golden["beam_ka"]["value"]) / L)
    assert approx(f[40:44], np.array(golden["beam_ku"]["value"]) / L**2)
    assert approx(f[44:48], np.array(golden["beam_kv"]["value"]) / L)
    assert approx(f[49:53], np.array(golden["beam_dL"]["value"]) * L)


EA, EI2, EI3, GJ, L, MU, IOTA = 10.0, 3.0, 2.0, 4.0, 2.0, 1.0, 5.0


def _res(x, **kw):
    f = _beam([L, 0.0, 0.0], EA, EI2, EI3, GJ, kw.pop("mu", MU), IOTA, **kw)
    X = np.asarray(x, dtype=float)[None]
    R, _ = O.beam_eval(f, X, mode=0)
    return R[0]


def test_beam_residual_tension():  # test/TestBeamElement.jl:52-58
    d = 0.1
    x = np.zeros(12)
    x[6] = d
    assert approx(_res(x), [-EA / L * d, 0, 0, 0, 0, 0, EA / L * d, 0, 0, 0, 0, 0])


def test_beam_residual_flex_translation():  # :60-66 (atol=1e-2)
    d = 0.01
    x = np.zeros(12)
    x[7] = d
    ref = [0, -12 * EI3 / L**3 * d, 0, 0, 0, -6 * EI3 / L**2 * d, 0, 12 * EI3 / L**3 * d, 0, 0, 0, -6 * EI3 / L**2 * d]
    assert approx(_res(x), ref, rtol=0.0, atol=1e-2)


def test_beam_residual_flex_rotation():  # :68-74 (atol=1e-2)
    r = 0.01
    x = np.zeros(12)
    x[11] = r
    ref = [0, 6 * EI3 / L**2 * r, 0, 0, 0, 2 * EI3 / L * r, 0, -6 * EI3 / L**2 * r, 0, 0, 0, 4 * EI3 / L * r]
    assert approx(_res(x), ref, rtol=0.0, atol=1e-2)


def test_beam_residual_torsion():  # :76-82
    r = 0.1
    x = np.zeros(12)
    x[9] = r
    assert approx(_res(x), [0, 0, 0, -GJ / L * r, 0, 0, 0, 0, 0, GJ / L * r, 0, 0])


def _diffed_zero():
    f = _beam([L, 0.0, 0.0], EA, EI2, EI3, GJ, MU, IOTA)
    return O.diffed("beam", f, np.zeros((1, 3, 12)))


def test_beam_stiffness():  # :107-172
    K = _diffed_zero()["K"][0]
    k = lambda i, j: K[i - 1, j - 1]  # noqa: E731
    checks = [((1, 1), EA / L), ((7, 7), EA / L), ((1, 7), -EA / L), ((7, 1), -EA / L),
              ((2, 2), 12 * EI3 / L**3), ((8, 8), 12 * EI3 / L**3), ((3, 3), 12 * EI2 / L**3), ((9, 9), 12 * EI2 / L**3),
              ((3, 9), -12 * EI2 / L**3), ((9, 3), -12 * EI2 / L**3), ((2, 8), -12 * EI3 / L**3), ((8, 2), -12 * EI3 / L**3),
              ((8, 6), -6 * EI3 / L**2), ((2, 12), 6 * EI3 / L**2), ((9, 5), 6 * EI2 / L**2), ((3, 11), -6 * EI2 / L**2),
              ((5, 5), 4 * EI2 / L), ((11, 11), 4 * EI2 / L), ((6, 6), 4 * EI3 / L), ((12, 12), 4 * EI3 / L),
              ((5, 11), 2 * EI2 / L), ((11, 5), 2 * EI2 / L), ((6, 12), 2 * EI3 / L), ((12, 6), 2 * EI3 / L),
              ((5, 9), 6 * EI2 / L**2), ((11, 3), -6 * EI2 / L**2), ((6, 8), -6 * EI3 / L**2), ((12, 2), 6 * EI3 / L**2),
              ((4, 4), GJ / L), ((10, 10), GJ / L), ((4, 10), -GJ / L), ((10, 4), -GJ / L)]
    for (i, j), v in checks:
        assert approx(k(i, j), v), (i, j)
    spurious = {1: [2, 3, 4, 5, 6, 8, 9, 10, 11, 12], 7: [2, 3, 4, 5, 6, 8, 9, 10, 11, 12],
                4: [1, 2, 3, 5, 6, 7, 8, 9, 11, 12], 10: [1, 2, 3, 5, 6, 7, 8, 9, 11, 12],
                2: [1, 3, 4, 5, 7, 9, 10, 11], 3: [1, 2, 4, 6, 7, 8, 10, 12], 8: [1, 3, 4, 5, 7, 9, 10, 11],
                9: [1, 2, 4, 6, 7, 8, 10, 12], 5: [1, 2, 4, 6, 7, 8, 10, 12], 6: [1, 3, 4, 5, 7, 9, 10, 11],
                11: [1, 2, 4, 6, 7, 8, 10, 12], 12: [1, 3, 4, 5, 7, 9, 10, 11]}
    for i, cols in spurious.items():
        assert np.linalg.norm(K[i - 1, np.array(cols) - 1]) <= 1e-12 * EA / L, i


def test_beam_mass():  # :175-239
    M = _diffed_zero()["M"][0]
    m = lambda i, j: M[i - 1, j - 1]  # noqa: E731
    checks = [((1, 1), MU * L / 3), ((7, 7), MU * L / 3), ((1, 7), MU * L / 6), ((7, 1), MU * L / 6),
              ((8, 8), 156 * MU * L / 420), ((2, 2), 156 * MU * L / 420), ((3, 3), 156 * MU * L / 420),
              ((9, 9), 156 * MU * L / 420), ((3, 9), 54 * MU * L / 420), ((9, 3), 54 * MU * L / 420),
              ((2, 8), 54 * MU * L / 420), ((8, 2), 54 * MU * L / 420), ((8, 6), 13 * MU * L**2 / 420),
              ((2, 12), -13 * MU * L**2 / 420), ((9, 5), -13 * MU * L**2 / 420), ((3, 11), 13 * MU * L**2 / 420),
              ((5, 5), 4 * MU * L**3 / 420), ((11, 11), 4 * MU * L**3 / 420), ((6, 6), 4 * MU * L**3 / 420),
              ((12, 12), 4 * MU * L**3 / 420), ((5, 11), -3 * MU * L**3 / 420), ((11, 5), -3 * MU * L**3 / 420),
              ((6, 12), -3 * MU * L**3 / 420), ((12, 6), -3 * MU * L**3 / 420), ((5, 9), -13 * MU * L**2 / 420),
              ((11, 3), 13 * MU * L**2 / 420), ((6, 8), 13 * MU * L**2 / 420), ((12, 2), -13 * MU * L**2 / 420),
              ((4, 4), IOTA * L / 4), ((10, 10), IOTA * L / 4), ((4, 10), IOTA * L / 4), ((10, 4), IOTA * L / 4)]
    for (i, j), v in checks:
        assert approx(m(i, j), v), (i, j)


def test_beam_weight():  # :242-255
    w = 10.0
    x = np.zeros(12)
    x[4] = w * L**3 / (24 * EI2)
    x[10] = -w * L**3 / (24 * EI2)
    assert approx(_res(x, w=w), [0, 0, w * L / 2, 0, 0, 0, 0, 0, w * L / 2, 0, 0, 0])


def test_beam_added_mass_and_damping():  # :257-326
    f = _beam([L, 0.0, 0.0], EA, EI2, EI3, GJ, 1.0, IOTA, Ca1=1.0, Ca2=2.0, Ca3=3.0)
    a1 = 4.0
    X = np.zeros((1, 3, 12))
    X[0, 2, 0] = X[0, 2, 6] = a1
    R, _ = O.beam_eval(f, X, mode=0)
    assert approx(R[0], [(1 + 1.0) * a1 * L / 2, 0, 0, 0, 0, 0, (1 + 1.0) * a1 * L / 2, 0, 0, 0, 0, 0])
    f = _beam([L, 0.0, 0.0], EA, EI2, EI3, GJ, 1.0, IOTA, Cl1=1.0, Cl2=2.0, Cl3=3.0, Cq1=0.1, Cq2=0.2, Cq3=0.3)
    v1 = 1.0
    X = np.zeros((1, 3, 12))
    X[0, 1, 0] = X[0, 1, 6] = v1
    R, _ = O.beam_eval(f, X, mode=0)
    q = (1.0 + 0.1 * abs(v1)) * v1 * L / 2
    assert approx(R[0], [q, 0, 0, 0, 0, 0, q, 0, 0, 0, 0, 0])


# ------------------------------------------------------------------ bar
def test_bar_constructor_and_residuals(golden):  # test/TestBarElement.jl
    EAb, L0, mub = 10.0, 2.0, 1.0
    mat = np.array([EAb, mub, 0, 0, 0, 0, 0, 0, 0.0])
    f = O.bar_construct([0, 0, 0.0], [L0, 0, 0.0], mat)
    assert approx(f[0, 20:24], golden["bar_wgp"]["value"])
    assert approx(f[0, 24:28], golden["bar_zgp"]["value"])
    assert approx(f[0, 30:34], golden["bar_psi1"]["value"])
    assert approx(f[0, 34:38], golden["bar_psi2"]["value"])
    dx = 0.1
    X = np.zeros((1, 1, 6))
    X[0, 0, 3] = dx
    R, _ = O.bar_eval(f, X, mode=0)
    assert approx(R[0], [-EAb / L0 * dx, 0, 0, EAb / L0 * dx, 0, 0])
    X = np.zeros((1, 3, 6))
    X[0, 0, 3] = dx
    d = O.diffed("bar", f, X)
    K, M = d["K"][0], d["M"][0]
    kt = (EAb / L0) * dx / (L0 + dx)
    for (i, j), v in [((1, 1), EAb / L0), ((4, 4), EAb / L0), ((1, 4), -EAb / L0), ((2, 2), kt), ((3, 3), kt),
                      ((5, 5), kt), ((6, 6), kt), ((2, 5), -kt), ((3, 6), -kt)]:
        assert approx(K[i - 1, j - 1], v, rtol=1e-6), (i, j)
    for (i, j), v in [((1, 1), mub * L0 / 3), ((2, 2), mub * L0 / 3), ((1, 4), mub * L0 / 6), ((3, 6), mub * L0 / 6)]:
        assert approx(M[i - 1, j - 1], v), (i, j)
    w = 10.0
    f = O.bar_construct([0, 0, 0.0], [L0, 0, 0.0], np.array([EAb, mub, w, 0, 0, 0, 0, 0, 0.0]))
    R, _ = O.bar_eval(f, np.zeros((1, 1, 6)), mode=0, t=0.0)
    assert approx(R[0], [0, 0, w * L0 / 2, 0, 0, w * L0 / 2])


# ------------------------------------------------------------------ assembly and solvers
def _turbine_anchor_model(sea_t=False, three=False):
    m = Model("TestModel")
    n1 = m.addnode([0, 0, 100.0])
    n2 = m.addnode([])
    n3 = m.addnode([])
    if not three:
        m.addelement(TE.Turbine, [n1, n2], seadrag=2.0, sea=lambda t, x: [1.0, 0.0], skydrag=3.0,
                     sky=lambda t, x: [0.0, 1.0])
        m.addelement(TE.AnchorLine, [n1, n3], Dxmtop=[5.0, 0, 0], xmbot=[150.0, 0], L=180.0, buoyancy=-1e3)
    else:
        m.addelement(TE.Turbine, [n1, n2], seadrag=1e6, sea=lambda t, x: [1.0 * t, 0.0], skydrag=1e5,
                     sky=lambda t, x: [0.0, 10.0])
        for i in range(3):
            al = np.array([math.cos(i * 2 * math.pi / 3), math.sin(i * 2 * math.pi / 3)])
            m.addelement(TE.AnchorLine, [n1, n3], Dxmtop=list(5 * al) + [0.0], xmbot=250 * al, L=290.0,
                         buoyancy=-5e3)
    return m


def test_disassembler_and_asm(golden):  # test/TestAssemble.jl:43-127
    m = _turbine_anchor_model()
    st = m.initialize()
    dis = st.dis
    assert dis.dis[0].index_X.tolist() == [[1, 2]] and dis.dis[0].index_A.tolist() == [[1, 2]]
    assert dis.dis[1].index_X.tolist() == [[1, 2, 3]] and dis.dis[1].index_A.tolist() == [[3, 4]]
    assert dis.fieldX == ["tx1", "tx2", "rx3"]
    prep = REF.Prepared(m, dis)
    assert prep.asm1[0].reshape(-1).tolist() == golden["asm_1_1"]["value"]
    assert prep.asm1[1].reshape(-1).tolist() == golden["asm_1_2"]["value"]
    assert prep.asm2[0].reshape(-1).tolist() == golden["asm_2_1"]["value"]
    assert prep.asm2[1].reshape(-1).tolist() == golden["asm_2_2"]["value"]


def test_assemble_values(golden):  # test/TestAssemble.jl:152-158
    m = _turbine_anchor_model()
    st = m.initialize()
    prep = REF.Prepared(m, st.dis)
    Ll, nz = REF.assemble(prep, (np.zeros(3),), (np.zeros(0),), -math.inf, "static", REF.newmark_coefficients(0, 1, 0.25, 0.5))
    assert approx(Ll, golden["assemble_Ll"]["value"])
    g = golden["assemble_Llx"]
    A = np.zeros((3, 3))
    A[np.array(g["I"]) - 1, np.array(g["J"]) - 1] = g["V"]
    assert approx(prep.matrix(nz).toarray(), A)


def test_sweepx0(golden):  # test/TestSweepX0.jl:9-29
    m = _turbine_anchor_model(three=True)
    st = m.initialize()
    out = REF.sweepx(m, st.dis, st, [0.0, 1.0], OX=0)
    assert approx(out[0][1][0], golden["sweepx0_X"]["value"])


def test_sweepx2_newmark(golden):  # test/TestSweepX2.jl:9-24
    m = Model("TestModel")
    nd = m.addnode([])
    m.addelement(TE.SdofOscillator, [nd], K1=1.0, K2=0.3, C1=1.0, C2=2.0, M1=3.0)
    st = m.initialize(time=0.0).copy(nXder=2)
    st.X[1][0] = 1.0
    out = REF.sweepx(m, st.dis, st, 0.4 * np.arange(1, 101), OX=2)
    X = np.array([o[1][d][0] for o in out for d in range(3)]).reshape(-1, 3)
    assert approx(X[::10, 0], golden["sweepx2_X"]["value"])
    assert approx(X[::10, 1], golden["sweepx2_X1"]["value"])
    assert approx(X[::10, 2], golden["sweepx2_X2"]["value"])


def test_dofconstraint_equal(golden):  # test/TestDofConstraints.jl:27-46, gap .3x1+.4x2
    from muscade_gpu.elements import DofConstraint

    m = Model("TestModel")
    n1 = m.addnode([0.0])
    m.addelement(DofConstraint, [n1], xinod=(1, 1), xfield=("t1", "t2"), lfield="λ", coeffs=[0.3, 0.4], offset=None)
    st = m.initialize()
    prep = REF.Prepared(m, st.dis)
    for x, key in (([4.0, -3.0, 10.0], "dofcon_equal_contact_R"), ([4.0, 3.0, 10.0], "dofcon_equal_gap_R")):
        Ll, nz = REF.assemble(prep, (np.array(x),), (np.zeros(0),), 0.0, "static", REF.newmark_coefficients(0, 1, 0.25, 0.5))
        assert approx(Ll, golden[key]["value"])
        assert approx(prep.matrix(nz).toarray(), [[0, 0, -0.3], [0, 0, -0.4], [-0.3, -0.4, 0]])


def _bend_tips(model, dis, states, tip):
    nod = np.asarray(model.dof_node["X"])
    fx = list(dis.fieldX)
    xyz0 = np.asarray(model.coord(tip))
    idx = [next(i for i in range(len(fx)) if fx[i] == f and nod[i] == tip) for f in ("t1", "t2", "t3")]
    return [xyz0 + np.asarray(X)[idx] for X in states]


def test_bend45_oracle_against_literature(golden):
    """The 45° cantilever bend of examples/StaticBeamAnalysis.jl:10-36, solved by
    the oracle's SweepX{0}: the tip coordinates at 300, 450 and 600 N agree with
    both published solutions the example quotes (:131-134) within 0.1 m (the
    two solutions differ from each other by up to 0.07 m)."""
    from muscade_gpu import workloads as W
    model, times, tip = W.bend45()
    st = model.initialize()
    ref = REF.sweepx(model, st.dis, st, times, OX=0, maxdx=1e-9)
    tips = _bend_tips(model, st.dis, [X[0] for _, X in ref[1:]], tip)
    for key in ("bend_tip_longva", "bend_tip_crisfield"):
        lit = np.asarray(golden[key]["value"])
        err = np.max(np.abs(np.asarray(tips) - lit))
        assert err <= 0.1, (key, tips, lit)
