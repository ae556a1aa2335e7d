"""The device element code (csrc/beam_math.hpp and bar_math.hpp, the bodies
of beam_kernel and bar_kernel) compiled for the host and compared with the
oracle's nested-dual evaluation of the same elements: R and the Newton matrix
of SweepX{0} (K) and of a Newmark iteration (K + a₁C + b₁M) for beams, R, K,
C and M for bars, within the element tolerance.  No GPU needed."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from muscade_gpu import workloads as W
from muscade_gpu.elements import AxisymmetricBarCrossSection, Bar3D
from muscade_gpu.model import Model
from oracle import lib as O
from oracle import reference as REF

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "muscade.jl_gb300", "csrc")
TOL = 1e-12  # relative to the largest entry, as the assembly parity tests


@pytest.fixture(scope="module")
def host_eval(tmp_path_factory):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no host C++ compiler")
    exe = str(tmp_path_factory.mktemp("ele") / "element_host_eval")
    subprocess.run([cxx, "-O2", "-std=c++17", "-I", CSRC, os.path.join(HERE, "element_host_eval.cpp"), "-o", exe],
                   check=True, capture_output=True)

    def run(kind, fields, X0, X1, X2, nder, p=(1.0, 0.0, 0.0), t=0.0):
        nx = X0.shape[1]
        lines = [f"{kind} {len(fields)} {nder} {p[0]!r} {p[1]!r} {p[2]!r} {t!r}"]
        for f, x0, x1, x2 in zip(fields, X0, X1, X2):
            lines.append(" ".join(repr(float(v)) for v in np.concatenate([f, x0, x1, x2])))
        out = subprocess.run([exe], input="\n".join(lines) + "\n", check=True, capture_output=True, text=True).stdout
        a = np.array([[float(v) for v in ln.split()] for ln in out.strip().splitlines()])
        return a[:, :nx], a[:, nx:].reshape(-1, nx, nx).transpose(0, 2, 1)  # K[e][i][j]

    return run


def _relerr(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


MODELS = {"cantilever": lambda: W.cantilever()[0], "lattice": lambda: W.lattice(5, 4, 3)[0],
          "risers": lambda: W.risers(nriser=2, nel=10)[0]}


@pytest.mark.parametrize("rot", ["rotated", "zero rotations"])
@pytest.mark.parametrize("name", list(MODELS))
def test_device_beam_code_matches_the_oracle(name, rot, host_eval):
    """Random states, and states whose nodal rotation dofs are zero (the
    θ = 0 branch of Rodrigues, taken at the start of every sweep)."""
    m = MODELS[name]()
    st = m.initialize()
    rng = np.random.default_rng(11)
    n = m.ndof["X"]
    X = [rng.normal(size=n) * 0.05 for _ in range(3)]
    if rot == "zero rotations":
        for f in ("r1", "r2", "r3"):
            for x in X:
                x[np.array([str(v) == f for v in st.dis.fieldX])] = 0.0
    U = (np.zeros(m.ndof["U"]),)
    c = REF.newmark_coefficients(2, 0.05, 0.25, 0.5)
    checked = 0
    for g, dg in zip(m.groups, st.dis.dis):
        if REF.group_kind(g) != "EulerBeam3D" or g.nele == 0:
            continue
        idx = dg.index_X - 1
        Xe = [x[idx] for x in X]
        fields = g.cat("ele")
        for mode, mref, cc in ((1, "static", REF.newmark_coefficients(0, 1.0, 0.25, 0.5)), (3, "iter", c)):
            Xs = (X[0],) if mode == 1 else tuple(X)
            Rr, Jr = REF.eval_group(m, g, dg, Xs, U, 0.3, mode, cc)
            nder = 1 if mode == 1 else 3
            Rh, Kh = host_eval("beam", fields, Xe[0], Xe[1], Xe[2], nder, (1.0, cc.get("a1", 0.0), cc.get("b1", 0.0)))
            assert _relerr(Rh, Rr) <= TOL, (name, mref)
            assert _relerr(Kh, Jr[:, :, :12]) <= TOL, (name, mref)
            checked += 1
    assert checked >= 2


def test_device_bar_code_matches_the_oracle(host_eval):
    rng = np.random.default_rng(5)
    n = 32
    m = Model()
    c1 = rng.normal(size=(n, 3))
    ids1 = m.addnode(c1)
    ids2 = m.addnode(c1 + rng.normal(size=(n, 3)))
    mat = AxisymmetricBarCrossSection(EA=10.0, mu=1.0, w=2.0, Cat=0.2, Clt=0.3, Cqt=0.4, Can=0.5, Cln=0.6, Cqn=0.7)
    m.addelement(Bar3D, np.stack([ids1, ids2], axis=1), mat=mat)
    fields = m.groups[0].cat("ele")
    X = rng.normal(size=(n, 3, 6)) * 0.3
    d = O.diffed("bar", fields, X, t=-7.0)
    for p, name in (((1.0, 0.0, 0.0), "K"), ((0.0, 1.0, 0.0), "C"), ((0.0, 0.0, 1.0), "M")):
        Rh, Kh = host_eval("bar", fields, X[:, 0], X[:, 1], X[:, 2], 3, p, -7.0)
        assert _relerr(Rh, d["R"]) <= TOL
        assert _relerr(Kh, d[name]) <= TOL, name
