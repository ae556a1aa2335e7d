"""Host logic of the product (CPU): model numbering, element fields, the
C-ABI library's exports, and the workload generators."""
import ctypes
import math
import os
import re

import numpy as np
import pytest

from conftest import ROOT, julia_isapprox as approx
from muscade_gpu import _lib
from muscade_gpu import workloads as W
from muscade_gpu.elements import BeamCrossSection, EulerBeam3D, beam_fields
from muscade_gpu.model import Model
from oracle import lib as O
from oracle import reference as REF


def test_numbering_matches_reference_golden(golden):  # test/TestAssemble.jl:53-67 via the oracle's test elements
    from oracle import testelements as TE

    m = Model()
    n1 = m.addnode([0, 0, 100.0])
    n2 = m.addnode([])
    n3 = m.addnode([])
    m.addelement(TE.Turbine, [n1, n2], seadrag=2.0, sea=None, skydrag=3.0, sky=None)
    m.addelement(TE.AnchorLine, [n1, n3], Dxmtop=[5.0, 0, 0], xmbot=[150.0, 0], L=180.0, buoyancy=-1e3)
    dis = m.initialize().dis
    assert dis.dis[0].index_X.tolist() == [[1, 2]]
    assert dis.dis[1].index_A.tolist() == [[3, 4]]
    assert dis.fieldX == ["tx1", "tx2", "rx3"]


def test_batched_numbering_equals_sequential():
    """Vectorised addelement with a node matrix numbers dofs like element-by-element calls."""
    rng = np.random.default_rng(3)
    ne = 40
    pairs = rng.integers(1, 16, size=(ne, 2))
    pairs = pairs[pairs[:, 0] != pairs[:, 1]]
    mat = BeamCrossSection(EA=1.0, EI2=1.0, EI3=1.0, GJ=1.0, mu=1.0, iota1=1.0)

    def build(batched):
        m = Model()
        m.addnode(np.stack([np.arange(15.0), np.arange(15.0) ** 1.3, np.zeros(15)], axis=1))
        if batched:
            m.addelement(EulerBeam3D, pairs, mat=mat, orient2=(0.0, 0.0, 1.0))
        else:
            for p in pairs:
                m.addelement(EulerBeam3D, p, mat=mat, orient2=(0.0, 0.0, 1.0))
        return m.initialize().dis.dis[0].index_X

    assert np.array_equal(build(True), build(False))


def test_beam_fields_match_oracle_constructor():
    rng = np.random.default_rng(4)
    n = 50
    c1 = rng.normal(size=(n, 3))
    c2 = c1 + rng.normal(size=(n, 3))
    o2 = rng.normal(size=(n, 3))
    mat = BeamCrossSection(EA=rng.uniform(1, 2, n), EI2=2.0, EI3=3.0, GJ=4.0, mu=5.0, iota1=6.0, w=0.5)
    ours = beam_fields(c1, c2, o2, mat.array(n))
    ref = O.beam_construct(c1, c2, o2, mat.array(n))
    assert np.max(np.abs(ours - ref)) <= 1e-14 * np.max(np.abs(ref))


def test_library_exports_every_declared_symbol():
    _lib.build()
    hdr = open(os.path.join(ROOT, "include", "muscade_gpu.h")).read()
    declared = set(re.findall(r"\b(mgpu_[A-Za-z_0-9]+)\s*\(", hdr))
    L = ctypes.CDLL(_lib.LIB)
    missing = [s for s in sorted(declared) if not hasattr(L, s)]
    assert not missing, missing
    assert declared >= set(_lib.SYMBOLS)


def test_workload_sizes():
    m, times = W.cantilever()
    assert m.ndof["X"] == 132 and len(times) == 10
    prep = REF.Prepared(m, m.initialize().dis)
    assert prep.nnz == 2214  # 20·144+6·4+1 element entries over 2,214 distinct pairs
    m, _ = W.lattice(6, 5, 4)
    nb = 5 * 5 * 4 + 6 * 4 * 4 + 6 * 5 * 3
    assert m.groups[0].nele == nb
    assert sum(g.nele for g in m.groups if g.key[1] == (1,) and g.key[0] == "DofConstraint") == 6 * 30
    m, t = W.risers(nriser=3, nel=10)
    assert m.ndof["X"] == 3 * (11 * 6 + 7) and len(t) == 2000
