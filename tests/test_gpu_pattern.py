"""The pattern of Lλx and the gather plans built on the device (a stable radix
sort of the element entries, pattern_dev.cu) against the host construction
(GPU): colptr, rowval and the asm maps bit-exact, and the assembled Lλ and
nzval bitwise equal (the plans list the same entries in the same order).  The
host construction is itself bit-exact against the oracle's asmmat!; models of
4 M element entries or more (the 60×60×20 lattice) use the device build by
default, and the benchmark-size test compares that one with the oracle.
"""
import numpy as np
import pytest

from muscade_gpu import _lib
from muscade_gpu import workloads as W
from muscade_gpu.device import DeviceModel

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built():
    _lib.build()


def _models():
    yield "lattice 7x6x4", *W.lattice(7, 6, 4)
    yield "risers 3x20", *W.risers(nriser=3, nel=20)
    params = W.batched_params(20, nel_range=(10, 40), seed=9)
    mb, _, tb = W.build_batched(params)
    yield "batched 20", mb, tb
    d0 = W.adjoint_beam(nel=15, nstep=3)
    y = np.zeros((3, len(d0["sensors"])))
    d = W.adjoint_beam(nel=15, nstep=3, measurements=(y, 1.0), a_weight=1.0)
    yield "costs", d["model"], d["times"]


@pytest.mark.parametrize("case", range(4))
def test_device_pattern_equals_host_pattern(monkeypatch, case):
    name, m, times = list(_models())[case]
    st = m.initialize(time=0.0) if name in ("risers 3x20", "costs") else m.initialize()
    out = {}
    for flag in ("0", "1"):
        monkeypatch.setenv("MGPU_DEVICE_PATTERN", flag)
        dm = DeviceModel(m, st.dis)
        if m.ndof["A"]:
            dm.set_A(np.ones(m.ndof["A"]))
        cp, rv = dm.pattern()
        asms = [dm.asm(ig) for ig in range(len(m.groups))]
        X = [np.random.default_rng(3).normal(size=m.ndof["X"]) * 1e-3]
        Ll, nz = dm.assemble(X, t=float(times[0]))
        dm.close()
        out[flag] = (cp, rv, asms, Ll, nz)
    h, d = out["0"], out["1"]
    assert np.array_equal(h[0], d[0]) and np.array_equal(h[1], d[1]), name
    for (a1, a2), (b1, b2) in zip(h[2], d[2]):
        assert np.array_equal(a1, b1) and np.array_equal(a2, b2), name
    assert np.array_equal(h[3], d[3]) and np.array_equal(h[4], d[4]), name
