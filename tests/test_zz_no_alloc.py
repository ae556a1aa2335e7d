"""The allocation-free beam assembly (mgpu_assemble_beams_noalloc).

Callers that cannot call cudaMalloc where they assemble -- inside a captured
CUDA graph, in a loop whose device memory was fixed beforehand, or when device
memory belongs to another runtime's pool -- pass their own device buffers to
this entry point; its only scratch is a fixed device array inside the library.
This test calls it through the C-ABI twice in a row (different states, so the
second call must not see the first call's scratch) and compares each result
with mgpu_assemble on a context built for the same beams, within 1e-12 of the
largest entry (both sum the element entries in the same order, so equality is
expected to the last bit).
"""
import ctypes

import numpy as np
import pytest

from muscade_gpu import _lib
from muscade_gpu.device import DeviceModel
from muscade_gpu.elements import BeamCrossSection, EulerBeam3D
from muscade_gpu.model import Model

pytestmark = pytest.mark.gpu
TOL = 1e-12


def beams_only_model(n_nodes=40, n_beams=90, seed=21):
    rng = np.random.default_rng(seed)
    m = Model()
    m.addnode(rng.normal(size=(n_nodes, 3)) * 3.0)
    pairs = []
    while len(pairs) < n_beams:
        a, b = rng.integers(1, n_nodes + 1, size=2)
        if a != b:
            pairs.append((a, b))
    mat = BeamCrossSection(EA=1e6 * rng.uniform(1, 2, n_beams), EI2=1e3, EI3=2e3, GJ=5e2, mu=1.0, iota1=0.1, w=3.0)
    m.addelement(EulerBeam3D, np.array(pairs), mat=mat, orient2=rng.normal(size=(n_beams, 3)))
    return m


def test_noalloc_assembly_matches_context_assembly_twice():
    torch = pytest.importorskip("torch")
    _lib.build()
    lib = _lib.load()
    m = beams_only_model()
    st = m.initialize()
    dm = DeviceModel(m, st.dis)
    asm1, asm2 = dm.asm(0)
    nele = m.groups[0].nele
    nX, nnz = m.ndof["X"], dm.nnz
    dev = torch.device("cuda:0")
    fields = torch.tensor(m.groups[0].cat("ele"), dtype=torch.float64, device=dev).contiguous()
    indexX = torch.tensor(st.dis.dis[0].index_X, dtype=torch.int64, device=dev).contiguous()
    a1 = torch.tensor(asm1, dtype=torch.int64, device=dev).contiguous()
    a2 = torch.tensor(asm2, dtype=torch.int64, device=dev).contiguous()
    Ll = torch.full((nX,), 7.0, dtype=torch.float64, device=dev)  # stale values must be overwritten
    nz = torch.full((nnz,), -3.0, dtype=torch.float64, device=dev)
    rng = np.random.default_rng(5)
    for call in range(2):
        xh = rng.normal(size=nX) * (0.02 if call == 0 else 0.2)
        x = torch.tensor(xh, dtype=torch.float64, device=dev)
        stream = torch.cuda.current_stream(dev).cuda_stream
        rc = lib.mgpu_assemble_beams_noalloc(nele, nX, nnz, fields.data_ptr(), indexX.data_ptr(), a1.data_ptr(),
                                             a2.data_ptr(), x.data_ptr(), Ll.data_ptr(), nz.data_ptr(),
                                             ctypes.c_void_p(stream))
        assert rc == 0, rc
        torch.cuda.synchronize(dev)
        Lref, nref = dm.assemble([xh])
        got_L, got_n = Ll.cpu().numpy(), nz.cpu().numpy()
        assert np.max(np.abs(got_L - Lref)) <= TOL * np.max(np.abs(Lref)), call
        assert np.max(np.abs(got_n - nref)) <= TOL * np.max(np.abs(nref)), call
    dm.close()


def test_noalloc_rejects_too_many_beams():
    torch = pytest.importorskip("torch")
    lib = _lib.load()
    t = torch.zeros(8, dtype=torch.float64, device="cuda:0")
    i = torch.ones(8, dtype=torch.int64, device="cuda:0")
    p = [t.data_ptr(), i.data_ptr(), i.data_ptr(), i.data_ptr(), t.data_ptr(), t.data_ptr(), t.data_ptr()]
    rc = lib.mgpu_assemble_beams_noalloc(4097, 1, 1, *p, None)  # size is checked before any device work
    assert rc == 8  # MGPU_ERR_SIZE
