"""The allocation-free beam assembly (mgpu_assemble_beams_noalloc).

Callers that cannot call cudaMalloc where they assemble -- inside a captured
CUDA graph, in a loop whose device memory was fixed beforehand, or when device
memory belongs to another runtime's pool -- pass their own device buffers to
this entry point; its only scratch is a fixed device array inside the library.
This test calls it through the C-ABI twice in a row (different states, so the
second call must not see the first call's scratch) and compares each result
with mgpu_assemble on a context built for the same beams and with the oracle's
assembly, within 1e-12 of the largest entry (mgpu_assemble sums the element
entries in the same order, so equality with it is expected to the last bit).
It also checks an element that lists one dof twice (its entries add into the
same places, one after the other, in the reference's entry order), an empty
call (the outputs are only zeroed), and times a call at the 4,096-beam limit.
"""
import ctypes

import numpy as np
import pytest

from muscade_gpu import _lib
from muscade_gpu.device import DeviceModel
from muscade_gpu.elements import BeamCrossSection, EulerBeam3D
from muscade_gpu.model import Model
from oracle import lib as O
from oracle import reference as REF

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
        # and the oracle's assembly (nested-dual elements, serial add_∂!)
        Lo, no = REF.assemble(REF.Prepared(m, st.dis), (xh,), (np.zeros(0),), 0.0, "static",
                              REF.newmark_coefficients(0, 1.0, 0.25, 0.5))
        assert np.max(np.abs(got_L - Lo)) <= TOL * np.max(np.abs(Lo)), call
        assert np.max(np.abs(got_n - no)) <= TOL * np.max(np.abs(no)), call
    dm.close()


def _call(lib, torch, nele, nX, nnz, fields, indexX, a1, a2, x, Ll, nz):
    dev = torch.device("cuda:0")
    stream = torch.cuda.current_stream(dev).cuda_stream
    return lib.mgpu_assemble_beams_noalloc(nele, nX, nnz, fields.data_ptr(), indexX.data_ptr(), a1.data_ptr(),
                                           a2.data_ptr(), x.data_ptr(), Ll.data_ptr(), nz.data_ptr(),
                                           ctypes.c_void_p(stream))


def test_noalloc_repeated_dof_and_empty_call():
    """An element whose dof list repeats a dof adds its entries into the same
    places one after the other, in the reference's entry order; nele = 0 only
    zeroes the outputs."""
    torch = pytest.importorskip("torch")
    _lib.build()
    lib = _lib.load()
    m = beams_only_model(n_nodes=12, n_beams=20, seed=4)
    st = m.initialize()
    idx = np.array(st.dis.dis[0].index_X, dtype=np.int64)
    idx[3, 8] = idx[3, 2]  # beam 4 lists one dof twice (a synthetic dof list)
    idx[9, 0] = idx[9, 11]
    nX = m.ndof["X"]
    colptr, rowval, asm1, asm2, nnz = REF.asm_pattern([idx], nX)
    ele = m.groups[0].cat("ele")
    xh = np.random.default_rng(8).normal(size=nX) * 0.05
    R, J = O.beam_eval(ele, xh[idx - 1][:, None, :], mode=1)
    Lexp, nexp = np.zeros(nX), np.zeros(nnz)
    O.scatter(asm1[0], asm2[0], R, J, Lexp, nexp)
    dev = torch.device("cuda:0")
    f = torch.tensor(ele, dtype=torch.float64, device=dev).contiguous()
    ix = torch.tensor(idx, dtype=torch.int64, device=dev).contiguous()
    a1 = torch.tensor(asm1[0], dtype=torch.int64, device=dev).contiguous()
    a2 = torch.tensor(asm2[0], dtype=torch.int64, device=dev).contiguous()
    x = torch.tensor(xh, dtype=torch.float64, device=dev)
    Ll = torch.full((nX,), 5.0, dtype=torch.float64, device=dev)
    nz = torch.full((nnz,), 5.0, dtype=torch.float64, device=dev)
    assert _call(lib, torch, m.groups[0].nele, nX, nnz, f, ix, a1, a2, x, Ll, nz) == 0
    torch.cuda.synchronize(dev)
    assert np.max(np.abs(Ll.cpu().numpy() - Lexp)) <= TOL * np.max(np.abs(Lexp))
    assert np.max(np.abs(nz.cpu().numpy() - nexp)) <= TOL * np.max(np.abs(nexp))
    Ll.fill_(5.0)
    nz.fill_(5.0)
    assert _call(lib, torch, 0, nX, nnz, f, ix, a1, a2, x, Ll, nz) == 0
    torch.cuda.synchronize(dev)
    assert not Ll.any().item() and not nz.any().item()


def test_noalloc_time_at_the_size_limit():
    """One call at MGPU_NOALLOC_MAX_BEAMS beams, timed with CUDA events on the
    call's stream (the figure is printed; the elements are summed one after
    another, so the call is latency-bound)."""
    torch = pytest.importorskip("torch")
    _lib.build()
    lib = _lib.load()
    m = beams_only_model(n_nodes=1500, n_beams=4096, seed=9)
    st = m.initialize()
    dm = DeviceModel(m, st.dis)
    asm1, asm2 = dm.asm(0)
    nnz = dm.nnz
    dm.close()
    nX = m.ndof["X"]
    dev = torch.device("cuda:0")
    f = torch.tensor(m.groups[0].cat("ele"), dtype=torch.float64, device=dev).contiguous()
    ix = torch.tensor(st.dis.dis[0].index_X, dtype=torch.int64, device=dev).contiguous()
    a1 = torch.tensor(asm1, dtype=torch.int64, device=dev).contiguous()
    a2 = torch.tensor(asm2, dtype=torch.int64, device=dev).contiguous()
    x = torch.tensor(np.random.default_rng(3).normal(size=nX) * 0.05, dtype=torch.float64, device=dev)
    Ll = torch.zeros(nX, dtype=torch.float64, device=dev)
    nz = torch.zeros(nnz, dtype=torch.float64, device=dev)
    assert _call(lib, torch, 4096, nX, nnz, f, ix, a1, a2, x, Ll, nz) == 0
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(3):
        assert _call(lib, torch, 4096, nX, nnz, f, ix, a1, a2, x, Ll, nz) == 0
    e1.record()
    torch.cuda.synchronize(dev)
    print(f"noalloc assembly of 4096 beams: {e0.elapsed_time(e1) / 3:.3f} ms per call")


def test_noalloc_rejects_too_many_beams():
    torch = pytest.importorskip("torch")
    lib = _lib.load()
    t = torch.zeros(8, dtype=torch.float64, device="cuda:0")
    i = torch.ones(8, dtype=torch.int64, device="cuda:0")
    p = [t.data_ptr(), i.data_ptr(), i.data_ptr(), i.data_ptr(), t.data_ptr(), t.data_ptr(), t.data_ptr()]
    rc = lib.mgpu_assemble_beams_noalloc(4097, 1, 1, *p, None)  # size is checked before any device work
    assert rc == 8  # MGPU_ERR_SIZE
