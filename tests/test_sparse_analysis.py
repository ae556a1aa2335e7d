"""The sparse direct solver's host analysis (CPU): ordering, symbolic
factorisation and assembly maps (muscade.jl_gb300/csrc/sparse_analysis.cpp,
compiled for the host from the same source).

A numpy multifrontal factorisation driven only by the analysis output -- the
matrix entries placed by `amap`, the children's Schur complements added
through `emap` in child order, partial LU of each front's pivots without
pivoting, then forward and backward substitution over the fronts -- must solve
Lλx Δx = Lλ like a sparse direct solve (scipy SuperLU) of the same assembled
system.  The system is equilibrated as the device solver does it, D Lλx D
with D = 1/√|diagonal| and, for a zero-diagonal multiplier, the scale that
makes its largest entry one in magnitude; the unscaled matrices have condition
numbers near 1e17 (metres, radians and newtons of multipliers), the scaled
ones 1e4-1e7.  Tolerances: normwise backward error ≤ 1e-15 (SuperLU's is of
the same order), and the scaled solution D⁻¹Δx within 1e-15·κ of a dense
LAPACK solve of the scaled system, relative to its largest entry (κ the
scaled condition number; SuperLU on the unscaled system is itself 1e3-1e4
times further from the dense solve).
This checks the analysis independently of its CUDA kernels, on lattices with
held base nodes (zero-diagonal multipliers, which must come after the dofs
they constrain), chains and unconnected models.
"""
import ctypes
import os
import subprocess

import numpy as np
import pytest
import scipy.sparse as sp
import scipy.sparse.linalg as spla

from muscade_gpu import workloads as W
from oracle import reference as REF

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libsparse_host.so")
SRC = [os.path.join(HERE, "sparse_host.cpp"), os.path.join(ROOT, "muscade.jl_gb300", "csrc", "sparse_analysis.cpp")]


def _lib():
    os.makedirs(BUILD, exist_ok=True)
    deps = SRC + [os.path.join(ROOT, "muscade.jl_gb300", "csrc", "sparse_analysis.hpp")]
    if not os.path.exists(LIB) or any(os.path.getmtime(s) > os.path.getmtime(LIB) for s in deps):
        subprocess.run(["g++", "-O2", "-std=c++17", "-shared", "-fPIC", "-o", LIB + ".tmp"] + SRC, check=True)
        os.replace(LIB + ".tmp", LIB)
    L = ctypes.CDLL(LIB)
    vp = ctypes.c_void_p
    L.sh_analyse.restype = vp
    L.sh_analyse.argtypes = [ctypes.c_int64, vp, vp, vp, vp, ctypes.c_int]
    L.sh_error.restype = ctypes.c_char_p
    L.sh_error.argtypes = [vp]
    L.sh_sizes.argtypes = [vp, vp]
    L.sh_get.argtypes = [vp, vp, vp, vp, vp, vp, vp]
    L.sh_free.argtypes = [vp]
    return L


def analyse(colptr, rowval, xyz, last, leaf=8):
    """colptr/rowval 1-based (as the oracle's pattern)."""
    L = _lib()
    n = len(colptr) - 1
    cp = np.ascontiguousarray(colptr - 1, dtype=np.int64)
    rv = np.ascontiguousarray(rowval - 1, dtype=np.int32)
    xyz = np.ascontiguousarray(xyz, dtype=np.float64)
    last = np.ascontiguousarray(last, dtype=np.uint8)
    h = L.sh_analyse(n, cp.ctypes.data, rv.ctypes.data, xyz.ctypes.data, last.ctypes.data, leaf)
    err = L.sh_error(h).decode()
    assert err == "", err
    s = np.zeros(8, dtype=np.int64)
    L.sh_sizes(h, s.ctypes.data)
    nf, nidx, nem = int(s[0]), int(s[1]), int(s[2])
    perm = np.zeros(n, dtype=np.int32)
    fr = np.zeros((nf, 9), dtype=np.int64)
    fidx = np.zeros(nidx, dtype=np.int32)
    emap = np.zeros(max(nem, 1), dtype=np.int32)
    amap = np.zeros(len(rv), dtype=np.int64)
    flops = ctypes.c_double()
    L.sh_get(h, perm.ctypes.data, fr.ctypes.data, fidx.ctypes.data, emap.ctypes.data, amap.ctypes.data,
             ctypes.byref(flops))
    L.sh_free(h)
    return dict(perm=perm, fronts=fr, fidx=fidx, emap=emap, amap=amap, fsize=int(s[3]), nheight=int(s[4]),
                max_children=int(s[5]), ngroups=int(s[6]), max_m=int(s[7]), flops=flops.value)


def multifrontal_solve(A, nzval, b):
    """Factor and solve with the analysis' fronts (numpy, FP64, no pivoting)."""
    F = np.zeros(A["fsize"])
    F[A["amap"]] = nzval
    fr = A["fronts"]
    nf = len(fr)
    blocks = {}
    children = [[] for _ in range(nf)]
    for f in range(nf):
        if fr[f, 6] >= 0:
            children[fr[f, 6]].append(f)
    for f in range(nf):  # postorder: children first
        off, idx, eoff, m, p = (int(v) for v in fr[f, :5])
        B = F[off:off + m * m].reshape(m, m, order="F").copy()
        for c in sorted(children[f], key=lambda c: fr[c, 8]):
            cm, cp, ce = int(fr[c, 3]), int(fr[c, 4]), int(fr[c, 2])
            e = A["emap"][ce:ce + cm - cp]
            B[np.ix_(e, e)] += blocks[c][cp:, cp:]
        for k in range(p):
            piv = B[k, k]
            assert piv != 0.0, (f, k)
            B[k + 1:, k] /= piv
            B[k + 1:, k + 1:] -= np.outer(B[k + 1:, k], B[k, k + 1:])
        blocks[f] = B
    n = len(b)
    perm = A["perm"]
    y = b[perm].astype(np.float64)  # elimination order
    for f in range(nf):  # forward, L unit lower
        idx, m, p, pos0 = int(fr[f, 1]), int(fr[f, 3]), int(fr[f, 4]), int(fr[f, 5])
        B = blocks[f]
        rows = A["fidx"][idx:idx + m]
        for k in range(p):
            y[rows[k + 1:]] -= B[k + 1:, k] * y[rows[k]]
    x = y.copy()
    for f in reversed(range(nf)):  # backward, U upper
        idx, m, p = int(fr[f, 1]), int(fr[f, 3]), int(fr[f, 4])
        B = blocks[f]
        rows = A["fidx"][idx:idx + m]
        for k in reversed(range(p)):
            x[rows[k]] = (x[rows[k]] - B[k, k + 1:] @ x[rows[k + 1:]]) / B[k, k]
    out = np.zeros(n)
    out[perm] = x
    return out


def equilibration(K, last):
    """D: 1/√|Kᵢᵢ| where the diagonal is not zero; for a multiplier i,
    1 / max_j |K_ji| D_j (the largest scaled entry of its column is 1)."""
    d = np.abs(K.diagonal())
    D = np.zeros(K.shape[0])
    nzd = d > 0
    D[nzd] = 1.0 / np.sqrt(d[nzd])
    Kc = K.tocsc()
    for i in np.nonzero(~nzd)[0]:
        a, b = Kc.indptr[i], Kc.indptr[i + 1]
        D[i] = 1.0 / np.max(np.abs(Kc.data[a:b]) * D[Kc.indices[a:b]])
    return D


def check_solve(A, prep, nz, Ll, last):
    K = prep.matrix(nz)
    D = equilibration(K, last)
    Ks = sp.diags(D) @ K @ sp.diags(D)
    Ks = Ks.tocsc()
    Ks.sort_indices()
    # the scaled values in the pattern's CSC order
    nzs = nz * D[prep.rowval - 1] * np.repeat(D, np.diff(prep.colptr))
    y = multifrontal_solve(A, nzs, D * Ll)
    x = D * y
    be = np.max(np.abs(K @ x - Ll)) / (abs(K).max() * np.max(np.abs(x)) + np.max(np.abs(Ll)))
    assert be <= 1e-15, be
    ref = spla.splu(K.tocsc()).solve(Ll)
    be_ref = np.max(np.abs(K @ ref - Ll)) / (abs(K).max() * np.max(np.abs(ref)) + np.max(np.abs(Ll)))
    assert be <= 1e3 * be_ref, (be, be_ref)
    Kd = Ks.toarray()
    yd = np.linalg.solve(Kd, D * Ll)
    err = np.max(np.abs(y - yd)) / np.max(np.abs(yd))
    assert err <= 1e-15 * np.linalg.cond(Kd), err


def dof_coords_and_multipliers(model, dis):
    nodes = np.asarray(model.dof_node["X"])
    xyz = np.stack([model.coord(int(i)) for i in nodes]).astype(np.float64)
    last = np.array([str(f).startswith("λ") for f in dis.fieldX], dtype=np.uint8)
    return xyz, last


def _system(model, seed=3, amp=0.02):
    st = model.initialize()
    prep = REF.Prepared(model, st.dis)
    rng = np.random.default_rng(seed)
    X = (rng.normal(size=model.ndof["X"]) * amp,)
    Ll, nz = REF.assemble(prep, X, (np.zeros(model.ndof["U"]),), 0.5, "static", REF.newmark_coefficients(0, 1, 0.25, 0.5))
    return st, prep, Ll, nz


@pytest.mark.parametrize("grid,leaf", [((5, 4, 3), 4), ((7, 6, 4), 8), ((6, 6, 6), 1)])
def test_lattice_multifrontal_solve_matches_direct_solve(grid, leaf):
    m, _ = W.lattice(*grid)
    st, prep, Ll, nz = _system(m)
    xyz, last = dof_coords_and_multipliers(m, st.dis)
    A = analyse(prep.colptr, prep.rowval, xyz, last, leaf=leaf)
    assert sorted(A["perm"]) == list(range(len(Ll)))
    # every multiplier comes after the dof it constrains
    ipos = np.empty_like(A["perm"])
    ipos[A["perm"]] = np.arange(len(ipos))
    K = prep.matrix(nz)
    for lam in np.nonzero(last)[0]:
        col = K[:, lam].nonzero()[0]
        assert all(ipos[c] < ipos[lam] for c in col if c != lam)
    check_solve(A, prep, nz, Ll, last)


def test_nested_dissection_of_a_box_uses_plane_separators():
    """On the 12×12×6 lattice the top separator is one grid plane: 12×6 nodes
    of 6 dofs, and the 6 multipliers of each of its 12 held base nodes; the
    fronts hold well under a third of a dense matrix's entries."""
    m, _ = W.lattice(12, 12, 6)
    st, prep, Ll, nz = _system(m)
    xyz, last = dof_coords_and_multipliers(m, st.dis)
    A = analyse(prep.colptr, prep.rowval, xyz, last, leaf=8)
    fr = A["fronts"]
    root = int(np.argmax(fr[:, 5]))  # the last front eliminated
    assert fr[root, 6] == -1 and fr[root, 4] == 12 * 6 * 6 + 12 * 6
    n = len(Ll)
    assert A["fsize"] < n * n / 3


def test_unconnected_models_and_chains():
    params = W.batched_params(3, nel_range=(10, 20), seed=4)
    mb, _, _ = W.build_batched(params)
    st, prep, Ll, nz = _system(mb, amp=0.01)
    xyz, last = dof_coords_and_multipliers(mb, st.dis)
    A = analyse(prep.colptr, prep.rowval, xyz, last, leaf=4)
    roots = np.nonzero(A["fronts"][:, 6] < 0)[0]
    assert len(roots) >= 3  # one tree per model at least
    check_solve(A, prep, nz, Ll, last)


def test_chained_substitution_schedule():
    """The chained substitutions (sparse_lu.cu, sp_fwdb_chain/sp_bwdb_chain)
    give front f's pivot tile t the flag (idx_f >> 6) + 2 f + t: the ranges of
    distinct fronts do not overlap and fit the flag array.  Work items are
    taken in the order t·nf + f (forward) and (np_f − 1 − t)·nf + f
    (backward); every tile an item waits for belongs to an earlier item, so a
    block that takes an item only ever waits for blocks that are running."""
    m, _ = W.lattice(9, 8, 5)
    st, prep, Ll, nz = _system(m)
    xyz, last = dof_coords_and_multipliers(m, st.dis)
    A = analyse(prep.colptr, prep.rowval, xyz, last, leaf=8)
    fr = A["fronts"]
    nf = len(fr)
    ntflag = len(A["fidx"]) // 64 + 2 * nf + 64
    spans = []
    for f in range(nf):
        idx, mf, pf = int(fr[f, 1]), int(fr[f, 3]), int(fr[f, 4])
        npt = (pf + 63) // 64
        base = (idx >> 6) + 2 * f
        spans.append((base, base + npt))
        assert base + npt <= ntflag
    spans.sort()
    assert all(a[1] <= b[0] for a, b in zip(spans, spans[1:]))
    # dependency order within one height's list of fronts (here: all fronts)
    fl = list(range(nf))
    npf = [(int(fr[f, 4]) + 63) // 64 for f in fl]
    ntf = [npf[k] + (int(fr[f, 3]) - int(fr[f, 4]) + 63) // 64 for k, f in enumerate(fl)]
    for k in range(nf):
        for t in range(ntf[k]):
            item = t * nf + k
            assert all(j * nf + k < item for j in range(min(t, npf[k])))
        for tb in range(npf[k]):
            t = npf[k] - 1 - tb
            item = tb * nf + k
            assert all((npf[k] - 1 - b) * nf + k < item for b in range(t + 1, npf[k]))


def _partial_lu(A, p):
    """Right-looking elimination of the first p pivots without row exchanges:
    L below the diagonal, U on and above, the Schur complement in the rest."""
    A = A.copy()
    for k in range(p):
        A[k + 1:, k] /= A[k, k]
        A[k + 1:, k + 1:] -= np.outer(A[k + 1:, k], A[k, k + 1:])
    return A


def _super_panel_lu(A, p, nb=64, sup=256):
    """The FP32 factorisation's block schedule (sparse_lu.cu, factorise): per
    super-panel of `sup` pivots, each `nb`-column block first takes the
    super-panel's earlier blocks (column block rows [k0, m) x [k0, min(k0+nb, p)),
    row block rows [k0, min(k0+nb, p)) x [min(k0+nb, p), m), K [s0, k0)), then its
    diagonal block is factored and its L and U panels solved against it; the
    trailing block [e0, m)^2, e0 = min(s0+sup, p), takes K [s0, e0) at once."""
    A = A.copy()
    m = A.shape[0]
    for s0 in range(0, p, sup):
        e0 = min(s0 + sup, p)
        for k0 in range(s0, e0, nb):
            kb = min(nb, p - k0)
            r1 = k0 + kb
            if k0 > s0:
                A[k0:, k0:r1] -= A[k0:, s0:k0] @ A[s0:k0, k0:r1]
                A[k0:r1, r1:] -= A[k0:r1, s0:k0] @ A[s0:k0, r1:]
            D = _partial_lu(A[k0:r1, k0:r1], kb)
            L = np.tril(D, -1) + np.eye(kb)
            U = np.triu(D)
            A[r1:, k0:r1] = np.linalg.solve(U.T, A[r1:, k0:r1].T).T
            A[k0:r1, r1:] = np.linalg.solve(L, A[k0:r1, r1:])
            A[k0:r1, k0:r1] = D
        A[e0:, e0:] -= A[e0:, s0:e0] @ A[s0:e0, e0:]
    return A


@pytest.mark.parametrize("m,p", [(300, 300), (700, 520), (600, 257), (900, 64), (513, 300), (130, 70), (1000, 1000)])
def test_super_panel_schedule(m, p):
    """The super-panel block schedule gives the partial LU of a front (its
    factors and Schur complement) to rounding, for pivot counts that are and
    are not multiples of the 64-column block and of the 256-pivot super-panel."""
    rng = np.random.default_rng(m + p)
    A = rng.normal(size=(m, m)) + np.eye(m) * m
    ref = _partial_lu(A, p)
    got = _super_panel_lu(A, p)
    assert np.max(np.abs(got - ref)) <= 1e-12 * np.max(np.abs(ref))
