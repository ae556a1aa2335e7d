"""Oracle (test infrastructure only): ctypes bindings to the C++ dual-number
restatement in oracle/csrc, and its build recipe.

Only tests/, __graft_entry__.smoke() and the CPU-baseline leg of bench.py use
this module; the product library never links or calls it.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "liboracle.so")
SRC = [os.path.join(HERE, "csrc", f) for f in ("oracle_api.cpp", "dual.hpp", "rotations.hpp", "beam.hpp", "bar.hpp")]


def build(force: bool = False) -> str:
    """Compile liboracle.so with g++ (OpenMP); skipped when up to date."""
    os.makedirs(BUILD, exist_ok=True)
    if not force and os.path.exists(LIB):
        t = os.path.getmtime(LIB)
        if all(os.path.getmtime(s) <= t for s in SRC):
            return LIB
    cmd = ["g++", "-O3", "-std=c++17", "-fopenmp", "-shared", "-fPIC", "-o", LIB + ".tmp", SRC[0]]
    subprocess.run(cmd, check=True)
    os.replace(LIB + ".tmp", LIB)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        _lib = ctypes.CDLL(build())
        P = ctypes.POINTER(ctypes.c_double)
        i64, i32, d = ctypes.c_int64, ctypes.c_int, ctypes.c_double
        _lib.oracle_beam_construct.argtypes = [i64, P, P, P, P, P]
        _lib.oracle_bar_construct.argtypes = [i64, P, P, P, d, P]
        _lib.oracle_beam_eval.argtypes = [i64, P, i32, P, P, i32, i32, d, d, P, P, P, P, P, i32]
        _lib.oracle_bar_eval.argtypes = [i64, P, i32, P, P, i32, d, i32, d, d, P, P, P, P, P, i32]
        _lib.oracle_sinc1k.argtypes = [i32, d]
        _lib.oracle_sinc1k.restype = d
        _lib.oracle_scac_derivs.argtypes = [d, P]
        _lib.oracle_rodrigues.argtypes = [P, P]
        _lib.oracle_rodrigues_roundtrip.argtypes = [P, P, P]
        _lib.oracle_nj.argtypes = [i32, i32, i32, i32]
        _lib.oracle_beam_results.argtypes = [i64, P, P, P]
        PI = ctypes.POINTER(ctypes.c_int64)
        _lib.oracle_scatter.argtypes = [i64, i32, i32, PI, PI, P, P, i32, P, P]
        _lib.oracle_scatter.restype = None
    return _lib


def _p(a):
    if a is None:
        return None
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _c(a, shape=None):
    if a is None:
        return None
    a = np.ascontiguousarray(a, dtype=np.float64)
    if shape is not None:
        a = a.reshape(shape)
    return a


NTHREADS = int(os.environ.get("ORACLE_THREADS", str(os.cpu_count() or 1)))


def beam_construct(c1, c2, orient2, mat):
    c1, c2, orient2, mat = (_c(np.atleast_2d(a)) for a in (c1, c2, orient2, mat))
    n = c1.shape[0]
    out = np.zeros((n, 69))
    bad = lib().oracle_beam_construct(n, _p(c1), _p(c2), _p(orient2), _p(mat), _p(out))
    if bad:
        raise ValueError("orient2 nearly parallel to the element")
    return out


def bar_construct(c1, c2, mat, epss=np.finfo(np.float64).eps):
    c1, c2, mat = (_c(np.atleast_2d(a)) for a in (c1, c2, mat))
    n = c1.shape[0]
    out = np.zeros((n, 38))
    lib().oracle_bar_construct(n, _p(c1), _p(c2), _p(mat), float(epss), _p(out))
    return out


def _eval(kind, ele, X, U=None, t=0.0, mode=0, a1=0.0, b1=0.0, scaleX=None, a=None, b=None, nthreads=None):
    nx = 12 if kind == "beam" else 6
    ele = _c(ele)
    n = ele.shape[0]
    X = _c(X)
    ND = X.size // (n * nx)
    X = X.reshape(n, ND, nx)
    U = _c(U)
    udof = U is not None
    nU = 3 if udof else 0
    NJ = lib().oracle_nj(nx, ND, nU, mode)
    R = np.zeros((n, nx))
    J = np.zeros((n, nx, NJ))
    scaleX = _c(scaleX)
    a, b = _c(a), _c(b)
    nt = NTHREADS if nthreads is None else nthreads
    if kind == "beam":
        rc = lib().oracle_beam_eval(n, _p(ele), ND, _p(X), _p(U), int(udof), mode, a1, b1, _p(scaleX), _p(a), _p(b),
                                    _p(R), _p(J), nt)
    else:
        rc = lib().oracle_bar_eval(n, _p(ele), ND, _p(X), _p(U), int(udof), float(t), mode, a1, b1, _p(scaleX), _p(a),
                                   _p(b), _p(R), _p(J), nt)
    if rc:
        raise ValueError(f"oracle {kind} eval rejected its arguments (code {rc})")
    return R, J


def beam_eval(ele, X, U=None, **kw):
    """Residual and partials of EulerBeam3D elements (see oracle_api.cpp for modes)."""
    return _eval("beam", ele, X, U, **kw)


def beam_results(ele, X):
    """EulerBeam3D element results (oracle_beam_results): ele (n, 69), X (n, 12) -> (n, 50)."""
    ele = _c(ele)
    X = _c(X)
    n = ele.shape[0]
    out = np.zeros((n, 50))
    lib().oracle_beam_results(n, _p(ele), _p(X), _p(out))
    return out


def bar_eval(ele, X, U=None, t=0.0, **kw):
    return _eval("bar", ele, X, U, t=t, **kw)


def diffed(kind, ele, X, U=None, t=0.0):
    """Like diffed_residual (src/Diagnostic.jl:929-965): R, and ∇R as dict K, C, M, H."""
    nx = 12 if kind == "beam" else 6
    R, J = _eval(kind, ele, X, U, t=t, mode=0)
    n = R.shape[0]
    ND = _c(X).size // (n * nx)
    out = {"R": R}
    for d, name in enumerate(("K", "C", "M")[:ND]):
        out[name] = J[:, :, d * nx:(d + 1) * nx]
    if U is not None:
        out["H"] = J[:, :, ND * nx:ND * nx + 3]
    return out


def scatter(asm1, asm2, R, J, Ll, nzval, minus_col=-1):
    """add_value!/add_∂! of one element type into Ll and nzval (in place),
    serial in element order like the reference.  asm1 (nele, nX), asm2
    (nele, nX*nX) 1-based (0 = skip), R (nele, nX), J (nele, nX, NJ)."""
    nele, nX = R.shape
    if nele == 0:
        return
    NJ = J.shape[2]
    a1 = np.ascontiguousarray(asm1, dtype=np.int64)
    a2 = np.ascontiguousarray(asm2, dtype=np.int64)
    R, J = _c(R), _c(J)
    assert a1.shape == (nele, nX) and a2.shape == (nele, nX * nX) and J.shape[:2] == (nele, nX)
    assert Ll.dtype == np.float64 and nzval.dtype == np.float64 and Ll.flags.c_contiguous and nzval.flags.c_contiguous
    assert a1.size == 0 or (a1.max() <= len(Ll) and a1.min() >= 0)
    assert a2.size == 0 or (a2.max() <= len(nzval) and a2.min() >= 0)
    PI = ctypes.POINTER(ctypes.c_int64)
    lib().oracle_scatter(nele, nX, NJ, a1.ctypes.data_as(PI), a2.ctypes.data_as(PI), _p(R), _p(J), int(minus_col),
                         _p(Ll), _p(nzval))


def sinc1k(k, x):
    return lib().oracle_sinc1k(int(k), float(x))


def scac_derivs(x):
    out = np.zeros(5)
    lib().oracle_scac_derivs(float(x), _p(out))
    return out


def rodrigues(v):
    v = _c(v)
    R = np.zeros(9)
    lib().oracle_rodrigues(_p(v), _p(R))
    return R.reshape(3, 3, order="F")


def rodrigues_roundtrip(v):
    v = _c(v)
    w = np.zeros(3)
    J = np.zeros(9)
    lib().oracle_rodrigues_roundtrip(_p(v), _p(w), _p(J))
    return w, J.reshape(3, 3)
