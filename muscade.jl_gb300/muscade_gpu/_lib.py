"""ctypes binding of the in-tree C-ABI library (include/muscade_gpu.h) and its build.

The library is compiled in-tree (muscade.jl_gb300/_build/libmuscade_gpu.so)
for sm_103a.  Loading fails loudly when it is missing: the package has no CPU
implementation of the device path.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.dirname(HERE)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(BUILD, "libmuscade_gpu.so")
SOURCES = ["mgpu.cu", "solver.cu", "adjoint.cu", "peak.cu", "noalloc.cu", "sparse_lu.cu", "lagrangian.cu",
           "pattern_dev.cu", "pattern.cpp", "sparse_analysis.cpp"]
HEADERS = ["tj.hpp", "beam_math.hpp", "beam_const.hpp", "bar_math.hpp", "ctx.hpp", "pattern.hpp", "band_rows.cuh",
           "band_torn.cuh", "band_bcr.cuh", "solver.hpp", "sparse_lu.hpp", "sparse_analysis.hpp", "tc.cuh"]
ARCH = "-gencode=arch=compute_103a,code=sm_103a"

# status codes
MGPU_OK = 0
ERRORS = {1: "argument", 2: "cuda", 3: "unsupported", 4: "nan", 5: "singular", 6: "noconvergence", 7: "nomem", 8: "size"}
EULERBEAM3D, BAR3D, DOFCONSTRAINT_X, DOFLOAD, DOFCOST, SINGLEUDOF, ACOST = 1, 2, 3, 4, 5, 6, 7
ASM_STATIC, ASM_STEP, ASM_ITER = 0, 1, 2


def sources():
    return [os.path.join(CSRC, s) for s in SOURCES if os.path.exists(os.path.join(CSRC, s))]


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile libmuscade_gpu.so with nvcc for sm_103a (skipped when up to date)."""
    os.makedirs(BUILD, exist_ok=True)
    deps = sources() + [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(PKG, "..", "include", "muscade_gpu.h")]
    if not force and os.path.exists(LIB):
        t = os.path.getmtime(LIB)
        if all(os.path.getmtime(d) <= t for d in deps if os.path.exists(d)):
            return LIB
    objs = []
    procs = []
    for s in sources():
        o = os.path.join(BUILD, os.path.basename(s) + ".o")
        cmd = ["nvcc", "-O3", "-std=c++17", ARCH, "-lineinfo", "-Xcompiler", "-fPIC,-fopenmp", "-c", s, "-o", o]
        procs.append((subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT), cmd))
        objs.append(o)
    for p, cmd in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            raise RuntimeError("nvcc failed: " + " ".join(cmd) + "\n" + out.decode(errors="replace"))
        if verbose and out:
            print(out.decode(errors="replace"))
    cmd = ["nvcc", "-shared", ARCH, "-Xcompiler", "-fopenmp", "-o", LIB + ".tmp"] + objs
    subprocess.run(cmd, check=True)
    os.replace(LIB + ".tmp", LIB)
    return LIB


class Group(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int32), ("nX", ctypes.c_int32), ("nU", ctypes.c_int32), ("ndata", ctypes.c_int32),
                ("nele", ctypes.c_int64), ("indexX", ctypes.POINTER(ctypes.c_int64)),
                ("indexU", ctypes.POINTER(ctypes.c_int64)), ("edata", ctypes.POINTER(ctypes.c_double)),
                ("indexA", ctypes.POINTER(ctypes.c_int64))]


class ModelDesc(ctypes.Structure):
    _fields_ = [("nX", ctypes.c_int64), ("nU", ctypes.c_int64), ("ngroup", ctypes.c_int32),
                ("groups", ctypes.POINTER(Group)), ("scaleX", ctypes.POINTER(ctypes.c_double)),
                ("device", ctypes.c_int32), ("nA", ctypes.c_int64)]


class Newmark(ctypes.Structure):
    _fields_ = [(k, ctypes.c_double) for k in ("a1", "a2", "a3", "b1", "b2", "b3")]


class SweepOpts(ctypes.Structure):
    _fields_ = [("beta", ctypes.c_double), ("gamma", ctypes.c_double), ("maxiter", ctypes.c_int32),
                ("maxdx", ctypes.c_double), ("maxLl", ctypes.c_double), ("fixed_iter", ctypes.c_int32),
                ("per_component", ctypes.c_int32), ("no_graph", ctypes.c_int32), ("device_loop", ctypes.c_int32)]


class Stats(ctypes.Structure):
    _fields_ = [("nstep_done", ctypes.c_int32), ("niter_total", ctypes.c_int32), ("fail_step", ctypes.c_int32),
                ("fail_iter", ctypes.c_int32), ("last_dx", ctypes.c_double), ("last_Ll", ctypes.c_double)]


class LinsolveInfo(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int32), ("ncomp", ctypes.c_int32), ("max_kl", ctypes.c_int32),
                ("max_ku", ctypes.c_int32), ("last_fallback", ctypes.c_int32), ("last_sweeps", ctypes.c_int32)]


class TuneReport(ctypes.Structure):
    _fields_ = [("elem_block", ctypes.c_int32), ("linsolve", ctypes.c_int32), ("ms_elem", ctypes.c_double * 3),
                ("ms_linsolve", ctypes.c_double * 6)]


class SparseReport(ctypes.Structure):
    _fields_ = [("nfront", ctypes.c_int32), ("nheight", ctypes.c_int32), ("nroot", ctypes.c_int32),
                ("max_front", ctypes.c_int32), ("max_pivots", ctypes.c_int32), ("fp64", ctypes.c_int32),
                ("front_entries", ctypes.c_int64), ("flops", ctypes.c_double), ("last_fallback", ctypes.c_int32),
                ("last_sweeps", ctypes.c_int32), ("last_perturbed", ctypes.c_int32),
                ("last_factor_ms", ctypes.c_double), ("last_refine_ms", ctypes.c_double)]


LINSOLVE = {"auto": 0, "f32ir": 1, "f64": 2, "block": 3, "torn": 4, "torn32": 5, "sparse": 6, "sparse64": 7}
LINSOLVE_NAME = {v: k for k, v in LINSOLVE.items()}

# every symbol the header declares (checked by the CPU test suite)
SYMBOLS = ["mgpu_create", "mgpu_destroy", "mgpu_last_error", "mgpu_nnz", "mgpu_get_pattern", "mgpu_get_asm",
           "mgpu_ntval", "mgpu_assemble", "mgpu_element_eval", "mgpu_upload_state", "mgpu_assemble_resident",
           "mgpu_download", "mgpu_time_assemble", "mgpu_sweepx", "mgpu_measure_fp64_peak",
           "mgpu_assemble_beams_noalloc", "mgpu_set_linear_solver", "mgpu_linear_solver_info", "mgpu_set_A",
           "mgpu_adjoint_sweepx", "mgpu_host_register", "mgpu_host_unregister", "mgpu_autotune",
           "mgpu_assemble_async", "mgpu_assemble_wait", "mgpu_sparse_info", "mgpu_element_lagrangian",
           "mgpu_tc_gemm_check", "mgpu_launch_count", "mgpu_sensitivity_sweepx", "mgpu_beam_results"]

_lib = None


def load():
    """Load the library (build it first if needed and nvcc is present)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB):
        raise RuntimeError(f"muscade_gpu: CUDA library not built ({LIB}); run __graft_entry__.build()")
    L = ctypes.CDLL(LIB)
    P = ctypes.POINTER
    d, i32, i64, vp = ctypes.c_double, ctypes.c_int32, ctypes.c_int64, ctypes.c_void_p
    pd = P(ctypes.c_double)
    pi64 = P(ctypes.c_int64)
    L.mgpu_create.argtypes = [P(vp), P(ModelDesc)]
    L.mgpu_destroy.argtypes = [vp]
    L.mgpu_destroy.restype = None
    L.mgpu_last_error.argtypes = [vp]
    L.mgpu_last_error.restype = ctypes.c_char_p
    L.mgpu_nnz.argtypes = [vp]
    L.mgpu_nnz.restype = i64
    L.mgpu_ntval.argtypes = [vp]
    L.mgpu_ntval.restype = i64
    L.mgpu_launch_count.argtypes = [vp]
    L.mgpu_launch_count.restype = i64
    L.mgpu_get_pattern.argtypes = [vp, pi64, pi64]
    L.mgpu_get_asm.argtypes = [vp, i32, pi64, pi64]
    L.mgpu_assemble.argtypes = [vp, i32, i32, pd, pd, d, pd, P(Newmark), pd, pd]
    L.mgpu_assemble_async.argtypes = [vp, i32, i32, pd, pd, d, pd, P(Newmark), pd, pd, pi64]
    L.mgpu_assemble_wait.argtypes = [vp, i64]
    L.mgpu_element_eval.argtypes = [vp, i32, i32, pd, pd, d, d, d, d, pd, pd, pd]
    L.mgpu_upload_state.argtypes = [vp, i32, pd, pd, pd]
    L.mgpu_assemble_resident.argtypes = [vp, i32, d, P(Newmark)]
    L.mgpu_download.argtypes = [vp, pd, pd]
    L.mgpu_time_assemble.argtypes = [vp, i32, d, P(Newmark), i32, i32, pd, pd, pd]
    L.mgpu_sweepx.argtypes = [vp, i32, i64, pd, d, i32, pd, pd, pd, P(SweepOpts), pd, P(Stats)]
    L.mgpu_measure_fp64_peak.argtypes = [i32, pd]
    L.mgpu_assemble_beams_noalloc.argtypes = [i64, i64, i64, vp, vp, vp, vp, vp, vp, vp, vp]
    L.mgpu_set_linear_solver.argtypes = [vp, i32]
    L.mgpu_linear_solver_info.argtypes = [vp, P(LinsolveInfo)]
    L.mgpu_sparse_info.argtypes = [vp, P(SparseReport)]
    L.mgpu_set_A.argtypes = [vp, pd]
    L.mgpu_host_register.argtypes = [vp, i64]
    L.mgpu_autotune.argtypes = [vp, i32, P(Newmark), P(TuneReport)]
    L.mgpu_host_unregister.argtypes = [vp]
    L.mgpu_adjoint_sweepx.argtypes = [vp, i32, i64, pd, d, i32, pd, pd, pd, P(SweepOpts), i64, pi64, pd, pd, i32, pd,
                                      pd, pd, pd, P(Stats)]
    L.mgpu_element_lagrangian.argtypes = [vp, i32, i32, pd, pd, pd, pd, pd, pd, pd, pd]
    L.mgpu_beam_results.argtypes = [vp, i32, i64, pd, pd]
    L.mgpu_sensitivity_sweepx.argtypes = [vp, i32, i64, pd, d, i32, pd, pd, pd, P(SweepOpts), i64, pi64, pd, pd, i32,
                                          pi64, pd, pd, P(Stats)]
    pf = P(ctypes.c_float)
    L.mgpu_tc_gemm_check.argtypes = [i32, i32, i32, i32, pf, pf, pf]
    for name in SYMBOLS:
        f = getattr(L, name)
        if f.restype is ctypes.c_int and name not in ("mgpu_destroy",):
            f.restype = ctypes.c_int
    _lib = L
    return L


def ptr(a, ctype=ctypes.c_double):
    if a is None:
        return None
    return a.ctypes.data_as(ctypes.POINTER(ctype))
