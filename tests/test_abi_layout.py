"""The ctypes mirror of the C ABI (muscade_gpu/_lib.py) against the header as
a C compiler lays it out: every struct's size and field offsets, and the
values of the status, element-kind, mission and solver-kind constants."""
import ctypes
import os
import shutil
import subprocess

import pytest

from muscade_gpu import _lib as L

HERE = os.path.dirname(os.path.abspath(__file__))
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

STRUCTS = {"mgpu_group": L.Group, "mgpu_model_desc": L.ModelDesc, "mgpu_newmark": L.Newmark,
           "mgpu_sweep_opts": L.SweepOpts, "mgpu_stats": L.Stats, "mgpu_linsolve_info": L.LinsolveInfo,
           "mgpu_tune_report": L.TuneReport, "mgpu_sparse_report": L.SparseReport}


@pytest.fixture(scope="module")
def layout(tmp_path_factory):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no host C compiler")
    exe = str(tmp_path_factory.mktemp("abi") / "abi_layout")
    subprocess.run([cc, "-std=c11", "-I", INCLUDE, os.path.join(HERE, "abi_layout.c"), "-o", exe], check=True,
                   capture_output=True)
    out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout.split("\n")
    sizes, offsets, consts = {}, {}, {}
    for line in out:
        p = line.split()
        if not p:
            continue
        if p[0] == "S":
            sizes[p[1]] = int(p[2])
        elif p[0] == "F":
            offsets[(p[1], p[2])] = int(p[3])
        else:
            consts[p[1]] = int(p[2])
    return sizes, offsets, consts


def test_struct_layouts_match(layout):
    sizes, offsets, _ = layout
    for name, cls in STRUCTS.items():
        assert ctypes.sizeof(cls) == sizes[name], name
        fields = [f[0] for f in cls._fields_]
        assert sorted(fields) == sorted(f for (s, f) in offsets if s == name), name
        for f in fields:
            assert getattr(cls, f).offset == offsets[(name, f)], (name, f)


def test_constants_match(layout):
    _, _, c = layout
    assert c["MGPU_OK"] == L.MGPU_OK
    for code, kind in L.ERRORS.items():
        name = {"argument": "ARG", "noconvergence": "NOCONV"}.get(kind, kind.upper())
        assert c["MGPU_ERR_" + name] == code
    assert (c["MGPU_EULERBEAM3D"], c["MGPU_BAR3D"], c["MGPU_DOFCONSTRAINT_X"], c["MGPU_DOFLOAD"]) == \
        (L.EULERBEAM3D, L.BAR3D, L.DOFCONSTRAINT_X, L.DOFLOAD)
    assert (c["MGPU_DOFCOST"], c["MGPU_SINGLEUDOF"], c["MGPU_ACOST"]) == (L.DOFCOST, L.SINGLEUDOF, L.ACOST)
    assert (c["MGPU_ASM_STATIC"], c["MGPU_ASM_STEP"], c["MGPU_ASM_ITER"]) == (L.ASM_STATIC, L.ASM_STEP, L.ASM_ITER)
    for kind, v in L.LINSOLVE.items():
        assert c["MGPU_LINSOLVE_" + kind.upper()] == v
