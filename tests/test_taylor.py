"""Truncated Taylor arithmetic of the beam element (csrc/tj.hpp) on the host:
the node-block products (r₂r₁ᵀ and r_Δ r₁ in the rotation core) and the FMA
forms agree with the general six-variable product to rounding."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "muscade.jl_gb300", "csrc")


def test_block_products_equal_the_general_product(tmp_path):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no host C++ compiler")
    exe = os.path.join(tmp_path, "taylor_check")
    subprocess.run([cxx, "-O1", "-std=c++17", "-I", CSRC, os.path.join(HERE, "taylor_check.cpp"), "-o", exe],
                   check=True, capture_output=True)
    out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout
    for line in out.strip().splitlines():
        vals = line.split()[1:]
        errs = dict(zip(vals[0::2], map(float, vals[1::2])))
        assert len(errs) == 7
        for name, e in errs.items():
            assert e <= 1e-14, (line, name)
