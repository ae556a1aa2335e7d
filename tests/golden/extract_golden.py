"""Extract the numeric golden values of the reference's own test suite.

Reads the reference's test files as text (they are Julia; nothing is
executed) and writes `reference_golden.json` next to this script.  Each entry
records the test file and line it was read from.  Run from the repository
root with the reference checkout at REFERENCE (default /root/reference):

    python tests/golden/extract_golden.py [REFERENCE]

The committed JSON is what the tests use; the reference tree is not needed at
test time.
"""
import json
import os
import re
import sys

REF = sys.argv[1] if len(sys.argv) > 1 else "/root/reference"
OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference_golden.json")


def line(path, lineno):
    with open(os.path.join(REF, path), encoding="utf-8") as f:
        return f.readlines()[lineno - 1]


def rhs(text):
    """Text right of the first '≈' (or '==') up to an optional atol/rtol."""
    if "≈" in text:
        t = text.split("≈", 1)[1]
    else:
        t = text.split("==", 1)[1]
    t = re.split(r"\batol\b|\brtol\b", t)[0]
    return t.strip().rstrip(",").strip()


def parse_vector(t):
    """Julia vector literal like [1.0, -2, 3e-5] -> list of floats."""
    t = t.strip()
    m = re.match(r"^\[(.*)\]", t, re.S)
    body = m.group(1)
    return [float(x) for x in re.split(r"[,\s]+", body.strip()) if x]


def parse_matrix(t):
    """Julia matrix literal [a b c; d e f] -> row-major list of rows."""
    m = re.match(r"^\[(.*)\]", t.strip(), re.S)
    rows = [r for r in m.group(1).split(";")]
    return [[float(x) for x in r.split()] for r in rows if r.strip()]


def vec_at(path, lineno):
    return {"src": f"{path}:{lineno}", "value": parse_vector(rhs(line(path, lineno)))}


def mat_at(path, lineno):
    return {"src": f"{path}:{lineno}", "value": parse_matrix(rhs(line(path, lineno)))}


def scaled_vec_at(path, lineno, scale):
    """Vector literal followed by an arithmetic suffix on L (e.g. `*L`, `/L^2`)."""
    t = rhs(line(path, lineno))
    m = re.match(r"^(\[.*?\])\s*(.*)$", t)
    vec = parse_vector(m.group(1))
    return {"src": f"{path}:{lineno}", "value": vec, "suffix": m.group(2).strip(), "L": scale}


def sparse_at(path, lineno):
    """sparse(I, J, V, m, n) literal -> dict."""
    t = rhs(line(path, lineno))
    m = re.match(r"^sparse\((\[.*?\]),\s*(\[.*?\]),\s*(\[.*?\]),\s*(\d+),\s*(\d+)\)", t)
    return {
        "src": f"{path}:{lineno}",
        "I": [int(v) for v in parse_vector(m.group(1))],
        "J": [int(v) for v in parse_vector(m.group(2))],
        "V": parse_vector(m.group(3)),
        "m": int(m.group(4)),
        "n": int(m.group(5)),
    }


def intcol_at(path, lineno):
    """Column literal like [1; 2; 4; 5;;] -> ints."""
    t = rhs(line(path, lineno))
    body = re.match(r"^\[(.*?)\]", t).group(1).replace(";;", "")
    return {"src": f"{path}:{lineno}", "value": [int(x) for x in re.split(r"[;\s]+", body) if x]}


g = {}
# ---- rotations  test/TestRotations.jl
R = "test/TestRotations.jl"
g["sinc1_theta"] = {"src": f"{R}:6", "value": [0.0, 1e-8, 1e-6, 1e-2, 0.1, 1.0, 3.141592653589793]}
for k, ln in zip(range(5), range(8, 13)):
    g[f"sinc1_d{k}"] = vec_at(R, ln)
g["scac_x"] = {"src": f"{R}:57", "value": [-1 + 1e-11, -1 + 1e-9, 0.0, 1 - 1e-9, 1 - 1e-11, 1.0]}
for k, ln in zip(range(5), range(59, 64)):
    g[f"scac_d{k}"] = vec_at(R, ln)
g["adjust_r"] = vec_at(R, 103)
g["adjust_u"] = vec_at(R, 104)

# ---- beam constructor  test/TestBeamElement.jl:15-31 (node2 at (4,3,0), L=5)
B = "test/TestBeamElement.jl"
g["beam_cm"] = vec_at(B, 16)
g["beam_rm"] = mat_at(B, 17)
g["beam_zgp"] = vec_at(B, 18)
g["beam_znod"] = vec_at(B, 19)
g["beam_tgm"] = vec_at(B, 20)
g["beam_tge"] = vec_at(B, 21)
g["beam_ya"] = vec_at(B, 23)
g["beam_yu"] = vec_at(B, 24)
g["beam_yv"] = scaled_vec_at(B, 25, 5.0)
g["beam_ka"] = scaled_vec_at(B, 26, 5.0)
g["beam_ku"] = scaled_vec_at(B, 27, 5.0)
g["beam_kv"] = scaled_vec_at(B, 28, 5.0)
g["beam_dL"] = scaled_vec_at(B, 30, 5.0)

# ---- bar constructor  test/TestBarElement.jl:17-26
BA = "test/TestBarElement.jl"
g["bar_wgp"] = vec_at(BA, 21)
g["bar_zgp"] = vec_at(BA, 22)
g["bar_psi1"] = vec_at(BA, 24)
g["bar_psi2"] = vec_at(BA, 25)

# ---- constraints  test/TestDofConstraints.jl:27-46
C = "test/TestDofConstraints.jl"
g["dofcon_equal_contact_R"] = vec_at(C, 32)
g["dofcon_equal_gap_R"] = vec_at(C, 42)

# ---- assembly  test/TestAssemble.jl
A = "test/TestAssemble.jl"
g["turbine_R"] = vec_at(A, 19)
g["turbine_La"] = mat_at(A, 22)
g["anchor_L_lambda"] = vec_at(A, 37)
g["anchor_L_x"] = vec_at(A, 38)
g["anchor_L_a"] = vec_at(A, 40)
g["asm_1_1"] = intcol_at(A, 123)
g["asm_1_2"] = intcol_at(A, 124)
g["asm_2_1"] = intcol_at(A, 125)
g["asm_2_2"] = intcol_at(A, 126)
g["prepare_Llx"] = sparse_at(A, 122)
g["assemble_Ll"] = vec_at(A, 156)
g["assemble_Llx"] = sparse_at(A, 157)

# ---- solvers
S0 = "test/TestSweepX0.jl"
g["sweepx0_X"] = vec_at(S0, 24)
S2 = "test/TestSweepX2.jl"
g["sweepx2_X"] = vec_at(S2, 21)
g["sweepx2_X1"] = vec_at(S2, 22)
g["sweepx2_X2"] = vec_at(S2, 23)

# ---- 45° cantilever bend (examples/StaticBeamAnalysis.jl): the tip coordinates
# of two published solutions that the example quotes in comments, at 300, 450
# and 600 N (x, y, z each)
E = "examples/StaticBeamAnalysis.jl"


def literature_row(path, lineno):
    t = line(path, lineno).split("##", 1)[1]
    nums = [float(x) for x in re.findall(r"-?\d+\.\d+", t)]
    return {"src": f"{path}:{lineno}", "value": [nums[0:3], nums[3:6], nums[6:9]]}


g["bend_tip_longva"] = literature_row(E, 133)
g["bend_tip_crisfield"] = literature_row(E, 134)

with open(OUT, "w") as f:
    json.dump(g, f, indent=1)
print(f"wrote {len(g)} golden entries to {OUT}")
