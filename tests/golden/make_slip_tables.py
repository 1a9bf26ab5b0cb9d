"""Golden slip tables and interaction matrices of the cubic slip types.

Reads, from a checkout of the reference, the slip directions and plane normals that
finalize_new_crystal assigns for slip_type 1 (fcc), 2 (bcc), 6 (roters), 7 (bcc12) and
8 (bcc48) (src/mod_crystals.f), and the Ma-Roters-Raabe interaction tables of the
12-system types (mm10_mrr_GHfcc / GHbcc / GHfcc12 / GHbcc12, src/mm10_e.f).  Writes
tests/golden/slip_tables.npz: b<type>, n<type> (systems x 3) and G<type>, H<type> (12 x 12,
G(alpha, beta) the reference's G(alpha, beta)).  Run from the repository root:

    python tests/golden/make_slip_tables.py <reference checkout>

The library and the oracle write these tables in their own code; the fixture pins both to
the reference's numbers.
"""
import os
import re
import sys

import numpy as np

# the Fortran names of the constants the tables are written with
CONSTS = {"f": None, "f2": None, "f3": None, "f112": None, "f211": None, "f123": None,
          "f213": None, "f312": None, "z0": None}


def fortran_value(expr, env):
    """A table entry or constant definition: a literal, a named constant, 1/sqrt(k),
    k/sqrt(m) or a sign in front of one of these."""
    e = expr.strip().lower().replace("d0", "").replace("dsqrt", "sqrt")
    sign = 1.0
    if e.startswith("-"):
        sign, e = -1.0, e[1:].strip()
    elif e.startswith("+"):
        e = e[1:].strip()
    m = re.fullmatch(r"([\d.]+)\s*/\s*sqrt\(\s*([\d.]+)\s*\)", e)
    if m:
        return sign * float(m.group(1)) / np.sqrt(float(m.group(2)))
    if e in env:
        return sign * env[e]
    return sign * float(e)


def slip_table(lines, slip_type):
    """Directions and normals assigned in the `slip_type .eq. <t>` branch."""
    start = next(i for i, ln in enumerate(lines)
                 if re.search(r"slip_type\s*\.eq\.\s*%d\s*\)" % slip_type, ln))
    env, b, n = {}, {}, {}
    for ln in lines[start + 1:]:
        s = ln.split("!")[0].strip()
        if re.match(r"(else)?if\s*\(", s.lower()) or s.lower().startswith("elseif") or \
                s.lower().startswith("endif") or s.lower().startswith("end if"):
            break
        if not s or ln[:1].lower() == "c":
            continue
        m = re.fullmatch(r"c_array\(num\)%(bi|ni)\(\s*(\d+)\s*,\s*(\d)\s*\)\s*=\s*(.+)", s)
        if m:
            (b if m.group(1) == "bi" else n)[(int(m.group(2)), int(m.group(3)))] = \
                fortran_value(m.group(4), env)
            continue
        m = re.fullmatch(r"(\w+)\s*=\s*(.+)", s)
        if m and m.group(1).lower() in CONSTS:
            env[m.group(1).lower()] = fortran_value(m.group(2), env)
    ns = max(k[0] for k in b)
    B = np.array([[b[(i, j)] for j in (1, 2, 3)] for i in range(1, ns + 1)])
    N = np.array([[n[(i, j)] for j in (1, 2, 3)] for i in range(1, ns + 1)])
    return B, N


def interaction(src, routine):
    i0 = src.index("subroutine %s(" % routine)
    body = src[i0:src.index("end subroutine", i0)]
    consts = {"zero": 0.0}
    for m in re.finditer(r"^\s+([GH]\d)\s*=\s*([+\-\d.D]+)", body, re.M):
        consts[m.group(1)] = float(m.group(2).replace("D", "e"))
    G = np.full((12, 12), np.nan)
    H = np.full((12, 12), np.nan)
    for m in re.finditer(r"^\s+([GH])\((\d+),(\d+)\)\s*=\s*(\w+)", body, re.M):
        (G if m.group(1) == "G" else H)[int(m.group(2)) - 1, int(m.group(3)) - 1] = \
            consts[m.group(4)]
    assert not np.isnan(G).any() and not np.isnan(H).any(), routine
    return G, H


if __name__ == "__main__":
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ["CPFFT_REFERENCE"]
    lines = open(os.path.join(ref, "src", "mod_crystals.f")).read().split("\n")
    esrc = open(os.path.join(ref, "src", "mm10_e.f")).read()
    out = {}
    for t in (1, 2, 6, 7, 8):
        B, N = slip_table(lines, t)
        assert np.allclose(np.linalg.norm(B, axis=1), 1) and np.allclose(np.linalg.norm(N, axis=1), 1)
        assert np.abs((B * N).sum(axis=1)).max() < 1e-15, t
        out["b%d" % t], out["n%d" % t] = B, N
    for t, routine in ((1, "mm10_mrr_GHfcc"), (2, "mm10_mrr_GHbcc"), (6, "mm10_mrr_GHfcc12"),
                       (7, "mm10_mrr_GHbcc12")):
        out["G%d" % t], out["H%d" % t] = interaction(esrc, routine)
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "slip_tables.npz")
    np.savez(path, **out)
    print("wrote", path, {k: v.shape for k, v in out.items()})
