"""Golden slip tables of the crystal slip types and interaction matrices of the 12-system
ones.

Reads, from a checkout of the reference, the slip directions and plane normals that
finalize_new_crystal assigns for slip_type 1 (fcc), 2 (bcc), 3 (single), 6 (roters),
7 (bcc12), 8 (bcc48), 9 (hcp6) and 10 (hcp18) (src/mod_crystals.f), and the
Ma-Roters-Raabe interaction tables of the 12-system types (mm10_mrr_GHfcc / GHbcc / GHfcc12 / GHbcc12, src/mm10_e.f).  Writes
tests/golden/slip_tables.npz: b<type>, n<type> (systems x 3) and G<type>, H<type> (12 x 12,
G(alpha, beta) the reference's G(alpha, beta)).  Run from the repository root:

    python tests/golden/make_slip_tables.py <reference checkout>

The library and the oracle write these tables in their own code; the fixture pins both to
the reference's numbers.
"""
import ast
import os
import re
import sys

import numpy as np


def _literal(text):
    """Fortran double literals (0.5d0, 1.d0, 3.0D-1) as Python floats."""
    return re.sub(r"(\d+\.\d*|\.\d+|\d+)[dD]([+-]?\d+)", r"\1e\2", text)


def fortran_value(expr, env):
    """Evaluate a table entry or constant definition of the reference: numbers, named
    constants, + - * / ** and sqrt.  The text is parsed, never executed."""
    ops = {ast.Add: lambda x, y: x + y, ast.Sub: lambda x, y: x - y,
           ast.Mult: lambda x, y: x * y, ast.Div: lambda x, y: x / y,
           ast.Pow: lambda x, y: x ** y}

    def ev(node):
        if isinstance(node, ast.Expression):
            return ev(node.body)
        if isinstance(node, ast.Constant) and isinstance(node.value, (int, float)):
            return float(node.value)
        if isinstance(node, ast.Name):
            return env[node.id.lower()]
        if isinstance(node, ast.UnaryOp) and isinstance(node.op, (ast.USub, ast.UAdd)):
            v = ev(node.operand)
            return -v if isinstance(node.op, ast.USub) else v
        if isinstance(node, ast.BinOp) and type(node.op) in ops:
            return ops[type(node.op)](ev(node.left), ev(node.right))
        if isinstance(node, ast.Call) and isinstance(node.func, ast.Name) and \
                node.func.id.lower() in ("sqrt", "dsqrt") and len(node.args) == 1:
            return float(np.sqrt(ev(node.args[0])))
        raise ValueError("unsupported expression: %s" % expr)

    return ev(ast.parse(_literal(expr.strip()), mode="eval"))


def slip_table(lines, slip_type):
    """Directions and normals assigned in the `slip_type .eq. <t>` branch, as many rows as
    its nslip; rows the branch does not assign stay zero, as the reference's crystal
    record does."""
    start = next(i for i, ln in enumerate(lines)
                 if re.search(r"slip_type\s*\.eq\.\s*%d\s*\)" % slip_type, ln))
    env, b, n, ns = {}, {}, {}, None
    for ln in lines[start + 1:]:
        if ln[:1] in "cC*!":             # fixed-form comment line
            continue
        s = ln.split("!")[0].strip()
        if not s:
            continue
        if re.match(r"(else\s*if|elseif|else$|endif|end\s+if)", s.lower()):
            break
        m = re.fullmatch(r"c_array\(num\)%(bi|ni)\(\s*(\d+)\s*,\s*(\d)\s*\)\s*=\s*(.+)", s)
        if m:
            (b if m.group(1) == "bi" else n)[(int(m.group(2)), int(m.group(3)))] = \
                fortran_value(m.group(4), env)
            continue
        m = re.fullmatch(r"c_array\(num\)%nslip\s*=\s*(.+)", s)
        if m:
            ns = int(fortran_value(m.group(1), env))
            continue
        m = re.fullmatch(r"(\w+)\s*=\s*(.+)", s)
        if m:
            env[m.group(1).lower()] = fortran_value(m.group(2), env)
    B = np.array([[b.get((i, j), 0.0) for j in (1, 2, 3)] for i in range(1, ns + 1)])
    N = np.array([[n.get((i, j), 0.0) for j in (1, 2, 3)] for i in range(1, ns + 1)])
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
    for t in (1, 2, 3, 6, 7, 8, 9, 10):
        B, N = slip_table(lines, t)
        live = np.linalg.norm(B, axis=1) > 0      # hcp18: six assigned systems of 18
        assert np.allclose(np.linalg.norm(B[live], axis=1), 1)
        assert np.allclose(np.linalg.norm(N[live], axis=1), 1)
        assert np.abs((B * N).sum(axis=1)).max() < 1e-15, t
        out["b%d" % t], out["n%d" % t] = B, N
    for t, routine in ((1, "mm10_mrr_GHfcc"), (2, "mm10_mrr_GHbcc"), (6, "mm10_mrr_GHfcc12"),
                       (7, "mm10_mrr_GHbcc12")):
        out["G%d" % t], out["H%d" % t] = interaction(esrc, routine)
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "slip_tables.npz")
    np.savez(path, **out)
    print("wrote", path, {k: v.shape for k, v in out.items()})
