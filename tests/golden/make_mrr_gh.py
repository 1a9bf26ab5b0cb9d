"""Golden interaction matrices of the Ma-Roters-Raabe hardening law for FCC crystals.

Reads the reference's own table, mm10_mrr_GHfcc (src/mm10_e.f), from a checkout of the
reference and writes tests/golden/mrr_gh_fcc.npz (G and H, 12 x 12, G(alpha, beta) the
reference's G(alpha, beta)).  Run from the repository root:

    python tests/golden/make_mrr_gh.py <reference checkout>

The oracle and the library form these matrices from the slip geometry; the fixture pins
them to the reference's numbers.
"""
import os
import re
import sys

import numpy as np


def parse(path):
    src = open(path).read()
    i0 = src.index("subroutine mm10_mrr_GHfcc(")
    body = src[i0:src.index("end subroutine", i0)]
    consts = {"zero": 0.0}
    for m in re.finditer(r"^\s+([GH]\d)\s*=\s*([+\-\d.D]+)", body, re.M):
        consts[m.group(1)] = float(m.group(2).replace("D", "e"))
    G = np.full((12, 12), np.nan)
    H = np.full((12, 12), np.nan)
    for m in re.finditer(r"^\s+([GH])\((\d+),(\d+)\)\s*=\s*(\w+)", body, re.M):
        (G if m.group(1) == "G" else H)[int(m.group(2)) - 1, int(m.group(3)) - 1] = consts[m.group(4)]
    assert not np.isnan(G).any() and not np.isnan(H).any()
    return G, H


if __name__ == "__main__":
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ["CPFFT_REFERENCE"]
    G, H = parse(os.path.join(ref, "src", "mm10_e.f"))
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "mrr_gh_fcc.npz")
    np.savez(out, G=G, H=H)
    print("wrote", out)
