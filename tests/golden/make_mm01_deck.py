"""Extract the reference's bilinear Mises example deck (examples/test_mm01.in) into
tests/golden/mm01_deck.npz: the grid, each voxel's material number (the deck's
`elements` ranges), the two materials' `properties bilinear` values, the loading and the
solver settings.  Runs where the reference tree is mounted; the .npz is committed so the
tests need no reference files.

    python tests/golden/make_mm01_deck.py [path/to/test_mm01.in]

Material values are stored as the reference holds them: single precision (matprp is
`real`, src/mod_fft.f:20), widened to double.
"""
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
DECK = "/root/reference/examples/test_mm01.in"
KEYS = ("e", "nu", "yld_pt", "tan_e", "beta")


def parse(text):
    lines = []
    for raw in text.splitlines():  # join continuation lines (trailing comma)
        s = raw.strip()
        if not s or s.lower().startswith("c ") or s.lower() == "c":
            continue
        if lines and lines[-1].endswith(","):
            lines[-1] = lines[-1] + " " + s
        else:
            lines.append(s)
    N = None
    materials, order = {}, []
    ranges = []
    strains = {}
    steps = None
    time_step = None
    tol = {}
    maxit = None
    mode = None
    for s in lines:
        low = s.lower()
        if low.startswith("number of grid"):
            N = int(low.split()[-1])
        elif low.startswith("material "):
            mode = ("material", s.split()[1])
            order.append(s.split()[1])
        elif mode and mode[0] == "material" and low.startswith("properties bilinear"):
            toks = s.replace(",", " ").split()[2:]
            vals = dict(e=30000.0, nu=0.3, yld_pt=0.0, tan_e=0.0, beta=1.0)  # mat_default
            for k in range(0, len(toks) - 1, 2):
                if toks[k] in vals:
                    vals[toks[k]] = float(toks[k + 1])
            materials[mode[1]] = vals
            mode = None
        elif low == "elements":
            mode = ("elements",)
        elif mode and mode[0] == "elements" and " material " in low:
            rng, _, name = s.split()
            a, _, b = rng.partition("-")
            ranges.append((int(a), int(b or a), name))
        elif low == "strains":
            mode = ("strains",)
        elif mode and mode[0] == "strains" and re.match(r"^[fp]_[xyz]{2}\s", low):
            k, v = s.split()
            strains[k.upper()] = float(v)
        elif low.startswith("step ") and "constraints" in low:
            span, _, mult = low.split()[1:4]
            a, _, b = span.partition("-")
            steps = (int(a), int(b or a), float(mult))
        elif low.startswith("time step"):
            time_step = float(low.split()[-1])
        elif low.startswith("convergence tolerance"):
            toks = low.split()
            tol = {toks[i]: float(toks[i + 1]) for i in (2, 4)}
        elif low.startswith("maximum iterations"):
            maxit = int(low.split()[-1])
        else:
            if mode and mode[0] != "material":
                mode = None
    return N, materials, order, ranges, strains, steps, time_step, tol, maxit


def main(path=DECK):
    N, materials, order, ranges, strains, steps, dt, tol, maxit = parse(open(path).read())
    N3 = N ** 3
    mat = np.zeros(N3, np.int32)
    for a, b, name in ranges:
        mat[a - 1:b] = order.index(name) + 1
    assert (mat > 0).all(), "every element needs a material"
    props = np.array([[np.float32(materials[m][k]) for k in KEYS] for m in order], np.float64)
    comps = ["F_XX", "F_XY", "F_XZ", "F_YX", "F_YY", "F_YZ", "F_ZX", "F_ZY", "F_ZZ"]
    F_max = np.array([strains.get(c, 0.0) for c in comps])
    np.savez(os.path.join(HERE, "mm01_deck.npz"), N=N, mat_list=mat, props=props,
             prop_keys=np.array(KEYS), F_max=F_max, step_first=steps[0], step_last=steps[1],
             step_mult=steps[2], time_step=dt, tol_nr=tol["nr"], tol_cg=tol["cg"],
             max_iter=maxit)
    print("N", N, "materials", order, "voxels per material",
          [int((mat == k + 1).sum()) for k in range(len(order))])


if __name__ == "__main__":
    main(*sys.argv[1:])
