"""Extract the reference's two example decks into test fixtures, with the oracle's results
over every load step of each:

  examples/test_mm01.in  -> tests/golden/mm01_deck.npz: the 7^3 grid, each voxel's
      material (the deck's `elements` ranges), the two `properties bilinear` materials, the
      loading and the solver settings;
  examples/test_mm10.in + angle_bc.in -> tests/golden/mm10_deck.npz: the 7^3 BCC-48
      bicrystal (Kocks angles per element from the orientation file), the loading and the
      solver settings (the crystal block is the package's rve.BCC48_DECK, checked here
      against the deck's keywords).

Runs where the reference tree is mounted; the .npz files are committed so the tests need
no reference files.  Material values are stored as the reference holds them: single
precision (matprp is `real`, src/mod_fft.f:20), widened to double.

    python tests/golden/make_example_decks.py path/to/reference/examples
    (or with the directory in the environment variable CPFFT_REFERENCE_EXAMPLES)
"""
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
EXAMPLES = os.environ.get("CPFFT_REFERENCE_EXAMPLES")
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


def oracle_run(N, mat, kocks, crystals, mises, F_max, nstep, mult, dt, tol_nr, tol_cg, maxit):
    """The oracle over every load step: P_bar, Newton counts, final P."""
    from cpfft_gb300 import rve
    from oracle import pyoracle as po
    load = rve.prescribed_stretch(F_max[[0, 4, 8]] * mult * nstep, nstep)
    o = po.Oracle(N, mat, kocks, crystals, dt, 0, nthreads=os.cpu_count())
    try:
        for k, p in mises.items():
            o.set_mises(k, p)
        o.nr3_begin(tol_cg)
        pb, nw = [], []
        for step in range(1, nstep + 1):
            rc, Pbar, st = o.nr3_step(step, load.BC_all[step - 1], load.isNBC, tol_nr, tol_cg,
                                      maxit)
            assert rc >= 0, (step, rc)
            pb.append(Pbar)
            nw.append(st["newton_iters"])
        return np.array(pb), np.array(nw, np.int32), o.fields()["Pn1"]
    finally:
        o.close()


def deck_common(N, strains, steps, dt, tol, maxit):
    comps = ["F_XX", "F_XY", "F_XZ", "F_YX", "F_YY", "F_YZ", "F_ZX", "F_ZY", "F_ZZ"]
    F_max = np.array([strains.get(c, 0.0) for c in comps])
    assert steps[0] == 1 and not F_max[[1, 2, 3, 5, 6, 7]].any()
    return dict(N=N, F_max=F_max, step_first=steps[0], step_last=steps[1], step_mult=steps[2],
                time_step=dt, tol_nr=tol["nr"], tol_cg=tol["cg"], max_iter=maxit)


def mm01_deck(examples):
    from cpfft_gb300 import rve
    N, materials, order, ranges, strains, steps, dt, tol, maxit = parse(
        open(os.path.join(examples, "test_mm01.in")).read())
    N3 = N ** 3
    mat = np.zeros(N3, np.int32)
    for a, b, name in ranges:
        mat[a - 1:b] = order.index(name) + 1
    assert (mat > 0).all(), "every element needs a material"
    props = np.array([[np.float32(materials[m][k]) for k in KEYS] for m in order], np.float64)
    d = deck_common(N, strains, steps, dt, tol, maxit)
    mises = {k + 1: dict(zip(KEYS, map(float, row))) for k, row in enumerate(props)}
    pb, nw, P = oracle_run(N, mat, np.zeros((3, N3)), [rve.NOT_A_CRYSTAL] * len(order), mises,
                           d["F_max"], steps[1], steps[2], dt, tol["nr"], tol["cg"], maxit)
    np.savez(os.path.join(HERE, "mm01_deck.npz"), mat_list=mat, props=props,
             prop_keys=np.array(KEYS), Pbar_oracle=pb, newton_oracle=nw, Pn1_oracle=P, **d)
    print("mm01 deck: N", N, "materials", order, "voxels per material",
          [int((mat == k + 1).sum()) for k in range(len(order))], "Newton", nw.tolist())


def mm10_deck(examples):
    from cpfft_gb300 import rve
    text = open(os.path.join(examples, "test_mm10.in")).read()
    N, _, _, _, strains, steps, dt, tol, maxit = parse(text)
    # the crystal block against the package's transcription of it
    flat = " ".join(text.replace(",", " ").split()).lower()
    c = rve.BCC48_DECK
    for key, val in (("e", c["e"]), ("nu", c["nu"]), ("tau_y", c["tau_y"]),
                     ("tau_v", c["tau_v"]), ("theta_0", c["theta_0"]),
                     ("voce_m", c["voce_m"]), ("gamma_bar", c["gamma_bar"])):
        m = re.search(r"\b%s ([-+0-9.e]+)" % key, flat)
        assert m and float(m.group(1)) == val, (key, m and m.group(1), val)
    assert "slip_type bcc48" in flat and "alter_mode on" in flat and "hardening voce" in flat
    fname = re.search(r"filename '([^']+)'", text).group(1)
    ang = np.loadtxt(os.path.join(examples, fname), delimiter=",")
    N3 = N ** 3
    assert ang.shape == (N3, 4) and (ang[:, 0] == np.arange(1, N3 + 1)).all()
    kocks = np.ascontiguousarray(ang[:, 1:4].T)
    mat = np.ones(N3, np.int32)
    d = deck_common(N, strains, steps, dt, tol, maxit)
    pb, nw, P = oracle_run(N, mat, kocks, [c], {}, d["F_max"], steps[1], steps[2], dt,
                           tol["nr"], tol["cg"], maxit)
    np.savez(os.path.join(HERE, "mm10_deck.npz"), mat_list=mat, kocks=kocks, Pbar_oracle=pb,
             newton_oracle=nw, Pn1_oracle=P, **d)
    print("mm10 deck: N", N, "orientations", np.unique(kocks.T, axis=0).tolist(), "Newton",
          nw.tolist())


if __name__ == "__main__":
    ex = sys.argv[1] if len(sys.argv) > 1 else EXAMPLES
    if not ex:
        sys.exit("usage: make_example_decks.py <reference examples directory> "
                 "(or set CPFFT_REFERENCE_EXAMPLES)")
    mm01_deck(ex)
    mm10_deck(ex)
