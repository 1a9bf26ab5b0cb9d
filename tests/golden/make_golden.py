"""Regenerate the golden fixtures of tests/test_golden.py from the CPU oracle.

The reference (Fortran + MKL) cannot be built without ifort and MKL and ships no test
outputs, so these fixtures are the oracle's own results on small seeded cases.  They
freeze the oracle (a change to the restatement that moves any of them fails the CPU
tests) and give the GPU tests a reference that needs no oracle build.

    python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from cpfft_gb300 import rve  # noqa: E402
from oracle import pyoracle as po  # noqa: E402

# (name, N, grains, seed, g_mapping)
STRESS_CASE = ("stress_n4", 4, 3, 41, 0)
GREEN_CASES = [("green_n5_ref", 5, 2, 42, 0), ("green_n6_centered", 6, 2, 43, 1)]
LOAD_CASE = ("load_n5", 5, 3, 44, 0)


def random_F(N, amp, seed):
    rng = np.random.default_rng(seed)
    Fn = np.zeros((9, N ** 3))
    Fn[[0, 4, 8]] = 1.0
    return Fn, Fn + amp * rng.standard_normal((9, N ** 3))


def oracle_for(N, grains, seed, gmap):
    r = rve.make_rve(N, grains, seed)
    return r, po.Oracle(N, r.mat_list, r.kocks, r.crystals, 1.0, gmap, nthreads=1)


def stress_fixture():
    name, N, g, seed, gmap = STRESS_CASE
    r, o = oracle_for(N, g, seed, gmap)
    try:
        Fn, Fn1 = random_F(N, 5e-4, seed)
        out = {"Fn": Fn, "Fn1": Fn1, "mat_list": r.mat_list, "kocks": r.kocks}
        for it in (0, 1):
            P, K, fails, _ = o.stress_update(1, it, Fn, Fn1)
            assert fails == 0
            out[f"P_it{it}"], out[f"K4_it{it}"] = P, K
        o.commit()
        out["hist_committed"] = o.history()[0]
        return name, out
    finally:
        o.close()


def green_fixture(case):
    name, N, g, seed, gmap = case
    r, o = oracle_for(N, g, seed, gmap)
    try:
        Fn, Fn1 = random_F(N, 1e-3, seed)
        _, K, _, _ = o.stress_update(1, 0, Fn, Fn1)
        x = np.random.default_rng(seed + 1).standard_normal((9, N ** 3))
        return name, {"Fn": Fn, "Fn1": Fn1, "x": x, "K4": K,
                      "mat_list": r.mat_list, "kocks": r.kocks,
                      "y_K": o.green(x, True, K4=K), "y_I": o.green(x, False, K4=K)}
    finally:
        o.close()


def load_fixture():
    name, N, g, seed, gmap = LOAD_CASE
    r, o = oracle_for(N, g, seed, gmap)
    load = rve.uniaxial_tension(0.03, 20)
    try:
        o.nr3_begin(1e-10)
        pbars, newton = [], []
        for step in (1, 2, 3):
            rc, Pbar, st = o.nr3_step(step, load.BC_all[step - 1], load.isNBC, 1e-6, 1e-10, 20)
            assert rc == 0
            pbars.append(Pbar)
            newton.append(st["newton_iters"])
        f = o.fields()
        return name, {"Pbar": np.array(pbars), "newton": np.array(newton),
                      "Fn1": f["Fn1"], "Pn1": f["Pn1"],
                      "mat_list": r.mat_list, "kocks": r.kocks}
    finally:
        o.close()


def main():
    po.build()
    for name, arrays in [stress_fixture()] + [green_fixture(c) for c in GREEN_CASES] + \
            [load_fixture()]:
        path = os.path.join(HERE, name + ".npz")
        np.savez_compressed(path, **arrays)
        print(path, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    main()
