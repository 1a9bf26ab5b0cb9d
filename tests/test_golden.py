"""Golden fixtures (tests/golden/*.npz, written by tests/golden/make_golden.py from the
CPU oracle on small seeded cases).

CPU tests: the oracle still reproduces its frozen outputs.  GPU tests: the C-ABI library
matches them with the parity tolerances (1e-8 per voxel for the stress update and the
load step's fields, 1e-11 for the Green operator, 1e-10 for P_bar), reading nothing but
the fixtures."""
import os

import numpy as np
import pytest

from cpfft_gb300 import rve

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def fixture(name):
    return np.load(os.path.join(GOLD, name + ".npz"))


def rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def per_voxel_rel(a, b):
    scale = np.maximum(np.abs(b).max(axis=0), 1e-6 * np.abs(b).max())
    return (np.abs(a - b).max(axis=0) / scale).max()


def crystals():
    return [dict(rve.FCC_VOCE)]


def n_of(d):
    return round(d["mat_list"].size ** (1.0 / 3.0))


def make_oracle(oracle, d, gmap):
    return oracle.Oracle(n_of(d), d["mat_list"], d["kocks"], crystals(), 1.0, gmap, nthreads=1)


def make_solver(gpulib, d, gmap):
    return gpulib.Solver(n_of(d), d["mat_list"], d["kocks"], crystals(), 1.0, gmap, 0)


# ---------------------------------------------------------------- CPU: oracle frozen
def test_oracle_stress_golden(oracle):
    d = fixture("stress_n4")
    o = make_oracle(oracle, d, 0)
    try:
        for it in (0, 1):
            P, K, fails, _ = o.stress_update(1, it, d["Fn"], d["Fn1"])
            assert fails == 0
            assert per_voxel_rel(P, d[f"P_it{it}"]) < 1e-12
            assert per_voxel_rel(K, d[f"K4_it{it}"]) < 1e-12
        o.commit()
        assert per_voxel_rel(o.history()[0], d["hist_committed"]) < 1e-12
    finally:
        o.close()


@pytest.mark.parametrize("name,gmap", [("green_n5_ref", 0), ("green_n6_centered", 1)])
def test_oracle_green_golden(oracle, name, gmap):
    d = fixture(name)
    o = make_oracle(oracle, d, gmap)
    try:
        assert rel(o.green(d["x"], True, K4=d["K4"]), d["y_K"]) < 1e-12
        assert rel(o.green(d["x"], False, K4=d["K4"]), d["y_I"]) < 1e-12
    finally:
        o.close()


def test_oracle_load_golden(oracle):
    d = fixture("load_n5")
    o = make_oracle(oracle, d, 0)
    load = rve.uniaxial_tension(0.03, 20)
    try:
        o.nr3_begin(1e-10)
        for step in (1, 2, 3):
            rc, Pbar, st = o.nr3_step(step, load.BC_all[step - 1], load.isNBC, 1e-6, 1e-10, 20)
            assert rc == 0
            assert rel(Pbar, d["Pbar"][step - 1]) < 1e-10
            assert st["newton_iters"] == d["newton"][step - 1]
        assert per_voxel_rel(o.fields()["Pn1"], d["Pn1"]) < 1e-10
    finally:
        o.close()


# ---------------------------------------------------------------- GPU: library vs golden
@pytest.mark.gpu
def test_gpu_stress_golden(gpulib):
    d = fixture("stress_n4")
    s = make_solver(gpulib, d, 0)
    try:
        for it in (0, 1):
            P, K, rc = s.drive_eps_sig(1, it, d["Fn"], d["Fn1"], want_K4=True)
            assert rc == 0
            assert per_voxel_rel(P, d[f"P_it{it}"]) < 1e-8
            assert per_voxel_rel(K, d[f"K4_it{it}"]) < 1e-8
        s.commit()
        _, _, H = s.fields(history=True)
        assert per_voxel_rel(H, d["hist_committed"]) < 1e-8
    finally:
        s.close()


@pytest.mark.gpu
@pytest.mark.parametrize("name,gmap", [("green_n5_ref", 0), ("green_n6_centered", 1)])
def test_gpu_green_golden(gpulib, name, gmap):
    d = fixture(name)
    s = make_solver(gpulib, d, gmap)
    try:
        s.set_K4(d["K4"])
        assert rel(s.G_K_dF(d["x"], True), d["y_K"]) < 1e-11
        assert rel(s.G_K_dF(d["x"], False), d["y_I"]) < 1e-11
    finally:
        s.close()


@pytest.mark.gpu
def test_gpu_load_golden(gpulib):
    d = fixture("load_n5")
    s = make_solver(gpulib, d, 0)
    load = rve.uniaxial_tension(0.03, 20)
    try:
        s.nr3_begin(1e-10)
        for step in (1, 2, 3):
            rc, Pbar, st = s.nr3_step(step, load.BC_all[step - 1], load.isNBC, 1e-6, 1e-10, 20)
            assert rc == 0
            assert rel(Pbar, d["Pbar"][step - 1]) < 1e-10
            assert st["newton_iters"] == d["newton"][step - 1]
        F, P = s.fields()
        assert per_voxel_rel(P, d["Pn1"]) < 1e-8
        assert rel(F, d["Fn1"]) < 1e-9
    finally:
        s.close()
