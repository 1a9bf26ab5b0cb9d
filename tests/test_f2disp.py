"""Nodal displacements (f2disp, src/f2disp.f:16-400): the GPU's separable DCT-I solve of
the reference's least-squares system against the oracle's element-by-element assembly and
sparse direct solve (oracle/f2disp_ref.py), on a random F field and on the field of a real
load step, with a non-cubic box."""
import numpy as np
import pytest

from cpfft_gb300 import rve
from oracle import f2disp_ref


def test_oracle_affine_field_is_exact():
    """A homogeneous F is reproduced exactly: u = (F - I) X, for every node."""
    N = 4
    Fbar = np.array([[1.02, 0.01, 0.0], [0.003, 0.99, -0.004], [0.0, 0.002, 1.01]])
    F = np.repeat(Fbar.reshape(9, 1), N ** 3, axis=1)
    L = (100.0, 80.0, 120.0)
    u = f2disp_ref.displacements(F, N, L)
    N1 = N + 1
    idx = np.arange(N1 ** 3)
    X = np.stack([(idx % N1) * L[0] / N, (idx // N1 % N1) * L[1] / N,
                  (idx // (N1 * N1)) * L[2] / N], axis=1)
    assert np.abs(u - X @ (Fbar - np.eye(3)).T).max() < 1e-10


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["random", "load_step"])
def test_gpu_f2disp(gpulib, case):
    N = 6 if case == "random" else 7
    L = (100.0, 80.0, 120.0)
    r = rve.make_rve(N, 3, 71)
    s = gpulib.Solver(N, r.mat_list, r.kocks, r.crystals, 1.0, gpulib.G_REF_SHIFT)
    try:
        if case == "random":
            rng = np.random.default_rng(3)
            F = np.zeros((9, N ** 3))
            F[[0, 4, 8]] = 1.0
            F = F + 0.01 * rng.standard_normal((9, N ** 3))
            s.set_F(F, F)
        else:
            load = rve.uniaxial_tension(0.02, 20)
            s.nr3_begin(1e-10)
            for step in (1, 2):
                s.nr3_step(step, load.BC_all[step - 1], load.isNBC, 1e-6, 1e-10, 20)
            F, _ = s.fields()
        u = s.f2disp(L)
        uo = f2disp_ref.displacements(F, N, L)
        # both solve for positions (magnitude ~ the box) and subtract the reference
        # coordinates, so the rounding scales with the box, not with u
        assert np.abs(u - uo).max() <= 1e-12 * max(L), np.abs(u - uo).max()
    finally:
        s.close()


@pytest.mark.gpu
def test_gpu_disp_file(gpulib, tmp_path):
    """oudisp's wnd file: the header and one (3e15.6) line per node of u."""
    import os
    from oracle import flat_ref
    N = 5
    r = rve.make_rve(N, 3, 72)
    s = gpulib.Solver(N, r.mat_list, r.kocks, r.crystals, 1.0, gpulib.G_REF_SHIFT)
    try:
        rng = np.random.default_rng(4)
        F = np.zeros((9, N ** 3))
        F[[0, 4, 8]] = 1.0
        F = F + 0.01 * rng.standard_normal((9, N ** 3))
        s.set_F(F, F)
        u = s.f2disp((100.0, 100.0, 100.0))
        s.write_disp_flat(3, (100.0, 100.0, 100.0), "rve5", str(tmp_path))
        lines = open(os.path.join(tmp_path, "wnd00003_text")).read().split("\n")
        assert lines[1] == "#  WARP3D nodal results: displacements  "
        assert lines[3] == "#  Model nodes, elements: %8d%8d" % ((N + 1) ** 3, N ** 3)
        body = lines[7:-1]
        assert len(body) == (N + 1) ** 3
        for n, line in enumerate(body):
            vals = [0.0 if abs(x) < 1e-30 else x for x in u[n]]
            assert line == "".join(flat_ref.e15_6(x) for x in vals)
    finally:
        s.close()
