"""BCC crystals with 48 slip systems (slip_type 8, src/mod_crystals.f:812-1207), the
crystal of the reference's example deck (examples/test_mm10.in): the slip geometry, the
stress update and whole load steps on the GPU against the oracle."""
import numpy as np
import pytest

from cpfft_gb300 import rve


def test_bcc48_geometry(oracle):
    C66, ms, qs = oracle.crystal_setup(rve.BCC48_DECK, np.zeros(3))
    assert ms.shape == (48, 6) and qs.shape == (48, 3)
    # Schmid tensors are traceless (b . n = 0) and distinct
    assert np.abs(ms[:, 0] + ms[:, 1] + ms[:, 2]).max() < 1e-15
    assert len({tuple(np.round(m, 12)) for m in ms}) == 48
    # isotropic stiffness: lambda + 2 mu on the diagonal
    e, nu = rve.BCC48_DECK["e"], rve.BCC48_DECK["nu"]
    assert abs(C66[0, 0] - e * (1 - nu) / ((1 + nu) * (1 - 2 * nu))) < 1e-8 * e


def rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def per_voxel_rel(a, b):
    scale = np.maximum(np.abs(b).max(axis=0), 1e-6 * np.abs(b).max())
    return (np.abs(a - b).max(axis=0) / scale).max()


@pytest.mark.gpu
def test_bcc48_stress_update_parity(gpulib, oracle):
    N = 5
    r = rve.make_rve(N, 3, 61, rve.BCC48_DECK)
    s = gpulib.Solver(N, r.mat_list, r.kocks, r.crystals, 10.0, gpulib.G_REF_SHIFT)
    o = oracle.Oracle(N, r.mat_list, r.kocks, r.crystals, 10.0, 0, nthreads=8)
    try:
        rng = np.random.default_rng(7)
        Fn = np.zeros((9, N ** 3))
        Fn[[0, 4, 8]] = 1.0
        Fn1 = Fn + 3e-3 * rng.standard_normal((9, N ** 3))
        for it in (0, 1, 2):
            P, K, rc = s.drive_eps_sig(1, it, Fn, Fn1, want_K4=True)
            Po, Ko, fails, _ = o.stress_update(1, it, Fn, Fn1)
            assert rc == (1 if fails else 0)
            assert per_voxel_rel(P, Po) < 1e-8
            # the tangent inherits the local solve's 1e-10 tolerance amplified by its
            # Jacobian's conditioning (48 systems, rate exponent 5.48): 6.5e-8 measured
            assert per_voxel_rel(K, Ko) < 5e-7
    finally:
        s.close()
        o.close()


@pytest.mark.gpu
def test_bcc48_example_deck_load_steps(gpulib, oracle):
    """The example deck's grid (7^3), crystal, time step (10 s) and loading (F_xx 0.03,
    F_yy -0.01, F_zz -0.01 in 10 steps), with seeded orientations: P_bar and per-voxel P
    of the first load steps against the oracle, identical Newton counts."""
    N = 7
    r = rve.make_rve(N, 5, 62, rve.BCC48_DECK)
    load = rve.prescribed_stretch([0.03, -0.01, -0.01], 10)
    s = gpulib.Solver(N, r.mat_list, r.kocks, r.crystals, 10.0, gpulib.G_REF_SHIFT)
    o = oracle.Oracle(N, r.mat_list, r.kocks, r.crystals, 10.0, 0, nthreads=8)
    try:
        s.nr3_begin(1e-10)
        o.nr3_begin(1e-10)
        for step in (1, 2, 3):
            rc, Pbar, st = s.nr3_step(step, load.BC_all[step - 1], load.isNBC, 1e-5, 1e-10, 10)
            rco, Pbo, sto = o.nr3_step(step, load.BC_all[step - 1], load.isNBC, 1e-5, 1e-10, 10)
            assert rc >= 0 and rco >= 0 and rc == rco
            assert rel(Pbar, Pbo) < 1e-9, (step, rel(Pbar, Pbo))
            assert st["newton_iters"] == sto["newton_iters"]
        F, P = s.fields()
        assert per_voxel_rel(P, o.fields()["Pn1"]) < 1e-8
    finally:
        s.close()
        o.close()
