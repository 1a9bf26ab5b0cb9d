"""Dislocation-density hardening: Ma-Roters-Raabe (h_type 7: mm10_slipinc_mrr ..
mm10_dgdd_mrr, src/mm10_b.f:2343-3325; mm10_init_mrr, src/mm10_a.f:2205-2223) and ORNL
(h_type 4: mm10_slipinc_ornl .. mm10_dgdd_ornl, src/mm10_b.f:3330-4370): twelve
dislocation densities as the slip resistance variables, a (6 + 12)-unknown local Newton.
The oracle against the reference's interaction tables, the Jacobian against central
differences (exact derivatives) and the reference's formulas' known mismatch, the local
solve's convergence, and the GPU kernels (stress_mrr.cu, stress_ornl.cu) against the
oracle."""
import os

import numpy as np
import pytest

from cpfft_gb300 import rve

LAWS = {"mrr": rve.MRR_FCC, "ornl": rve.ORNL_FCC}
law = pytest.mark.parametrize("law", sorted(LAWS))
KOCKS = np.array([20.0, 35.0, 50.0])
GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "slip_tables.npz")


def stretch(F0, a=1e-3):
    F1 = F0.copy()
    F1[0, 0] += a
    F1[1, 1] -= 0.5 * a
    F1[2, 2] -= 0.5 * a
    return F1


def test_interaction_matrices_match_the_reference_table(oracle):
    """The forest / parallel projections formed from the slip geometry equal
    mm10_mrr_GHfcc's table (src/mm10_e.f), read from the reference into the fixture."""
    G, H = oracle.mrr_interaction()
    ref = np.load(GOLDEN)
    assert np.abs(G - ref["G1"]).max() < 1e-15
    assert np.abs(H - ref["H1"]).max() < 1e-15
    # systems on one plane: no forest component, full parallel component
    for p in range(4):
        blk = slice(3 * p, 3 * p + 3)
        assert np.all(G[blk, blk] == 0.0) and np.allclose(H[blk, blk], 1.0)


def initial_x(rng):
    return np.concatenate([[150., -60., -80., 20., 10., -15.], 1e6 * (1 + 0.3 * rng.random(12))])


def fd_jacobian(oracle, crystal, x, D, hs=1e-4):
    J = np.zeros((18, 18))
    for c in range(18):
        h = hs * max(abs(x[c]), 1.0)
        xp, xm = x.copy(), x.copy()
        xp[c] += h
        xm[c] -= h
        J[:, c] = (oracle.mrr_residual(crystal, KOCKS, D, 1.0, xp)[0] -
                   oracle.mrr_residual(crystal, KOCKS, D, 1.0, xm)[0]) / (2 * h)
    return J


@law
def test_exact_jacobian_against_finite_differences(oracle, law):
    """exact_j22 = 1: the 18 x 18 Jacobian differentiates the residual (rows scaled by their
    largest entry; rows of systems that do not slip are at the differences' noise floor)."""
    D = np.array([1e-3, -4e-4, -6e-4, 2e-4, 1e-4, -1e-4])
    x = initial_x(np.random.default_rng(0))
    R, J = oracle.mrr_residual(LAWS[law], KOCKS, D, 1.0, x)
    Jfd = fd_jacobian(oracle, LAWS[law], x, D)
    rowmax = np.maximum(np.abs(Jfd).max(axis=1), np.abs(J).max(axis=1))
    sig = rowmax > 1e-3
    err = np.abs(J - Jfd)[sig] / rowmax[sig][:, None]
    assert err.max() < 1e-4
    # the stress rows (J11, J12): the differences' truncation error of the steep slip law
    assert (np.abs(J[:6] - Jfd[:6]) / rowmax[:6, None]).max() < 1e-5


@law
def test_reference_jacobian_differs_where_the_reference_does(oracle, law):
    """exact_j22 = 0 takes the reference's mm10_estress_mrr / mm10_ehard_mrr: sqrt(rho_F)
    where mm10_h_mrr has sqrt(rho_P) (src/mm10_b.f:2635 against :2952, :3075).  Its
    stress rows agree with the exact ones; its density rows do not."""
    D = np.array([1e-3, -4e-4, -6e-4, 2e-4, 1e-4, -1e-4])
    x = initial_x(np.random.default_rng(0))
    _, Je = oracle.mrr_residual(LAWS[law], KOCKS, D, 1.0, x)
    _, Jr = oracle.mrr_residual(dict(LAWS[law], exact_j22=0), KOCKS, D, 1.0, x)
    assert np.abs(Je[:6] - Jr[:6]).max() == 0.0
    scale = np.abs(Je[6:, :6]).max()
    assert np.abs(Je[6:, :6] - Jr[6:, :6]).max() > 1e-2 * scale


@law
def test_local_solve_converges_to_the_residual_root(oracle, law):
    """First implicit pass of step 1 (rotation-free stretch, Rp = I): the converged
    (sigma, rho) zeroes the residual; exact and reference Jacobians reach the same state,
    the exact one in fewer iterations."""
    F1 = stretch(np.eye(3), 2e-3)
    out = {}
    for ex in (1, 0):
        cr = dict(LAWS[law], exact_j22=ex)
        r = oracle.voxel_update(cr, KOCKS, 1.0, 1, 1, np.eye(3), F1)
        assert r["iters"] > 0
        h = r["hist"]
        x = np.concatenate([h[0:6], h[31:43]])
        D = h[16:22]
        R, _ = oracle.mrr_residual(cr, KOCKS, D, 1.0, x)
        assert np.abs(R[:6]).max() < 1e-8 * np.abs(x[:6]).max()
        assert np.abs(R[6:]).max() < 1e-8 * np.abs(x[6:]).max()
        out[ex] = (x, r["iters"])
    assert np.abs(out[1][0] - out[0][0]).max() < 1e-8 * np.abs(out[1][0]).max()
    assert out[1][1] < out[0][1]


@law
def test_densities_grow_under_monotonic_loading(oracle, law):
    """Ten plastic steps: the local Newton converges in a few iterations each, the stress
    saturates below the elastic line and the densities of the active systems grow (those
    of systems that barely slip may lose a little to annihilation)."""
    hist, F0 = None, np.eye(3)
    rho0 = None
    for step in range(1, 11):
        F1 = stretch(F0)
        r = oracle.voxel_update(LAWS[law], KOCKS, 1.0, step, 1, F0, F1, hist)
        assert 0 < r["iters"] <= 6, (step, r["iters"])
        if rho0 is None:
            rho0 = r["hist"][31:43].copy()
        hist, F0 = r["hist"], F1
    rho = hist[31:43]
    assert rho.min() > (1 - 1e-6) * rho0.min() and rho.max() > 1.5 * LAWS[law]["theta_0"]
    assert 100.0 < hist[0] < 400.0


@law
def test_tangent_against_finite_differences(oracle, law):
    """dP/dF of a plastic step (exact local Jacobian: T = (J11 - J12 J22^-1 J21)^-1 C)
    against a central difference of P."""
    hist, Fs = None, [np.eye(3)]
    for step in (1, 2, 3):
        F1 = stretch(Fs[-1])
        hist = oracle.voxel_update(LAWS[law], KOCKS, 1.0, step, 1, Fs[-1], F1, hist)["hist"]
        Fs.append(F1)
    rng = np.random.default_rng(1)
    Fa = Fs[-1]
    Fb = stretch(Fa) + 2e-4 * rng.standard_normal((3, 3))
    r = oracle.voxel_update(LAWS[law], KOCKS, 1.0, 4, 1, Fa, Fb, hist)
    d = 1e-7
    Afd = np.zeros((9, 9))
    for m in range(9):
        e = np.zeros(9)
        e[m] = d
        Pp = oracle.voxel_update(LAWS[law], KOCKS, 1.0, 4, 1, Fa, Fb + e.reshape(3, 3), hist)["P"]
        Pm = oracle.voxel_update(LAWS[law], KOCKS, 1.0, 4, 1, Fa, Fb - e.reshape(3, 3), hist)["P"]
        Afd[:, m] = (Pp - Pm) / (2 * d)
    # the tangent is symmetrised (mm10_a_make_symm_1) and neglects the rotation update
    assert np.abs(r["A"] - Afd).max() < 2e-2 * np.abs(Afd).max()


@law
def test_oracle_load_steps(oracle, law):
    """Whole load steps of a 5^3 LAWS[law] grid in the oracle: the Newton loop converges."""
    N = 5
    r = rve.make_rve(N, 3, 94, LAWS[law])
    load = rve.prescribed_stretch([0.003, -0.0015, -0.0015], 3)
    o = oracle.Oracle(N, r.mat_list, r.kocks, r.crystals, 1.0, 0, nthreads=4)
    try:
        o.nr3_begin(1e-10)
        for step in (1, 2, 3):
            rc, Pbar, st = o.nr3_step(step, load.BC_all[step - 1], load.isNBC, 1e-5, 1e-10, 10)
            assert rc == 0 and st["local_fallbacks"] == 0
        assert o.history()[0].shape == (oracle.HIST_WORDS_MRR, N ** 3)
    finally:
        o.close()


def per_voxel_rel(a, b):
    scale = np.maximum(np.abs(b).max(axis=0), 1e-6 * np.abs(b).max())
    return (np.abs(a - b).max(axis=0) / scale).max()


@pytest.mark.gpu
@law
@pytest.mark.parametrize("exact", [1, 0])
def test_gpu_mrr_stress_update_parity(gpulib, oracle, law, exact):
    """P, dP/dF and the twelve densities and rates of the GPU LAWS[law] kernel against the oracle
    over the passes of two steps, with the exact and with the reference's Jacobian."""
    N = 5
    crystal = dict(LAWS[law], exact_j22=exact)
    r = rve.make_rve(N, 4, 95, crystal)
    s = gpulib.Solver(N, r.mat_list, r.kocks, r.crystals, 1.0, gpulib.G_REF_SHIFT)
    o = oracle.Oracle(N, r.mat_list, r.kocks, r.crystals, 1.0, 0, nthreads=8)
    try:
        rng = np.random.default_rng(8)
        Fn = np.zeros((9, N ** 3))
        Fn[[0, 4, 8]] = 1.0
        Fn1 = Fn + 1.0e-3 * rng.standard_normal((9, N ** 3))
        Fn1[0] += 2e-3
        for step, (Fa, Fb) in enumerate([(Fn, Fn1), (Fn1, Fn1 + (Fn1 - Fn))], start=1):
            for it in (0, 1, 2):
                P, K, rc = s.drive_eps_sig(step, it, Fa, Fb, want_K4=True)
                Po, Ko, fails, _ = o.stress_update(step, it, Fa, Fb)
                assert rc == (1 if fails else 0)
                assert per_voxel_rel(P, Po) < 1e-8, (step, it)
                assert per_voxel_rel(K, Ko) < 1e-7, (step, it)
            s.commit()
            o.commit()
            hg = s.fields(history=True)[2]
            ho = o.history()[0]
            assert hg.shape == ho.shape == (gpulib.HIST_WORDS_MRR, N ** 3)
            for w in range(31, 55):
                assert np.abs(hg[w] - ho[w]).max() <= 1e-9 * np.abs(ho[w]).max() + 1e-12, w
    finally:
        s.close()
        o.close()


@pytest.mark.gpu
@law
def test_gpu_mrr_load_steps(gpulib, oracle, law):
    """Whole load steps (7^3, uniaxial-strain stretch 1e-3 a step): P_bar and Newton
    counts against the oracle."""
    N = 7
    r = rve.make_rve(N, 6, 96, LAWS[law])
    load = rve.prescribed_stretch([0.004, -0.002, -0.002], 4)
    s = gpulib.Solver(N, r.mat_list, r.kocks, r.crystals, 1.0, gpulib.G_REF_SHIFT)
    o = oracle.Oracle(N, r.mat_list, r.kocks, r.crystals, 1.0, 0, nthreads=8)
    try:
        s.nr3_begin(1e-10)
        o.nr3_begin(1e-10)
        for step in (1, 2, 3):
            rc, Pbar, st = s.nr3_step(step, load.BC_all[step - 1], load.isNBC, 1e-5, 1e-10, 10)
            rco, Pbo, sto = o.nr3_step(step, load.BC_all[step - 1], load.isNBC, 1e-5, 1e-10, 10)
            assert rc >= 0 and rco >= 0 and rc == rco
            assert np.abs(Pbar - Pbo).max() < 1e-10 * np.abs(Pbo).max(), step
            assert st["newton_iters"] == sto["newton_iters"]
    finally:
        s.close()
        o.close()


@pytest.mark.gpu
@law
def test_gpu_mrr_mixed_form(gpulib, oracle, law):
    """The fast form (FP32 inner Krylov with the reference-medium preconditioner, FP32
    tangent, voxel queue) on an LAWS[law] grid: P_bar within 1e-6 of the plain oracle."""
    N = 8
    r = rve.make_rve(N, 6, 97, LAWS[law])
    load = rve.prescribed_stretch([0.004, -0.002, -0.002], 4)
    s = gpulib.Solver(N, r.mat_list, r.kocks, r.crystals, 1.0, gpulib.G_CENTERED,
                      gpulib.PREC_MIXED)
    o = oracle.Oracle(N, r.mat_list, r.kocks, r.crystals, 1.0, 1, nthreads=8)
    try:
        s.set_mode(gpulib.PREC_MIXED, gpulib.TANGENT_F32)
        s.set_precond(gpulib.PRECOND_REFERENCE)
        s.set_schedule(gpulib.SCHED_QUEUE)
        s.nr3_begin(1e-10)
        o.nr3_begin(1e-10)
        for step in (1, 2):
            rc, Pbar, st = s.nr3_step(step, load.BC_all[step - 1], load.isNBC, 1e-6, 1e-10, 20)
            rco, Pbo, sto = o.nr3_step(step, load.BC_all[step - 1], load.isNBC, 1e-6, 1e-10, 20)
            assert rc >= 0 and rco >= 0
            assert np.abs(Pbar - Pbo).max() < 1e-6 * np.abs(Pbo).max(), step
    finally:
        s.close()
        o.close()
