"""Bilinear Mises material (mm01, src/mm01.f): the oracle's restatement against the
model's own identities, and the GPU path (launch_mises) against the oracle on a grid
mixing mm01 and crystal voxels.  The reference's mm01 example deck runs in
tests/test_example_decks.py."""
import numpy as np
import pytest

from cpfft_gb300 import rve

MAT1, MAT2 = rve.MM01_DECK
SQ2, ROOT3 = 1.414213562373095, 1.7320508075688  # mm01_init's constants


def stretch(F0, dxx, dyy, dzz):
    F1 = F0.copy()
    F1[0, 0] += dxx
    F1[1, 1] += dyy
    F1[2, 2] += dzz
    return F1


def dev_norm(s):
    """sqrt(s:s) of a deviator in Voigt form with tensor shears (mm01's mrts)."""
    return np.sqrt(s[0] ** 2 + s[1] ** 2 + s[2] ** 2 + 2 * (s[3] ** 2 + s[4] ** 2 + s[5] ** 2))


def test_elastic_step_is_hooke(oracle):
    """Below yield the unrotated stress is the isotropic C times the strain increment."""
    m = MAT1
    F1 = stretch(np.eye(3), 2e-4, -1e-4, 5e-5)
    r = oracle.mises_update(m, 1, np.eye(3), F1)
    e, nu = m["e"], m["nu"]
    lam, G = e * nu / ((1 + nu) * (1 - 2 * nu)), e / (2 * (1 + nu))
    # the unrotated strain increment of a pure stretch: ln-free mid-point rate, diagonal
    d = np.array([(F1[i, i] - 1) / (0.5 * (F1[i, i] + 1)) for i in range(3)])
    sig = lam * d.sum() + 2 * G * d
    assert np.abs(r["sig"][:3] - sig).max() < 1e-10 * np.abs(sig).max()
    assert np.abs(r["sig"][3:]).max() < 1e-12 * np.abs(sig).max()
    assert r["hist"][9] == 3.0  # not yielding
    C = r["cep"]
    assert abs(C[0, 0] - (lam + 2 * G)) < 1e-9 * C[0, 0] and abs(C[3, 3] - G) < 1e-9 * G


@pytest.mark.parametrize("beta", [1.0, 0.5, 0.0])
def test_plastic_steps_stay_on_the_yield_surface(oracle, beta):
    """After each plastic step: |dev(sigma) - alpha| = sqrt(2) k_n+1 (the return map), and
    k_n+1 = (yld + beta h eps_p) / sqrt(3) (linear isotropic hardening of the accumulated
    plastic strain); the back stress stays deviatoric."""
    m = dict(MAT1, beta=beta)
    h = m["tan_e"] * m["e"] / (m["e"] - m["tan_e"])
    F0, hist = np.eye(3), None
    for step in range(1, 7):
        F1 = stretch(F0, 8e-3, -3e-3, -5e-3)
        r = oracle.mises_update(m, step, F0, F1, hist)
        H = r["hist"]
        s = r["sig"].copy()
        s[:3] -= s[:3].mean()
        alpha = H[11:17]
        k1, epsp = H[7], H[8]
        assert H[9] == 1.0, step  # yielding
        assert abs(dev_norm(s - alpha) - SQ2 * k1) < 1e-9 * k1
        assert abs(k1 - (m["yld_pt"] + beta * h * epsp) / ROOT3) < 1e-9 * k1
        assert abs(alpha[:3].sum()) < 1e-9 * max(1.0, np.abs(alpha).max())
        hist, F0 = H, F1
    if beta == 1.0:
        assert np.abs(hist[11:17]).max() == 0.0  # purely isotropic: no back stress


def test_tangent_against_finite_differences(oracle):
    """dP/dF (cnst1 through cep2A) against a central difference of P on a plastic step;
    cnst1 keeps the reference's 10-digit sqrt(2), so the match is to ~1e-9 only."""
    m = MAT2
    F0 = np.eye(3)
    F1 = stretch(F0, 1.2e-2, -4e-3, -6e-3)
    h0 = oracle.mises_update(m, 1, F0, F1)["hist"]
    rng = np.random.default_rng(5)
    F2 = stretch(F1, 6e-3, -2e-3, -3e-3) + 1e-3 * rng.standard_normal((3, 3))
    r = oracle.mises_update(m, 2, F1, F2, h0)
    assert r["hist"][9] == 1.0
    d = 1e-7
    Afd = np.zeros((9, 9))
    for k in range(9):
        dk = np.zeros(9)
        dk[k] = d
        Pp = oracle.mises_update(m, 2, F1, F2 + dk.reshape(3, 3), h0)["P"]
        Pm = oracle.mises_update(m, 2, F1, F2 - dk.reshape(3, 3), h0)["P"]
        Afd[:, k] = (Pp - Pm) / (2 * d)
    assert np.abs(r["A"] - Afd).max() < 1e-6 * np.abs(Afd).max()


def test_plastic_work_matches_the_dissipation(oracle):
    """Isotropic hardening, proportional loading: the plastic work increment equals
    the yield stress times the equivalent plastic strain increment to first order."""
    m = dict(MAT1, beta=1.0)
    F0, hist = np.eye(3), None
    for step in range(1, 4):
        F1 = stretch(F0, 8e-3, -4e-3, -4e-3)
        r = oracle.mises_update(m, step, F0, F1, hist)
        H = r["hist"]
        if step > 1:
            dwp = H[18] - hist[18]
            debar = H[19] - hist[19]
            sbar = 0.5 * ROOT3 * (H[7] + hist[7])  # Mises stress = sqrt(3) k
            assert abs(dwp - sbar * debar) < 2e-3 * dwp
        hist, F0 = H, F1


def mixed_grid(N, seed):
    """Material 1: FCC crystals; materials 2 and 3: the deck's two bilinear materials."""
    r = rve.make_rve(N, 3, seed)
    rng = np.random.default_rng(seed)
    mat = rng.integers(1, 4, N ** 3).astype(np.int32)
    crystals = [r.crystals[0], rve.NOT_A_CRYSTAL, rve.NOT_A_CRYSTAL]
    return mat, r.kocks, crystals


def per_voxel_rel(a, b):
    scale = np.maximum(np.abs(b).max(axis=0), 1e-6 * np.abs(b).max())
    return (np.abs(a - b).max(axis=0) / scale).max()


def test_oracle_mixed_grid_dispatch(oracle):
    """The oracle's grid path gives every mm01 voxel the single-point result."""
    N = 3
    mat, kocks, crystals = mixed_grid(N, 81)
    o = oracle.Oracle(N, mat, kocks, crystals, 1.0, 0, nthreads=1)
    try:
        o.set_mises(2, MAT1)
        o.set_mises(3, MAT2)
        rng = np.random.default_rng(2)
        Fn = np.zeros((9, N ** 3))
        Fn[[0, 4, 8]] = 1.0
        Fn1 = Fn + 4e-3 * rng.standard_normal((9, N ** 3))
        P, K, fails, _ = o.stress_update(1, 1, Fn, Fn1)
        assert fails == 0
        for v in np.nonzero(mat > 1)[0][:5]:
            r = oracle.mises_update(MAT1 if mat[v] == 2 else MAT2, 1, Fn[:, v].reshape(3, 3),
                                    Fn1[:, v].reshape(3, 3))
            assert np.array_equal(r["P"], P[:, v])
            assert np.array_equal(r["A"].ravel(), K[:, v])
    finally:
        o.close()


@pytest.mark.gpu
def test_gpu_mixed_grid_stress_update(gpulib, oracle):
    """One grid with crystal and mm01 voxels: P, dP/dF and the history words of both
    kinds against the oracle, over a step's Newton passes and a second step."""
    N = 5
    mat, kocks, crystals = mixed_grid(N, 82)
    s = gpulib.Solver(N, mat, kocks, crystals, 1.0, gpulib.G_REF_SHIFT)
    o = oracle.Oracle(N, mat, kocks, crystals, 1.0, 0, nthreads=8)
    try:
        for k, m in ((2, MAT1), (3, MAT2)):
            s.set_mises(k, **m)
            o.set_mises(k, m)
        rng = np.random.default_rng(3)
        Fn = np.zeros((9, N ** 3))
        Fn[[0, 4, 8]] = 1.0
        Fn1 = Fn + 6e-3 * rng.standard_normal((9, N ** 3))
        for it in (0, 1, 2):
            P, K, rc = s.drive_eps_sig(1, it, Fn, Fn1, want_K4=True)
            Po, Ko, fails, _ = o.stress_update(1, it, Fn, Fn1)
            assert rc == (1 if fails else 0)
            m01 = mat > 1
            assert per_voxel_rel(P[:, m01], Po[:, m01]) < 1e-12
            assert per_voxel_rel(K[:, m01], Ko[:, m01]) < 1e-11
            assert per_voxel_rel(P[:, ~m01], Po[:, ~m01]) < 1e-8
        s.commit()
        o.commit()
        m01 = mat > 1
        hg = s.fields(history=True)[2]
        ho = o.history()[0]
        assert np.abs(hg[:, m01] - ho[:, m01]).max() < 1e-11 * max(1.0, np.abs(ho[:, m01]).max())
        Fn2 = Fn1 + 6e-3 * rng.standard_normal((9, N ** 3))  # step 2 reads the stored state
        P, K, rc = s.drive_eps_sig(2, 1, Fn1, Fn2, want_K4=True)
        Po, Ko, fails, _ = o.stress_update(2, 1, Fn1, Fn2)
        assert per_voxel_rel(P[:, m01], Po[:, m01]) < 1e-12
        assert per_voxel_rel(K[:, m01], Ko[:, m01]) < 1e-11
    finally:
        s.close()
        o.close()


def test_not_a_crystal_constant():
    """The Python constant, the material helper and include/cpfft_gpu.h agree."""
    import cpfft_gb300
    assert cpfft_gb300.NOT_A_CRYSTAL == rve.NOT_A_CRYSTAL["slip_type"] == 0


@pytest.mark.gpu
def test_gpu_undefined_material_fails_loudly(gpulib):
    N = 3
    mat = np.ones(N ** 3, np.int32)
    s = gpulib.Solver(N, mat, np.zeros((3, N ** 3)), [rve.NOT_A_CRYSTAL], 1.0)
    try:
        Fn = np.zeros((9, N ** 3))
        Fn[[0, 4, 8]] = 1.0
        with pytest.raises(RuntimeError, match="set_mises"):
            s.drive_eps_sig(1, 0, Fn, Fn)
        with pytest.raises(RuntimeError):
            s.set_mises(1, e=100.0, nu=0.3, yld_pt=1.0, tan_e=200.0)  # tan_e >= e
    finally:
        s.close()


@pytest.mark.gpu
def test_gpu_mixed_grid_fast_form(gpulib):
    """Crystal and mm01 voxels on one grid in the fast form (FP32 inner CG with the
    reference-medium preconditioner, iterate + trial starts, FP32 tangent, the voxel
    queue, whose ordering mixes the mm01 voxels the crystal kernel skips) against the plain
    FP64 form: P_bar within 1e-6, the same Newton counts."""
    N = 16
    mat, kocks, crystals = mixed_grid(N, 83)
    load = rve.uniaxial_tension(0.02, 20)
    out = []
    for fast in (False, True):
        s = gpulib.Solver(N, mat, kocks, crystals, 1.0, gpulib.G_CENTERED,
                          gpulib.PREC_MIXED if fast else gpulib.PREC_FP64)
        try:
            for k, m in ((2, MAT1), (3, MAT2)):
                s.set_mises(k, **m)
            if fast:
                s.set_mode(gpulib.PREC_MIXED, gpulib.START_ITERATE | gpulib.START_TRIAL |
                           gpulib.TANGENT_F32)
                s.set_precond(gpulib.PRECOND_REFERENCE)
                s.set_schedule(gpulib.SCHED_QUEUE)
            s.nr3_begin(1e-10)
            pb, its = [], []
            for step in (1, 2, 3):
                rc, Pbar, st = s.nr3_step(step, load.BC_all[step - 1], load.isNBC, 1e-6, 1e-10, 20)
                assert rc == 0
                pb.append(Pbar)
                its.append(st["newton_iters"])
            out.append((np.array(pb), its))
        finally:
            s.close()
    (pb0, it0), (pb1, it1) = out
    assert np.abs(pb1 - pb0).max() < 1e-6 * np.abs(pb0).max()
    assert it1 == it0
