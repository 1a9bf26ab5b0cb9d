"""The oracle's global loop (FFT_nr3: Newton, fftPcg, tangent_homo, NBC_update, G_K_dF) on
closed-form problems, with the FFT program's original St-Venant-Kirchhoff material
(constitutive, src/mm00.f:13-60; stiff phase K 8.33, mu 3.86, soft phase K 0.833,
mu 0.386): a homogeneous grid under uniaxial stress and a two-phase laminate, whose
discrete solution is the exact laminate solution (fields vary along x alone, so the Green
operator keeps F's second and third columns uniform and the traction P e1 continuous)."""
import numpy as np

from cpfft_gb300 import rve

STIFF = (8.33, 3.86)
SOFT = (0.833, 0.386)


def test_svk_tangent_against_finite_differences(oracle):
    F = np.eye(3) + 0.05 * np.random.default_rng(1).standard_normal((3, 3))
    P, A = oracle.svk_point(*STIFF, F)
    d = 1e-7
    Afd = np.zeros((9, 9))
    for m in range(9):
        e = np.zeros(9)
        e[m] = d
        Pp, _ = oracle.svk_point(*STIFF, F + e.reshape(3, 3))
        Pm, _ = oracle.svk_point(*STIFF, F - e.reshape(3, 3))
        Afd[:, m] = ((Pp - Pm) / (2 * d)).ravel()
    assert np.abs(A - Afd).max() < 1e-8 * np.abs(Afd).max()
    # P = F S with S from the Green-Lagrange strain
    E = 0.5 * (F.T @ F - np.eye(3))
    K, mu = STIFF
    S = (K - 2 * mu / 3) * np.trace(E) * np.eye(3) + 2 * mu * E
    assert np.abs(P - F @ S).max() < 1e-14


def grid(oracle, N, mat):
    o = oracle.Oracle(N, mat, np.zeros((3, N ** 3)), [rve.NOT_A_CRYSTAL] * 2, 1.0, 0,
                      nthreads=2)
    o.set_svk(1, *STIFF)
    o.set_svk(2, *SOFT)
    return o


def test_homogeneous_uniaxial_stress(oracle):
    """One phase, F_xx prescribed, the shears F_xy, F_xz, F_yz held at 0 and the other P
    components at 0 (mixed boundary conditions): F_yy = F_zz from S_yy = 0 and
    P_xx = F_xx S_xx, in closed form."""
    N = 3
    o = grid(oracle, N, np.ones(N ** 3, np.int32))
    load = rve.uniaxial_tension(0.02, 20)
    K, mu = STIFF
    lam = K - 2 * mu / 3
    try:
        o.nr3_begin(1e-10)
        for step in (1, 2, 3):
            rc, Pbar, _ = o.nr3_step(step, load.BC_all[step - 1], load.isNBC, 1e-8, 1e-10, 20)
            assert rc == 0
            fxx = load.BC_all[step - 1][0]
            Exx = 0.5 * (fxx ** 2 - 1)
            Eyy = -lam * Exx / (2 * lam + 2 * mu)
            Sxx = lam * (Exx + 2 * Eyy) + 2 * mu * Exx
            assert abs(Pbar[0] - fxx * Sxx) < 1e-9 * abs(fxx * Sxx)
            assert np.abs(np.delete(Pbar, 0)).max() < 1e-9 * abs(Pbar[0])
            F = o.fields()["Fn1"]
            fyy = np.sqrt(1 + 2 * Eyy)
            assert np.abs(F[4] - fyy).max() < 1e-10 and np.abs(F[8] - fyy).max() < 1e-10
    finally:
        o.close()


def laminate_solution(Fbar, fa):
    """Phase A (volume fraction fa) and B: F's first column per phase, the others shared,
    traction P e1 equal in both; Newton on the three unknowns of phase A's column."""
    import scipy.optimize

    def fields(a):
        FA, FB = Fbar.copy(), Fbar.copy()
        FA[:, 0] = a
        FB[:, 0] = (Fbar[:, 0] - fa * a) / (1 - fa)
        return FA, FB

    def res(a):
        FA, FB = fields(a)
        return (np.asarray(oracle_svk(STIFF, FA))[:, 0] - np.asarray(oracle_svk(SOFT, FB))[:, 0])

    a = scipy.optimize.fsolve(res, Fbar[:, 0].copy(), xtol=1e-13)
    FA, FB = fields(a)
    PA, PB = oracle_svk(STIFF, FA), oracle_svk(SOFT, FB)
    return FA, FB, PA, PB


def oracle_svk(km, F):
    from oracle import pyoracle
    return pyoracle.svk_point(*km, F)[0]


def test_two_phase_laminate(oracle):
    """Stiff layers (x-planes 0, 1) and soft layers (2-4) of a 5^3 grid under a prescribed
    F_bar with shears: every voxel's F and P and P_bar against the laminate solution."""
    N = 5
    c = np.arange(N ** 3) // (N * N)  # the x index (slowest memory axis)
    mat = np.where(c < 2, 1, 2).astype(np.int32)
    fa = 2 / N
    o = grid(oracle, N, mat)
    dF = np.array([[2.0, 0.5, -0.3], [0.4, -1.0, 0.2], [-0.6, 0.3, -0.7]]) * 1e-3
    isNBC = np.zeros(9, np.int32)
    try:
        o.nr3_begin(1e-10)
        for step in (1, 2, 3):
            Fbar = np.eye(3) + step * dF
            rc, Pbar, _ = o.nr3_step(step, Fbar.ravel(), isNBC, 1e-8, 1e-10, 20)
            assert rc == 0
            FA, FB, PA, PB = laminate_solution(Fbar, fa)
            assert np.abs(FA - FB).max() > 0.5 * np.abs(dF).max() * step  # a real contrast
            f = o.fields()
            F, P = f["Fn1"], f["Pn1"]
            for ph, Fx, Px in ((1, FA, PA), (2, FB, PB)):
                sel = mat == ph
                assert np.abs(F[:, sel] - Fx.ravel()[:, None]).max() < 1e-10
                assert np.abs(P[:, sel] - Px.ravel()[:, None]).max() < 1e-8 * np.abs(PA).max()
            Pref = fa * PA + (1 - fa) * PB
            assert np.abs(Pbar - Pref.ravel()).max() < 1e-8 * np.abs(Pref).max()
    finally:
        o.close()


def test_laminate_under_uniaxial_stress(oracle):
    """The laminate with mixed boundary conditions (F_xx, F_xy, F_xz, F_yz prescribed, the
    other five P_bar components zero): the closed form now solves for the free components
    of F_bar together with the layers' first columns, which exercises tangent_homo and
    NBC_update on a heterogeneous grid."""
    import scipy.optimize
    N = 5
    c = np.arange(N ** 3) // (N * N)
    mat = np.where(c < 2, 1, 2).astype(np.int32)
    fa = 2 / N
    load = rve.uniaxial_tension(0.02, 20)
    free = np.nonzero(load.isNBC)[0]  # the components with P_bar prescribed (zero)
    o = grid(oracle, N, mat)
    try:
        o.nr3_begin(1e-10)
        for step in (1, 2, 3):
            bc = load.BC_all[step - 1]

            def unpack(x):
                Fbar = bc.copy()
                Fbar[free] = x[3:]
                Fbar = Fbar.reshape(3, 3)
                FA, FB = Fbar.copy(), Fbar.copy()
                FA[:, 0] = x[:3]
                FB[:, 0] = (Fbar[:, 0] - fa * x[:3]) / (1 - fa)
                return FA, FB

            def res(x):
                FA, FB = unpack(x)
                PA, PB = oracle_svk(STIFF, FA), oracle_svk(SOFT, FB)
                Pbar = (fa * PA + (1 - fa) * PB).ravel()
                return np.concatenate([PA[:, 0] - PB[:, 0], Pbar[free]])

            x0 = np.concatenate([bc.reshape(3, 3)[:, 0], np.eye(3).ravel()[free]])
            x = scipy.optimize.fsolve(res, x0, xtol=1e-13)
            assert np.abs(res(x)).max() < 1e-12
            FA, FB = unpack(x)
            PA, PB = oracle_svk(STIFF, FA), oracle_svk(SOFT, FB)
            rc, Pbar, _ = o.nr3_step(step, bc, load.isNBC, 1e-8, 1e-10, 20)
            assert rc == 0
            Pref = (fa * PA + (1 - fa) * PB).ravel()
            assert np.abs(Pbar - Pref).max() < 1e-8 * np.abs(Pref).max(), step
            F = o.fields()["Fn1"]
            for ph, Fx in ((1, FA), (2, FB)):
                assert np.abs(F[:, mat == ph] - Fx.ravel()[:, None]).max() < 1e-9, (step, ph)
    finally:
        o.close()
