"""CPU checks that pin the oracle to analytic known answers (parity with the reference
itself is unpinned: the reference ships no tests or golden data and cannot be built
here).  No GPU is touched."""
import numpy as np
import pytest
import scipy.linalg

from cpfft_gb300 import rve


def test_fft_matches_numpy(oracle):
    rng = np.random.default_rng(0)
    for N in (5, 7, 8, 12, 15, 16):
        x = rng.random((N, N, N)) + 1j * rng.random((N, N, N))
        y = oracle.fft3(x, -1)
        ref = np.fft.fftn(x)
        assert np.abs(y - ref).max() <= 1e-13 * np.abs(ref).max()
        z = oracle.fft3(y, +1)
        assert np.abs(z - x).max() <= 1e-13


def test_polar_matches_scipy(oracle):
    rng = np.random.default_rng(1)
    for _ in range(20):
        F = np.eye(3) + 0.2 * rng.standard_normal((3, 3))
        if np.linalg.det(F) <= 0.1:
            continue
        R = oracle.polar(F)
        Rr, _ = scipy.linalg.polar(F)
        assert np.abs(R - Rr).max() < 1e-12
    assert np.abs(oracle.polar(np.eye(3)) - np.eye(3)).max() == 0.0


def test_kocks_round_trip():
    rng = np.random.default_rng(2)
    M = rve.quat_to_matrix(rve.haar_quaternions(50, rng))
    M2 = rve.kocks_matrix(rve.matrix_to_kocks(M))
    assert np.abs(M - M2).max() < 1e-12
    assert np.allclose(np.linalg.det(M2), 1.0)


def test_crystal_setup_rotates_stiffness(oracle):
    """C in the sample frame equals the 4th-order rotation of the crystal stiffness."""
    cr = dict(rve.FCC_VOCE)
    ang = np.array([20.0, 35.0, 70.0])
    C66, ms, qs = oracle.crystal_setup(cr, ang)
    g = rve.kocks_matrix(ang)[0]
    # crystal-frame 4th-order tensor from Voigt (tensor shear on stress, engineering on strain)
    vi = [(0, 0), (1, 1), (2, 2), (0, 1), (1, 2), (0, 2)]
    C0 = np.zeros((6, 6))
    C0[:3, :3] = [[cr["C11"], cr["C12"], cr["C13"]], [cr["C12"], cr["C11"], cr["C13"]],
                  [cr["C13"], cr["C13"], cr["C33"]]]
    C0[3, 3], C0[4, 4], C0[5, 5] = cr["C44"], cr["C55"], cr["C55"]
    C4 = np.zeros((3, 3, 3, 3))
    for a, (i, j) in enumerate(vi):
        for b, (k, l) in enumerate(vi):
            for (p, q) in {(i, j), (j, i)}:
                for (r, s) in {(k, l), (l, k)}:
                    C4[p, q, r, s] = C0[a, b]
    Q = g.T  # crystal -> sample
    C4s = np.einsum("ia,jb,kc,ld,abcd->ijkl", Q, Q, Q, Q, C4)
    Cs = np.array([[C4s[i, j, k, l] for (k, l) in vi] for (i, j) in vi])
    assert np.abs(Cs - C66).max() < 1e-8 * np.abs(C66).max()
    # Schmid tensors: traceless, unit-norm slip direction and normal are orthogonal
    assert np.abs(ms[:, :3].sum(axis=1)).max() < 1e-14


def _voxel(oracle, cr, kocks, step, it, Fn, Fn1, hist=None):
    return oracle.voxel_update(cr, kocks, 1.0, step, it, Fn, Fn1, hist)


def test_cep2A_exact_for_elastic_predictor(oracle):
    """At step 1, iter 0 the stress is C:d with the elastic tangent, so the analytic
    dP/dF of cep2A must equal a central finite difference of P (src/cep2A.f:9-10)."""
    cr = dict(rve.FCC_VOCE)
    rng = np.random.default_rng(3)
    kocks = np.array([30.0, 40.0, 50.0])
    Fn = np.eye(3)
    Fn1 = np.eye(3) + 1e-3 * rng.standard_normal((3, 3))
    r = _voxel(oracle, cr, kocks, 1, 0, Fn, Fn1)
    h = 1e-7
    Afd = np.zeros((9, 9))
    for m in range(9):
        d = np.zeros(9)
        d[m] = h
        Pp = _voxel(oracle, cr, kocks, 1, 0, Fn, Fn1 + d.reshape(3, 3))["P"]
        Pm = _voxel(oracle, cr, kocks, 1, 0, Fn, Fn1 - d.reshape(3, 3))["P"]
        Afd[:, m] = (Pp - Pm) / (2 * h)
    assert np.abs(r["A"] - Afd).max() < 1e-7 * np.abs(Afd).max()


def test_elastic_predictor_golden(oracle):
    """Independent numpy restatement of the kinematics + elastic predictor."""
    cr = dict(rve.FCC_VOCE)
    kocks = np.array([12.0, 55.0, 200.0])
    rng = np.random.default_rng(4)
    Fn = np.eye(3)
    Fn1 = np.eye(3) + 5e-4 * rng.standard_normal((3, 3))
    C66, _, _ = oracle.crystal_setup(cr, kocks)
    Fh = 0.5 * (Fn + Fn1)
    Rh, _ = scipy.linalg.polar(Fh)
    R1, _ = scipy.linalg.polar(Fn1)
    L = (Fn1 - Fn) @ np.linalg.inv(Fh)
    D = 0.5 * (L + L.T)
    d = Rh.T @ D @ Rh
    dv = np.array([d[0, 0], d[1, 1], d[2, 2], 2 * d[0, 1], 2 * d[1, 2], 2 * d[0, 2]])
    s = C66 @ dv
    t = np.array([[s[0], s[3], s[5]], [s[3], s[1], s[4]], [s[5], s[4], s[2]]])
    T = R1 @ t @ R1.T
    P = np.linalg.det(Fn1) * T @ np.linalg.inv(Fn1).T
    r = _voxel(oracle, cr, kocks, 1, 0, Fn, Fn1)
    assert np.abs(r["P"] - P.ravel()).max() < 1e-10 * np.abs(P).max()


@pytest.mark.parametrize("exact", [1, 0])
def test_local_jacobian_against_finite_differences(oracle, exact):
    """The mm10 local Newton converges quadratically with the exact d(R2)/d(tau);
    the reference's extra sign(1, slip increment) factor (src/mm10_b.f:1942-1968)
    costs iterations once slip reverses.  Both settings must reach the same state."""
    cr = dict(rve.FCC_VOCE)
    cr["exact_j22"] = exact
    kocks = np.array([30.0, 40.0, 50.0])
    hist, F0 = None, np.eye(3)
    its = []
    for s in range(1, 9):
        F1 = F0.copy()
        F1[0, 0] += 4e-4
        F1[1, 1] -= 2e-4
        F1[2, 2] -= 2e-4
        r = _voxel(oracle, cr, kocks, s, 1, F0, F1, hist)
        assert r["iters"] >= 0
        its.append(r["iters"])
        hist, F0 = r["hist"], F1
    if exact:
        assert max(its) <= 4
    test_local_jacobian_against_finite_differences.state = getattr(
        test_local_jacobian_against_finite_differences, "state", {})
    test_local_jacobian_against_finite_differences.state[exact] = hist.copy()
    st = test_local_jacobian_against_finite_differences.state
    if len(st) == 2:
        assert np.abs(st[0] - st[1]).max() < 1e-7 * np.abs(st[1]).max()


def _rve(oracle, N, gmap, crystal=None, ngr=3, seed=7):
    r = rve.make_rve(N, ngr, seed, crystal)
    return r, oracle.Oracle(N, r.mat_list, r.kocks, r.crystals, 1.0, gmap, nthreads=4)


@pytest.mark.parametrize("N,gmap", [(7, 0), (8, 1), (9, 1)])
def test_green_operator_is_a_projector(oracle, N, gmap):
    """Ghat annihilates uniform fields and G(G(x)) = G(x) (odd N, and even N with the
    Nyquist-filtered centered mapping)."""
    r, o = _rve(oracle, N, gmap)
    rng = np.random.default_rng(N)
    x = rng.standard_normal((9, N ** 3))
    gx = o.green(x, flgK=False)
    ggx = o.green(gx, flgK=False)
    assert np.abs(ggx - gx).max() < 1e-12 * np.abs(gx).max()
    const = np.ones((9, N ** 3)) * np.arange(1, 10)[:, None]
    assert np.abs(o.green(const, flgK=False)).max() < 1e-12
    o.close()


def test_even_N_reference_mapping_is_not_a_projector(oracle):
    """Even N, reference mapping: the Green operator is applied one frequency bin off
    (q = k - 1) and no longer annihilates the mean (the defect of
    src/FFT_init.f:146-147 with src/FFT_init.f:354-385)."""
    r, o = _rve(oracle, 8, 0)
    const = np.ones((9, 8 ** 3))
    assert np.abs(o.green(const, flgK=False)).max() > 1e-3
    o.close()


def test_homogeneous_crystal_stays_uniform(oracle):
    """A single-orientation RVE under mixed BCs keeps uniform fields, and the averaged
    P equals the one-voxel response under the same F history."""
    cr = dict(rve.FCC_VOCE)
    N = 5
    r = rve.make_rve(N, 1, 3, cr)
    o = oracle.Oracle(N, r.mat_list, r.kocks, r.crystals, 1.0, 0, nthreads=2)
    assert o.nr3_begin(1e-10) == 0
    load = rve.uniaxial_tension(0.01, 10)
    hist = None
    F0 = np.eye(3)
    for s in range(1, 4):
        rc, Pbar, st = o.nr3_step(s, load.BC_all[s - 1], load.isNBC, 1e-6, 1e-10, 20)
        assert rc == 0
        f = o.fields()
        F1 = f["Fn1"][:, 0].reshape(3, 3)
        assert np.abs(f["Fn1"] - f["Fn1"][:, :1]).max() < 1e-9
        v = oracle.voxel_update(cr, r.kocks[:, 0], 1.0, s, 1, F0, F1, hist)
        assert np.abs(v["P"] - Pbar).max() < 1e-6 * np.abs(Pbar).max()
        hist, F0 = v["hist"], F1
        # natural BCs: prescribed-zero P components
        assert np.abs(Pbar[load.isNBC == 1]).max() < 1e-6 * abs(Pbar[0])
    o.close()
