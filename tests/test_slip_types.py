"""The slip types besides fcc and bcc48 (src/incrystal.f:64-83): bcc (2, {110}<111>),
roters (6, the FCC systems in Roters' order) and bcc12 (7, bcc48's first twelve), with 12
systems and so served by the 12-system stress kernels and every hardening law; single
(3, one system), hcp6 (9, basal and prismatic) and hcp18 (10: the reference assigns only
hcp6's six systems and leaves twelve zero vectors), with Voce hardening (the reference's
MRR / ORNL interaction tables exist for the cubic types only, src/mm10_e.f:16-38).

The oracle's tables and interaction matrices against the reference's own
(tests/golden/slip_tables.npz, read from src/mod_crystals.f and src/mm10_e.f by
tests/golden/make_slip_tables.py); the library's refusals; the GPU's stress update and
load steps against the oracle."""
import ctypes
import os

import numpy as np
import pytest

from cpfft_gb300 import rve

GOLDEN = np.load(os.path.join(os.path.dirname(__file__), "golden", "slip_tables.npz"))
KOCKS = np.array([20.0, 35.0, 70.0])
TYPES12 = [1, 2, 6, 7]


def schmid(b, n, kocks):
    """The sample-frame Schmid tensors (Voigt, engineering shear) and spin vectors of the
    systems (b, n) for a crystal at `kocks` (setup_mm10_rknstr, mm10_et2ev / mm10_wt2wv)."""
    tr = rve.kocks_matrix(kocks)[0].T
    bs, ns = b @ tr.T, n @ tr.T
    A = bs[:, :, None] * ns[:, None, :]
    S, W = 0.5 * (A + A.transpose(0, 2, 1)), 0.5 * (A - A.transpose(0, 2, 1))
    ms = np.stack([S[:, 0, 0], S[:, 1, 1], S[:, 2, 2], 2 * S[:, 0, 1], 2 * S[:, 1, 2],
                   2 * S[:, 0, 2]], axis=1)
    qs = np.stack([W[:, 1, 2], W[:, 0, 2], W[:, 0, 1]], axis=1)
    return ms, qs


@pytest.mark.parametrize("slip_type", [1, 2, 3, 6, 7, 8, 9, 10])
def test_oracle_slip_tables_match_the_reference(oracle, slip_type):
    cr = dict(rve.BCC48_DECK if slip_type == 8 else rve.FCC_VOCE, slip_type=slip_type)
    _, ms, qs = oracle.crystal_setup(cr, KOCKS)
    ms_ref, qs_ref = schmid(GOLDEN["b%d" % slip_type], GOLDEN["n%d" % slip_type], KOCKS)
    assert ms.shape == ms_ref.shape
    assert np.abs(ms - ms_ref).max() < 1e-15 and np.abs(qs - qs_ref).max() < 1e-15


@pytest.mark.parametrize("slip_type", [1, 2, 3, 6, 7, 8, 9, 10])
def test_library_slip_tables_match_the_reference(gpulib, slip_type):
    """The tables the library hands its stress kernels (cpfft_slip_systems, host only)
    equal the reference's bit for bit; hcp18 runs as its six assigned systems."""
    b, n = gpulib.slip_systems(slip_type)
    b_ref, n_ref = GOLDEN["b%d" % slip_type], GOLDEN["n%d" % slip_type]
    if slip_type == 10:
        assert not b_ref[6:].any() and not n_ref[6:].any()
        b_ref, n_ref = b_ref[:6], n_ref[:6]
    assert np.array_equal(b, b_ref) and np.array_equal(n, n_ref)


def test_library_slip_tables_refuse_unknown_types(gpulib):
    for bad in (0, 4, 11):
        with pytest.raises(gpulib.CpfftError):
            gpulib.slip_systems(bad)


@pytest.mark.parametrize("slip_type", TYPES12)
def test_oracle_interaction_matches_the_reference(oracle, slip_type):
    """mm10_mrr_GH's table for the slip type equals the geometric forest / parallel
    projections of its systems."""
    G, H = oracle.mrr_interaction(slip_type)
    assert np.abs(G - GOLDEN["G%d" % slip_type]).max() < 1e-15
    assert np.abs(H - GOLDEN["H%d" % slip_type]).max() < 1e-15


def test_library_refuses_mixed_and_unknown_slip_types(gpulib):
    """cpfft_init checks the crystals before any device work."""
    L = gpulib.load_library()
    N = 2
    ml = np.array([1, 2, 1, 2, 1, 2, 1, 2], dtype=np.int32)
    ka = np.zeros(3 * N ** 3)
    P = ctypes.POINTER
    mlp = ml.ctypes.data_as(P(ctypes.c_int))
    kap = ka.ctypes.data_as(P(ctypes.c_double))
    mixed = gpulib.crystal_struct([dict(rve.FCC_VOCE), dict(rve.FCC_VOCE, slip_type=2)])
    assert L.cpfft_init(N, mlp, kap, mixed, 2, 1.0, 0) == -5
    assert b"share the slip type" in L.cpfft_last_error()
    for bad in (4, 5, 11, 12):       # no table (halite, 11, has a keyword but none)
        cr = gpulib.crystal_struct([dict(rve.FCC_VOCE, slip_type=bad)] * 2)
        assert L.cpfft_init(N, mlp, kap, cr, 2, 1.0, 0) == -5, bad
    # MTS and the dislocation-density laws need a 12-system type
    for law, st in ((rve.MRR_FCC, 8), (rve.MRR_FCC, 9), (rve.ORNL_FCC, 3), (rve.MTS_FCC, 10)):
        cr = gpulib.crystal_struct([dict(law, slip_type=st)] * 2)
        assert L.cpfft_init(N, mlp, kap, cr, 2, 1.0, 0) == -5, (law["h_type"], st)


def test_hcp18_is_hcp6_with_twelve_null_systems(oracle):
    """The oracle restates hcp18 with its eighteen systems; the twelve zero vectors add
    exact zeros, so every output equals hcp6's bit for bit (the library runs hcp18 grids
    on the 6-system kernel)."""
    I3 = np.eye(3)
    F0 = I3
    h6 = h18 = None
    for step in (1, 2, 3):
        F1 = F0 + 1.5e-3 * np.array([[1.0, 0.2, 0.0], [0.1, -0.5, 0.3], [0.0, 0.2, -0.5]])
        a = oracle.voxel_update(rve.HCP_VOCE, KOCKS, 1.0, step, 1, F0, F1, h6)
        b = oracle.voxel_update(dict(rve.HCP_VOCE, slip_type=10), KOCKS, 1.0, step, 1, F0, F1,
                                h18)
        assert a["iters"] > 0
        for k in ("P", "A", "hist"):
            assert np.array_equal(a[k], b[k]), (step, k)
        h6, h18, F0 = a["hist"], b["hist"], F1


def hexagonal_rotations():
    """The 12 proper rotations of the hexagonal group about the crystal's c axis (z)."""
    out = []
    for k in range(6):
        t = np.pi / 3 * k
        S = np.array([[np.cos(t), -np.sin(t), 0.0], [np.sin(t), np.cos(t), 0.0], [0, 0, 1.0]])
        out += [S, np.diag([1.0, -1.0, -1.0]) @ S]
    return out


def hex_departure(oracle, cr):
    """Largest relative change of P and dP/dF over two plastic steps when the lattice
    orientation g is replaced by S g, S a hexagonal rotation."""
    g = rve.kocks_matrix(KOCKS)[0]
    I3 = np.eye(3)
    F = I3 + 2e-3 * np.array([[1.0, 0.3, -0.2], [0.1, -0.4, 0.25], [-0.15, 0.2, -0.5]])

    def run(kocks):
        a = oracle.voxel_update(cr, kocks, 1.0, 1, 1, I3, F)
        b = oracle.voxel_update(cr, kocks, 1.0, 2, 1, F, F @ F, a["hist"])
        assert a["iters"] > 0
        return a, b

    a1, a2 = run(KOCKS)
    worst = 0.0
    for S in hexagonal_rotations():
        b1, b2 = run(rve.matrix_to_kocks((S @ g)[None])[0])
        for x, y in ((b1["P"], a1["P"]), (b1["A"], a1["A"]), (b2["P"], a2["P"])):
            worst = max(worst, np.abs(x - y).max() / np.abs(y).max())
    return worst


@pytest.mark.parametrize("slip_type", [9, 10])
def test_hcp_is_hexagonally_symmetric(oracle, slip_type):
    """With transversely isotropic elasticity (C44 = C55 = (C11 - C12) / 2, so that the
    reference's C66 = C55 is the hexagonal value) the basal and prismatic systems make the
    response invariant under the hexagonal rotations, to round-off.  With C55 away from
    (C11 - C12) / 2 the reference's C66 = C55 breaks that symmetry."""
    c11, c12 = rve.HCP_VOCE["C11"], rve.HCP_VOCE["C12"]
    ti = dict(rve.HCP_VOCE, slip_type=slip_type, C44=(c11 - c12) / 2, C55=(c11 - c12) / 2)
    assert hex_departure(oracle, ti) < 1e-13
    assert hex_departure(oracle, dict(rve.HCP_VOCE, slip_type=slip_type)) > 1e-6


def per_voxel_rel(a, b):
    scale = np.maximum(np.abs(b).max(axis=0), 1e-6 * np.abs(b).max())
    return (np.abs(a - b).max(axis=0) / scale).max()


CASES = {"bcc_voce": dict(rve.FCC_VOCE, slip_type=2),
         "roters_voce": dict(rve.FCC_VOCE, slip_type=6),
         "bcc12_voce": dict(rve.FCC_VOCE, slip_type=7),
         "bcc_mrr": dict(rve.MRR_FCC, slip_type=2),
         "bcc12_mts": dict(rve.MTS_FCC, slip_type=7),
         "single_voce": dict(rve.FCC_VOCE, slip_type=3),
         "hcp6_voce": rve.HCP_VOCE,
         "hcp18_voce": dict(rve.HCP_VOCE, slip_type=10)}


@pytest.mark.gpu
@pytest.mark.parametrize("case", sorted(CASES))
def test_gpu_stress_update_parity(gpulib, oracle, case):
    """P and dP/dF per voxel over the passes of two steps, and the history after each."""
    N = 5
    r = rve.make_rve(N, 4, 97, CASES[case])
    s = gpulib.Solver(N, r.mat_list, r.kocks, r.crystals, 1.0, gpulib.G_REF_SHIFT)
    o = oracle.Oracle(N, r.mat_list, r.kocks, r.crystals, 1.0, 0, nthreads=8)
    try:
        rng = np.random.default_rng(9)
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
            assert hg.shape == ho.shape
            for w in range(hg.shape[0]):
                assert np.abs(hg[w] - ho[w]).max() <= 1e-9 * np.abs(ho[w]).max() + 1e-12, w
    finally:
        s.close()
        o.close()


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["bcc_voce", "roters_voce", "hcp6_voce", "hcp18_voce"])
def test_gpu_load_steps(gpulib, oracle, case):
    """Whole load steps (7^3, stretch 1e-3 a step): P_bar and Newton counts."""
    N = 7
    r = rve.make_rve(N, 6, 98, CASES[case])
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
