"""GPU parity: every entry point of the C-ABI against the CPU oracle on the same seeded
inputs.  Tolerances: per-voxel P, dP/dF and history within 1e-8 relative (FP64 stress
update); the Green operator within 1e-11 relative; CG solutions within the CG
tolerance; load-step P_bar within 1e-10 relative of the oracle (the plain FP64 form)."""
import numpy as np
import pytest

from cpfft_gb300 import rve

pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def per_voxel_rel(a, b):
    """max over voxels of |a - b|_inf / max(|b|_inf, floor) per voxel."""
    scale = np.maximum(np.abs(b).max(axis=0), 1e-6 * np.abs(b).max())
    return (np.abs(a - b).max(axis=0) / scale).max()


def make_pair(gpulib, oracle, N, ngr=4, seed=11, gmap=0, crystal=None, precision=0):
    r = rve.make_rve(N, ngr, seed, crystal)
    s = gpulib.Solver(N, r.mat_list, r.kocks, r.crystals, 1.0, gmap, precision)
    o = oracle.Oracle(N, r.mat_list, r.kocks, r.crystals, 1.0, gmap, nthreads=8)
    return r, s, o


def random_F(N, amp, seed):
    rng = np.random.default_rng(seed)
    Fn = np.zeros((9, N ** 3))
    Fn[[0, 4, 8]] = 1.0
    Fn1 = Fn + amp * rng.standard_normal((9, N ** 3))
    return Fn, Fn1


@pytest.mark.parametrize("exact", [1, 0])
def test_stress_update_parity(gpulib, oracle, exact):
    cr = dict(rve.FCC_VOCE)
    cr["exact_j22"] = exact
    N = 8
    r, s, o = make_pair(gpulib, oracle, N, crystal=cr)
    try:
        Fn, Fn1 = random_F(N, 4e-4, 1)
        for it in (0, 1, 2):
            P, K, rc = s.drive_eps_sig(1, it, Fn, Fn1, want_K4=True)
            Po, Ko, fails, _ = o.stress_update(1, it, Fn, Fn1)
            # with the reference's d(R2)/d(tau) a few random-shear voxels exhaust miter;
            # both sides then keep sigma_n and the elastic tangent and report it
            assert rc == (1 if fails else 0)
            if exact:
                assert fails == 0
            assert per_voxel_rel(P, Po) < 1e-8
            assert per_voxel_rel(K, Ko) < 1e-8
        # a second step on top of the committed history
        s.commit()
        o.commit()
        Fn2 = Fn1 + (Fn1 - Fn)
        for it in (0, 1):
            P, K, rc = s.drive_eps_sig(2, it, Fn1, Fn2, want_K4=True)
            Po, Ko, fails, _ = o.stress_update(2, it, Fn1, Fn2)
            assert rc == (1 if fails else 0)
            assert per_voxel_rel(P, Po) < 1e-8
            assert per_voxel_rel(K, Ko) < 1e-8
        _, _, H = s.fields(history=True)
        Ho, Ho1 = o.history()
        assert per_voxel_rel(H, Ho) < 1e-8
    finally:
        s.close()
        o.close()


@pytest.mark.parametrize("N,gmap", [(5, 0), (7, 0), (8, 1), (9, 0), (12, 1), (15, 0), (16, 1),
                                    (16, 0), (32, 1), (32, 0), (64, 1), (128, 1)])
def test_green_parity(gpulib, oracle, N, gmap):
    """Sizes 32-256 that are powers of two run the warp-FFT passes, the others the
    shared-memory Stockham passes."""
    r, s, o = make_pair(gpulib, oracle, N, gmap=gmap)
    try:
        Fn, Fn1 = random_F(N, 1e-3, 2)
        _, K, _ = s.drive_eps_sig(1, 0, Fn, Fn1, want_P=False, want_K4=True)
        rng = np.random.default_rng(N)
        x = rng.standard_normal((9, N ** 3))
        for flgK in (True, False):
            y = s.G_K_dF(x, flgK)
            yo = o.green(x, flgK, K4=K)
            assert rel(y, yo) < 1e-11, (flgK, rel(y, yo))
    finally:
        s.close()
        o.close()


@pytest.mark.parametrize("precision,precond", [(0, 0), (1, 0), (1, 1)])
def test_cg_parity(gpulib, oracle, precision, precond):
    N = 9
    r, s, o = make_pair(gpulib, oracle, N, precision=precision)
    if precond:
        s.set_precond(gpulib.PRECOND_REFERENCE)
    try:
        Fn, Fn1 = random_F(N, 1e-3, 3)
        _, K, _ = s.drive_eps_sig(1, 1, Fn, Fn1, want_P=False, want_K4=True)
        o.stress_update(1, 1, Fn, Fn1)
        b = -o.green(np.ones((9, N ** 3)) * 1e-3, True)
        x, its = s.fftPcg(b, 1e-10)
        xo, itso, rc = o.cg(b, 1e-10)
        assert rc == 0
        # both meet ||r|| <= 1e-10 ||b|| and stay in the range of G; the solutions agree
        # to that tolerance times the operator's conditioning
        assert rel(x, xo) < 1e-7, rel(x, xo)
        res = o.green(x, True) - b
        assert np.linalg.norm(res) <= 1.5e-10 * np.linalg.norm(b)
        if precision == 0:
            assert abs(its - itso) <= 2
    finally:
        s.close()
        o.close()


def test_tangent_homo_parity(gpulib, oracle):
    N = 7
    r, s, o = make_pair(gpulib, oracle, N)
    try:
        s.nr3_begin(1e-10)
        o.nr3_begin(1e-10)
        C = s.tangent_homo(1e-10)
        Co, rc = o.tangent_homo(1e-10)
        assert rc >= 0
        assert rel(C, Co) < 1e-9
    finally:
        s.close()
        o.close()


@pytest.mark.parametrize("case", ["fcc_voce_odd", "faithful_j22", "even_centered", "mixed",
                                  "mixed_precond", "mixed_fast", "equilibrium",
                                  "mixed_fast_equilibrium"])
def test_load_step_parity(gpulib, oracle, case):
    cr = dict(rve.FCC_VOCE)
    N, gmap, inc, nsteps, precision, tolP = 9, 0, 1e-3, 3, 0, 1e-10
    if case == "faithful_j22":
        cr["exact_j22"] = 0
        inc = 2.5e-4
    elif case == "even_centered":
        N, gmap, nsteps = 8, 1, 2
    elif case in ("mixed", "mixed_precond", "mixed_fast", "mixed_fast_equilibrium"):
        precision, tolP = 1, 1e-6
    r, s, o = make_pair(gpulib, oracle, N, ngr=4, seed=21, gmap=gmap, crystal=cr,
                        precision=precision)
    if case in ("mixed_precond", "mixed_fast", "mixed_fast_equilibrium"):
        s.set_precond(gpulib.PRECOND_REFERENCE)
    # the equilibrium stop test (both sides): tight enough to add Newton iterations
    eq_tol = 1e-8 if case.endswith("equilibrium") else 0.0
    if eq_tol:
        s.set_equilibrium_tol(eq_tol)
        o.set_equilibrium_tol(eq_tol)
    if case.startswith("mixed_fast"):  # the fast local starts and FP32 tangent too
        s.set_mode(gpulib.PREC_MIXED, gpulib.START_ITERATE | gpulib.START_TRIAL |
                   gpulib.TANGENT_F32)
        s.set_schedule(gpulib.SCHED_QUEUE)
    load = rve.uniaxial_tension(inc * 20, 20)
    try:
        s.nr3_begin(1e-10)
        o.nr3_begin(1e-10)
        for step in range(1, nsteps + 1):
            rc, Pbar, st = s.nr3_step(step, load.BC_all[step - 1], load.isNBC, 1e-6, 1e-10, 20)
            rco, Pbo, sto = o.nr3_step(step, load.BC_all[step - 1], load.isNBC, 1e-6, 1e-10, 20)
            assert rc == 0 and rco == 0
            assert rel(Pbar, Pbo) < tolP, (step, rel(Pbar, Pbo))
            if eq_tol:
                assert st["res_equil"] <= eq_tol and sto["res_equil"] <= eq_tol
            if precision == 0:
                assert st["newton_iters"] == sto["newton_iters"]
                assert st["nbc_iters"] == sto["nbc_iters"]
        F, P = s.fields()
        fo = o.fields()
        assert per_voxel_rel(P, fo["Pn1"]) < (1e-8 if precision == 0 else 1e-5)
        assert rel(F, fo["Fn1"]) < (1e-9 if precision == 0 else 1e-6)
    finally:
        s.close()
        o.close()


@pytest.mark.parametrize("N", [32, 64, 128, 256])
def test_green_fp32_warp_path(gpulib, N):
    """The FP32 register-FFT passes (powers of two 32-256) against the FP64 operator on the
    same tangent: agreement to FP32 rounding of an N^3 transform."""
    r = rve.make_rve(N, 8, 13)
    s = gpulib.Solver(N, r.mat_list, r.kocks, r.crystals, 1.0, gpulib.G_CENTERED,
                      gpulib.PREC_MIXED)
    try:
        Fn, Fn1 = random_F(N, 1e-3, 4)
        s.drive_eps_sig(1, 0, Fn, Fn1, want_P=False)
        x = np.random.default_rng(N).standard_normal((9, N ** 3))
        for flgK in (True, False):
            y64 = s.G_K_dF(x, flgK)
            y32 = s.G_K_dF_f32(x.astype(np.float32), flgK)
            assert rel(y32, y64) < 1e-5, (flgK, rel(y32, y64))
    finally:
        s.close()


@pytest.mark.parametrize("N", [32, 64, 128])
def test_precond_cg_warp_path(gpulib, N):
    """Reference-medium preconditioned mixed CG on the warp-FFT sizes: the solution of the
    plain FP64 CG (itself checked against the oracle above) to the CG tolerance, the
    reference's stop test met on the FP64 residual, in fewer FP32 iterations than the
    unpreconditioned mixed CG on the same system."""
    r = rve.make_rve(N, 8, 17)
    s = gpulib.Solver(N, r.mat_list, r.kocks, r.crystals, 1.0, gpulib.G_CENTERED)
    try:
        Fn, Fn1 = random_F(N, 2e-3, 5)
        s.drive_eps_sig(1, 1, Fn, Fn1, want_P=False)
        b = -s.G_K_dF(np.ones((9, N ** 3)) * 1e-3, True)
        x64, it64 = s.fftPcg(b, 1e-10)
        s.set_mode(gpulib.PREC_MIXED)
        s.drive_eps_sig(1, 1, Fn, Fn1, want_P=False)  # the FP32 tangent
        xm, itm = s.fftPcg(b, 1e-10)
        s.set_precond(gpulib.PRECOND_REFERENCE)
        xp, itp = s.fftPcg(b, 1e-10)
        for x in (xm, xp):
            assert rel(x, x64) < 1e-7, rel(x, x64)
            res = s.G_K_dF(x, True) - b
            assert np.linalg.norm(res) <= 1.5e-10 * np.linalg.norm(b)
        assert itp < itm, (itp, itm, it64)
    finally:
        s.close()


@pytest.mark.parametrize("N", [32, 64, 128, 256])
@pytest.mark.parametrize("tc", [2, 4, -2, -4])
def test_green_fp32_tile_shapes(gpulib, N, tc):
    """Every tile shape of the FP32 register passes the autotuner chooses from, pinned with
    cpfft_set_tiles: the shared-memory slowest-axis pass (tc > 0) and the one holding each
    column's rows in registers (tc < 0), against the FP64 operator on the same tangent."""
    r = rve.make_rve(N, 8, 13)
    s = gpulib.Solver(N, r.mat_list, r.kocks, r.crystals, 1.0, gpulib.G_CENTERED,
                      gpulib.PREC_MIXED)
    try:
        Fn, Fn1 = random_F(N, 1e-3, 4)
        s.drive_eps_sig(1, 0, Fn, Fn1, want_P=False)
        s.set_tiles(16, tc)
        assert s.tuning()["fp32_tiles"] == [16, tc]
        x = np.random.default_rng(N).standard_normal((9, N ** 3))
        for flgK in (True, False):
            y64 = s.G_K_dF(x, flgK)
            y32 = s.G_K_dF_f32(x.astype(np.float32), flgK)
            assert rel(y32, y64) < 1e-5, (flgK, rel(y32, y64))
    finally:
        s.close()


@pytest.mark.parametrize("tc", [4, -2, -4])
@pytest.mark.parametrize("N", [32, 64, 128])
def test_precond_cg_tile_shapes(gpulib, N, tc):
    """The reference-medium operator (it couples a column's rows) through each slowest-axis
    pass: the preconditioned mixed CG reaches the plain FP64 CG's solution."""
    r = rve.make_rve(N, 8, 17)
    s = gpulib.Solver(N, r.mat_list, r.kocks, r.crystals, 1.0, gpulib.G_CENTERED)
    try:
        Fn, Fn1 = random_F(N, 2e-3, 5)
        s.drive_eps_sig(1, 1, Fn, Fn1, want_P=False)
        b = -s.G_K_dF(np.ones((9, N ** 3)) * 1e-3, True)
        x64, _ = s.fftPcg(b, 1e-10)
        s.set_mode(gpulib.PREC_MIXED)
        s.set_tiles(16, tc)
        s.drive_eps_sig(1, 1, Fn, Fn1, want_P=False)
        s.set_precond(gpulib.PRECOND_REFERENCE)
        xp, _ = s.fftPcg(b, 1e-10)
        assert rel(xp, x64) < 1e-7, rel(xp, x64)
        res = s.G_K_dF(xp, True) - b
        assert np.linalg.norm(res) <= 1.5e-10 * np.linalg.norm(b)
    finally:
        s.close()


def test_queue_chunk_autotuned(gpulib):
    """The voxel-queue chunk and persistent blocks per SM are chosen on the first implicit
    queue pass from timed runs of that pass, and the results equal those of the
    one-block-per-128-voxels schedule."""
    N = 16
    r = rve.make_rve(N, 4, 29)
    Fn, Fn1 = random_F(N, 1e-3, 6)
    out = []
    for sched in (gpulib.SCHED_BLOCKS, gpulib.SCHED_QUEUE):
        s = gpulib.Solver(N, r.mat_list, r.kocks, r.crystals, 1.0, gpulib.G_CENTERED,
                          gpulib.PREC_MIXED)
        try:
            s.set_mode(gpulib.PREC_MIXED, gpulib.START_TRIAL)
            s.set_schedule(sched)
            assert s.queue_chunk()["chunk"] == 0
            P, K, _ = s.drive_eps_sig(1, 1, Fn, Fn1, want_K4=True)
            q = s.queue_chunk()
            if sched == gpulib.SCHED_QUEUE:
                assert q["chunk"] in (128, 256, 512) and q["blocks_per_sm"] in ("all", 1)
                assert all(t > 0 for t in q["ms_128_256_512"] + q["ms_one_block_per_sm"])
            out.append((P, K))
        finally:
            s.close()
    assert np.array_equal(out[0][0], out[1][0]) and np.array_equal(out[0][1], out[1][1])


@pytest.mark.parametrize("N", [32, 64, 128])
def test_green_double_float(gpulib, N):
    """The double-float operator of mixed precision against the native FP64 operator on the
    same tangent: FP64 accuracy (well inside the 1e-10 CG tolerance it serves)."""
    r = rve.make_rve(N, 8, 13)
    s = gpulib.Solver(N, r.mat_list, r.kocks, r.crystals, 1.0, gpulib.G_CENTERED,
                      gpulib.PREC_MIXED)
    try:
        Fn, Fn1 = random_F(N, 1e-3, 4)
        s.drive_eps_sig(1, 1, Fn, Fn1, want_P=False)
        x = np.random.default_rng(N).standard_normal((9, N ** 3))
        for flgK in (True, False):
            y64 = s.G_K_dF(x, flgK)
            ydf = s.G_K_dF_df(x, flgK)
            assert rel(ydf, y64) < 1e-12, (flgK, rel(ydf, y64))
    finally:
        s.close()


def test_inexact_newton_vs_fp64_32(gpulib):
    """Inexact Newton in the fast form (Eisenstat-Walker forcing, eta_max 1e-2) under the
    equilibrium test, against the plain FP64 form with every system solved to 1e-10: both
    meet the equilibrium tolerance, P_bar agrees to 1e-7, and the fast form needs fewer
    Krylov iterations."""
    N = 32
    r = rve.make_rve(N, 8, 23)
    load = rve.uniaxial_tension(0.02, 20)
    out = []
    for fast in (False, True):
        s = gpulib.Solver(N, r.mat_list, r.kocks, r.crystals, 1.0, gpulib.G_CENTERED,
                          gpulib.PREC_MIXED if fast else gpulib.PREC_FP64)
        try:
            s.set_equilibrium_tol(1e-7)
            if fast:
                s.set_mode(gpulib.PREC_MIXED, gpulib.START_ITERATE | gpulib.START_TRIAL |
                           gpulib.TANGENT_F32)
                s.set_precond(gpulib.PRECOND_REFERENCE)
                s.set_inexact_newton(1e-2)
            s.nr3_begin(1e-10)
            pb, cg = [], 0
            for step in (1, 2, 3):
                rc, Pbar, st = s.nr3_step(step, load.BC_all[step - 1], load.isNBC, 1e-6, 1e-10,
                                          30)
                assert rc >= 0 and st["res_equil"] <= 1e-7
                pb.append(Pbar)
                cg += st["cg_iters"]
            out.append((np.array(pb), cg))
        finally:
            s.close()
    (p64, cg64), (pfast, cgfast) = out
    assert rel(pfast, p64) < 1e-7, rel(pfast, p64)
    assert cgfast < cg64


def test_mixed_fast_vs_fp64_32(gpulib):
    """The fast form at a warp-FFT size (FP32 inner CG with the reference-medium
    preconditioner, double-float outer residuals, iterate + trial local starts, FP32
    tangent, voxel-queue stress passes) against the
    plain FP64 form (itself checked against the oracle above) on the same 32^3 RVE: P_bar
    within 1e-6 relative, per-voxel P within 1e-5, the same global iteration counts."""
    N = 32
    r = rve.make_rve(N, 8, 23)
    load = rve.uniaxial_tension(0.02, 20)
    out = []
    for fast in (False, True):
        s = gpulib.Solver(N, r.mat_list, r.kocks, r.crystals, 1.0, gpulib.G_CENTERED,
                          gpulib.PREC_MIXED if fast else gpulib.PREC_FP64)
        try:
            if fast:
                s.set_mode(gpulib.PREC_MIXED, gpulib.START_ITERATE | gpulib.START_TRIAL |
                           gpulib.TANGENT_F32)
                s.set_precond(gpulib.PRECOND_REFERENCE)
                s.set_schedule(gpulib.SCHED_QUEUE)
            s.nr3_begin(1e-10)
            pb, its = [], []
            for step in range(1, 4):
                rc, Pbar, st = s.nr3_step(step, load.BC_all[step - 1], load.isNBC, 1e-6, 1e-10, 20)
                assert rc == 0
                pb.append(Pbar)
                its.append((st["newton_iters"], st["nbc_iters"]))
            F, P = s.fields()
            out.append((np.array(pb), its, P))
        finally:
            s.close()
    (pb0, it0, P0), (pb1, it1, P1) = out
    assert rel(pb1, pb0) < 1e-6, rel(pb1, pb0)
    assert per_voxel_rel(P1, P0) < 1e-5
    assert it1 == it0


def test_voxel_queue_schedule_is_exact(gpulib):
    """The persistent kernel's cost-sorted voxel queue computes every voxel exactly as the
    in-order blocks do: identical fields and iteration counts after load steps."""
    N = 16
    r = rve.make_rve(N, 8, 29)
    load = rve.uniaxial_tension(0.02, 20)
    out = []
    for sched in (gpulib.SCHED_BLOCKS, gpulib.SCHED_QUEUE):
        s = gpulib.Solver(N, r.mat_list, r.kocks, r.crystals, 1.0, gpulib.G_CENTERED,
                          gpulib.PREC_MIXED)
        try:
            s.set_mode(gpulib.PREC_MIXED, gpulib.START_ITERATE | gpulib.START_TRIAL)
            s.set_precond(gpulib.PRECOND_REFERENCE)
            s.set_schedule(sched)
            s.nr3_begin(1e-10)
            its = []
            for step in range(1, 4):
                rc, Pbar, st = s.nr3_step(step, load.BC_all[step - 1], load.isNBC, 1e-6, 1e-10, 20)
                assert rc == 0
                its.append((st["newton_iters"], st["cg_iters"], st["local_iters"]))
            F, P, H = s.fields(history=True)
            out.append((F, P, H, its))
        finally:
            s.close()
    (F0, P0, H0, i0), (F1, P1, H1, i1) = out
    assert i0 == i1
    assert np.array_equal(P0, P1) and np.array_equal(F0, F1) and np.array_equal(H0, H1)
