"""Failure detection: where the reference stops the job (die_abort, src/mpi_code.f:35-53)
the library returns a status code, and a context stays usable after a refused call.

The faults are made on the host: an iteration cap that the loop cannot meet (the Newton
loop's maxIter, src/FFT_nr3.f:116-119) and a CG tolerance outside (eps, 1) (fftPcg's
"improper CG tolerance", src/FFT_nr3.f:248-251).  Every loop involved is bounded and
every error is a returned code; nothing here can fault, trap or hang a GPU."""
import numpy as np
import pytest

from cpfft_gb300 import rve

NEWTON_MAXIT, CG_TOL = -2, -8


def workload(N=7):
    r = rve.make_rve(N, 4, 5)
    return r, rve.uniaxial_tension(0.02, 20)


@pytest.mark.parametrize("max_iter", [1, 3])
def test_oracle_newton_cap(oracle, max_iter):
    """The 7^3 uniaxial-tension step 1 needs more than three Newton iterations."""
    r, load = workload()
    o = oracle.Oracle(7, r.mat_list, r.kocks, r.crystals, 1.0, 0, nthreads=8)
    try:
        o.nr3_begin(1e-10)
        rc, _, _ = o.nr3_step(1, load.BC_all[0], load.isNBC, 1e-6, 1e-10, max_iter)
        assert rc == NEWTON_MAXIT
    finally:
        o.close()


def test_oracle_cg_tolerance_out_of_range(oracle):
    r, _ = workload(5)
    o = oracle.Oracle(5, r.mat_list, r.kocks, r.crystals, 1.0, 0, nthreads=8)
    try:
        b = -o.green(np.ones((9, 125)) * 1e-3, True)
        for tol in (0.0, 1e-17, 1.0, 2.0):
            assert o.cg(b, tol)[2] == CG_TOL, tol
    finally:
        o.close()


@pytest.mark.gpu
@pytest.mark.parametrize("max_iter", [1, 3])
def test_gpu_newton_cap(gpulib, max_iter):
    r, load = workload()
    s = gpulib.Solver(7, r.mat_list, r.kocks, r.crystals, 1.0, gpulib.G_REF_SHIFT)
    try:
        s.nr3_begin(1e-10)
        with pytest.raises(gpulib.CpfftError) as err:
            s.nr3_step(1, load.BC_all[0], load.isNBC, 1e-6, 1e-10, max_iter)
        assert err.value.code == NEWTON_MAXIT
        assert "does not converge" in str(err.value)
    finally:
        s.close()


@pytest.mark.gpu
def test_gpu_cg_tolerance_out_of_range_then_usable(gpulib, oracle):
    """Refused tolerances return CPFFT_ERR_CG_TOL; the same context then solves to 1e-10
    and agrees with the oracle."""
    N = 9
    r = rve.make_rve(N, 3, 7)
    s = gpulib.Solver(N, r.mat_list, r.kocks, r.crystals, 1.0, gpulib.G_REF_SHIFT)
    o = oracle.Oracle(N, r.mat_list, r.kocks, r.crystals, 1.0, 0, nthreads=8)
    try:
        rng = np.random.default_rng(3)
        Fn = np.zeros((9, N ** 3))
        Fn[[0, 4, 8]] = 1.0
        Fn1 = Fn + 1e-3 * rng.standard_normal((9, N ** 3))
        s.drive_eps_sig(1, 1, Fn, Fn1, want_P=False, want_K4=True)
        o.stress_update(1, 1, Fn, Fn1)
        b = -o.green(np.ones((9, N ** 3)) * 1e-3, True)
        for tol in (0.0, 1.0):
            with pytest.raises(gpulib.CpfftError) as err:
                s.fftPcg(b, tol)
            assert err.value.code == CG_TOL, tol
        x, _ = s.fftPcg(b, 1e-10)
        xo, _, rc = o.cg(b, 1e-10)
        assert rc == 0
        assert np.abs(x - xo).max() < 1e-7 * np.abs(xo).max()
    finally:
        s.close()
        o.close()
