"""The P_bar update inside the Newton iteration (cpfft_set_coupled_bc, an extension of the
reference's nested loops of src/FFT_nr3.f:75-171): the oracle's coupled steps against its
nested ones, and the GPU's coupled steps against the oracle's."""
import numpy as np
import pytest

from cpfft_gb300 import rve


def run_oracle(oracle, r, load, coupled, steps, N):
    o = oracle.Oracle(N, r.mat_list, r.kocks, r.crystals, 1.0, 0, nthreads=8)
    try:
        o.set_equilibrium_tol(1e-6)
        o.set_coupled_bc(coupled)
        o.nr3_begin(1e-10)
        out = []
        for step in range(1, steps + 1):
            rc, Pb, st = o.nr3_step(step, load.BC_all[step - 1], load.isNBC, 1e-6, 1e-10, 30)
            assert rc == 0, (coupled, step, rc)
            out.append((Pb, st))
        return out
    finally:
        o.close()


LOADS = {"plane_strain": lambda: rve.plane_strain_compression(0.10, 100),
         "uniaxial": lambda: rve.uniaxial_tension(0.02, 20)}


@pytest.mark.parametrize("loading", sorted(LOADS))
@pytest.mark.parametrize("mode", [1, 2])
def test_oracle_coupled_against_nested(oracle, mode, loading):
    """9^3, 3 steps of plane-strain compression (two prescribed stresses) or uniaxial
    tension (eight): both reach P_bar within tolNR of the prescribed stresses and the
    equilibrium tolerance; the coupled iteration takes fewer stress passes (mode 2, its
    first stress pass implicit: at most half; uniaxial step 2 takes 5 against 18, mode 1
    11), and the two P_bar agree within the tolerance they share."""
    N = 9
    r = rve.make_rve(N, 8, 3, rve.FCC_VOCE)
    load = LOADS[loading]()
    nested = run_oracle(oracle, r, load, 0, 3, N)
    coupled = run_oracle(oracle, r, load, mode, 3, N)
    for (Pn, sn), (Pc, sc) in zip(nested, coupled):
        assert sc["res_equil"] <= 1e-6 and sc["res_pbar"] <= 1e-6
        if mode == 2:
            assert sc["stress_updates"] * 2 <= sn["stress_updates"]
        else:
            assert sc["stress_updates"] < sn["stress_updates"]
        assert np.abs(Pc - Pn).max() < 1e-6 * np.abs(Pn).max()


@pytest.mark.gpu
@pytest.mark.parametrize("mode", [1, 2])
def test_gpu_coupled_fp64_against_oracle(gpulib, oracle, mode):
    """The GPU's coupled steps in the plain FP64 form (FP64 CG to 1e-10) against the
    oracle's: P_bar to 1e-10, the same Newton and stress-pass counts."""
    N = 9
    r = rve.make_rve(N, 8, 3, rve.FCC_VOCE)
    load = rve.plane_strain_compression(0.10, 100)
    ref = run_oracle(oracle, r, load, mode, 3, N)
    s = gpulib.Solver(N, r.mat_list, r.kocks, r.crystals, 1.0, gpulib.G_REF_SHIFT)
    try:
        s.set_equilibrium_tol(1e-6)
        s.set_coupled_bc(mode)
        s.nr3_begin(1e-10)
        for step, (Po, so) in enumerate(ref, start=1):
            rc, Pb, st = s.nr3_step(step, load.BC_all[step - 1], load.isNBC, 1e-6, 1e-10, 30)
            assert rc == 0
            assert np.abs(Pb - Po).max() < 1e-10 * np.abs(Po).max(), step
            assert st["newton_iters"] == so["newton_iters"]
            assert st["stress_updates"] == so["stress_updates"]
    finally:
        s.close()


@pytest.mark.gpu
def test_gpu_coupled_fast_form(gpulib, oracle):
    """The fast form (FP32 inner Krylov, inexact Newton, coupled P_bar update) on a 16^3
    plane-strain workload against the oracle's nested FP64 loops: P_bar within 1e-6, the
    equilibrium residual within 1e-6."""
    N = 16
    r = rve.make_rve(N, 8, 3, rve.FCC_VOCE)
    load = rve.plane_strain_compression(0.10, 100)
    o = oracle.Oracle(N, r.mat_list, r.kocks, r.crystals, 1.0, 1, nthreads=8)
    s = gpulib.Solver(N, r.mat_list, r.kocks, r.crystals, 1.0, gpulib.G_CENTERED,
                      gpulib.PREC_MIXED)
    try:
        o.set_equilibrium_tol(1e-6)
        o.nr3_begin(1e-10)
        s.set_mode(gpulib.PREC_MIXED, gpulib.START_TRIAL | gpulib.START_ITERATE |
                   gpulib.TANGENT_F32)
        s.set_precond(gpulib.PRECOND_REFERENCE)
        s.set_schedule(gpulib.SCHED_QUEUE)
        s.set_equilibrium_tol(1e-6)
        s.set_inexact_newton(1e-2)
        s.set_coupled_bc(2)
        s.nr3_begin(1e-10)
        for step in (1, 2, 3):
            rco, Po, so = o.nr3_step(step, load.BC_all[step - 1], load.isNBC, 1e-6, 1e-10, 30)
            rc, Pb, st = s.nr3_step(step, load.BC_all[step - 1], load.isNBC, 1e-6, 1e-10, 30)
            assert rc == 0 and rco == 0
            assert st["res_equil"] <= 1e-6
            assert np.abs(Pb - Po).max() < 1e-6 * np.abs(Po).max(), step
            assert st["stress_updates"] < so["stress_updates"]
    finally:
        s.close()
        o.close()
