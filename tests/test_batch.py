"""Many RVEs at once (cpfft_batch_solve): several contexts, each on its own CUDA stream,
driven by worker threads over a largest-first queue.  Each RVE's results must equal a
solve of that RVE on its own (every reduction and transform has a fixed order, so the
match is exact), for the plain FP64 form and the fast mixed form, with RVEs of different
grid sizes (odd / even, Stockham / register-FFT sizes) in one batch."""
import numpy as np
import pytest

from cpfft_gb300 import rve

pytestmark = pytest.mark.gpu


def rves(specs, nsteps):
    out = []
    for N, ngr, seed, gmap in specs:
        r = rve.make_rve(N, ngr, seed)
        load = rve.uniaxial_tension(0.02, 20)
        out.append(dict(N=N, mat_list=r.mat_list, kocks=r.kocks, crystals=r.crystals, tstep=1.0,
                        g_mapping=gmap, BC_all=load.BC_all, isNBC=load.isNBC, nsteps=nsteps))
    return out


def solo(gpulib, d, precision, options, precond, schedule, newton=None):
    s = gpulib.Solver(d["N"], d["mat_list"], d["kocks"], d["crystals"], 1.0, d["g_mapping"],
                      precision)
    try:
        for m, p in (d.get("mises") or {}).items():
            s.set_mises(m, **p)
        s.set_mode(precision, options)
        if precision == gpulib.PREC_MIXED:
            s.set_precond(precond)
            s.set_schedule(schedule)
        if newton:
            s.set_equilibrium_tol(newton["equilibrium_tol"])
            s.set_inexact_newton(newton["eta_max"])
            s.set_tangent_tol(newton["tangent_tol"])
            s.set_coupled_bc(newton["coupled_bc"])
        s.nr3_begin(1e-10)
        pb = []
        for step in range(1, d["nsteps"] + 1):
            rc, Pbar, _ = s.nr3_step(step, d["BC_all"][step - 1], d["isNBC"], 1e-6, 1e-10, 20)
            assert rc >= 0
            pb.append(Pbar)
        F, P = s.fields()
        return np.array(pb), F, P
    finally:
        s.close()


# the fast form's Newton options (cpfft_newton)
FAST_NEWTON = dict(equilibrium_tol=1e-6, eta_max=1e-2, tangent_tol=1e-2, coupled_bc=2)


@pytest.mark.parametrize("form", ["fp64", "fast", "fast_newton"])
def test_batch_equals_solo(gpulib, form):
    """fast_newton adds the equilibrium test, inexact Newton and the coupled P_bar update
    (cpfft_batch_solve_newton) to the fast form."""
    specs = [(9, 4, 41, gpulib.G_REF_SHIFT), (8, 3, 42, gpulib.G_CENTERED),
             (16, 6, 43, gpulib.G_CENTERED), (32, 8, 44, gpulib.G_CENTERED),
             (7, 3, 45, gpulib.G_REF_SHIFT)]
    newton = FAST_NEWTON if form == "fast_newton" else None
    if form == "fp64":
        prec, opts = gpulib.PREC_FP64, 0
    else:
        prec = gpulib.PREC_MIXED
        opts = gpulib.START_ITERATE | gpulib.START_TRIAL | gpulib.TANGENT_F32
    batch = rves(specs, 2)
    res = gpulib.batch_solve(batch, precision=prec, options=opts,
                             precond=gpulib.PRECOND_REFERENCE, schedule=gpulib.SCHED_QUEUE,
                             tolNR=1e-6, nthreads=3, want_fields=True, newton=newton)
    for d, r in zip(batch, res):
        assert r["status"] >= 0 and r["steps_done"] == 2, r["error"]
        assert r["voxel_updates"] > 0
        pb, F, P = solo(gpulib, d, prec, opts, gpulib.PRECOND_REFERENCE, gpulib.SCHED_QUEUE,
                        newton)
        assert np.array_equal(r["Pbar"], pb), (d["N"], np.abs(r["Pbar"] - pb).max())
        assert np.array_equal(r["F"], F) and np.array_equal(r["P"], P), d["N"]


def test_batch_reports_errors(gpulib):
    d = rves([(8, 3, 46, gpulib.G_CENTERED)], 1)
    d[0]["crystals"] = [dict(d[0]["crystals"][0], slip_type=11)]  # halite: cpfft_init refuses
    with pytest.raises(gpulib.CpfftError):
        gpulib.batch_solve(d, precision=gpulib.PREC_FP64, nthreads=1)


def test_batch_other_material_models(gpulib):
    """A batch mixing an MTS-hardened grid and a grid of bilinear Mises (mm01) materials
    with a crystal: each equals its solo solve."""
    batch = []
    r = rve.make_rve(9, 4, 47, rve.MTS_FCC)
    load = rve.uniaxial_tension(0.02, 20)
    batch.append(dict(N=9, mat_list=r.mat_list, kocks=r.kocks, crystals=r.crystals, tstep=1.0,
                      g_mapping=gpulib.G_REF_SHIFT, BC_all=load.BC_all, isNBC=load.isNBC,
                      nsteps=2))
    r = rve.make_rve(8, 3, 48)
    mat = np.random.default_rng(48).integers(1, 4, 8 ** 3).astype(np.int32)
    batch.append(dict(N=8, mat_list=mat, kocks=r.kocks,
                      crystals=[r.crystals[0], rve.NOT_A_CRYSTAL, rve.NOT_A_CRYSTAL], tstep=1.0,
                      g_mapping=gpulib.G_CENTERED, BC_all=load.BC_all, isNBC=load.isNBC,
                      nsteps=2, mises={2: rve.MM01_DECK[0], 3: rve.MM01_DECK[1]}))
    res = gpulib.batch_solve(batch, precision=gpulib.PREC_FP64, tolNR=1e-6, nthreads=2,
                             want_fields=True)
    for d, r in zip(batch, res):
        assert r["status"] >= 0 and r["steps_done"] == 2, r["error"]
        pb, F, P = solo(gpulib, d, gpulib.PREC_FP64, 0, gpulib.PRECOND_REFERENCE,
                        gpulib.SCHED_QUEUE)
        assert np.array_equal(r["Pbar"], pb), (d["N"], np.abs(r["Pbar"] - pb).max())
        assert np.array_equal(r["P"], P), d["N"]
