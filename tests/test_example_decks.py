"""The reference's two example decks, as shipped (extracted by
tests/golden/make_example_decks.py into tests/golden/mm01_deck.npz and mm10_deck.npz,
with the oracle's results over all ten load steps):

  examples/test_mm01.in            7^3, two bilinear Mises materials (mm01);
  examples/test_mm10.in + angle_bc.in   7^3 BCC-48 bicrystal (0 and 45 degrees), Voce.

Both: F_xx 0.03 / F_yy -0.01 / F_zz -0.01 (test_mm10) or 0.3 / -0.1 / -0.1 (test_mm01)
per unit, constraints 0.1 over steps 1-10, time step 10, NR 1e-5, CG 1e-10, at most 10
Newton iterations.  The CPU tests pin the oracle to its recorded results; the GPU tests
run the ten steps through the C-ABI and compare P_bar, the Newton counts and the final P.
"""
import os

import numpy as np
import pytest

from cpfft_gb300 import rve

HERE = os.path.dirname(os.path.abspath(__file__))
MM01 = np.load(os.path.join(HERE, "golden", "mm01_deck.npz"))
MM10 = np.load(os.path.join(HERE, "golden", "mm10_deck.npz"))


def loading(d):
    nstep = int(d["step_last"])
    diag = d["F_max"][[0, 4, 8]] * float(d["step_mult"]) * nstep
    return rve.prescribed_stretch(diag, nstep)


def setup_mm01(d):
    keys = [str(k) for k in d["prop_keys"]]
    props = [dict(zip(keys, map(float, row))) for row in d["props"]]
    N = int(d["N"])
    return dict(N=N, mat=d["mat_list"].astype(np.int32), kocks=np.zeros((3, N ** 3)),
                crystals=[rve.NOT_A_CRYSTAL] * len(props),
                mises={k + 1: p for k, p in enumerate(props)})


def setup_mm10(d):
    return dict(N=int(d["N"]), mat=d["mat_list"].astype(np.int32),
                kocks=np.ascontiguousarray(d["kocks"]), crystals=[rve.BCC48_DECK], mises={})


DECKS = {"mm01": (MM01, setup_mm01), "mm10": (MM10, setup_mm10)}


def test_fixtures_are_the_decks():
    """The fixtures' grids and materials: 7^3; mm01 with the deck's two materials on a
    5x5x4 inclusion of mat2; mm10 a bicrystal of 196 + 147 voxels."""
    assert int(MM01["N"]) == 7 and int(MM10["N"]) == 7
    keys = [str(k) for k in MM01["prop_keys"]]
    for row, ref in zip(MM01["props"], rve.MM01_DECK):
        assert dict(zip(keys, map(float, row))) == ref
    assert sorted(np.bincount(MM01["mat_list"])[1:].tolist()) == [100, 243]
    ang = sorted(map(tuple, np.unique(MM10["kocks"].T, axis=0).tolist()))
    assert ang == [(0.0, 0.0, 0.0), (45.0, 0.0, 0.0)]
    assert sorted(np.unique(MM10["kocks"][0], return_counts=True)[1].tolist()) == [147, 196]


def run(solver, d, nsteps):
    load = loading(d)
    tol_nr, tol_cg, maxit = float(d["tol_nr"]), float(d["tol_cg"]), int(d["max_iter"])
    solver.nr3_begin(tol_cg)
    pb, nw = [], []
    for step in range(1, nsteps + 1):
        rc, Pbar, st = solver.nr3_step(step, load.BC_all[step - 1], load.isNBC, tol_nr, tol_cg,
                                       maxit)
        assert rc >= 0, (step, rc)
        pb.append(Pbar)
        nw.append(st["newton_iters"])
    return np.array(pb), nw


@pytest.mark.parametrize("deck", ["mm01", "mm10"])
def test_oracle_reproduces_its_recorded_deck_runs(oracle, deck):
    d, setup = DECKS[deck]
    c = setup(d)
    o = oracle.Oracle(c["N"], c["mat"], c["kocks"], c["crystals"], float(d["time_step"]), 0,
                      nthreads=4)
    try:
        for k, p in c["mises"].items():
            o.set_mises(k, p)
        pb, nw = run(o, d, int(d["step_last"]))
        assert nw == d["newton_oracle"].tolist()
        assert np.abs(pb - d["Pbar_oracle"]).max() <= 1e-12 * np.abs(d["Pbar_oracle"]).max()
    finally:
        o.close()


@pytest.mark.gpu
@pytest.mark.parametrize("deck", ["mm01", "mm10"])
def test_gpu_runs_the_deck(gpulib, deck):
    """All ten load steps on the GPU (plain FP64 form): P_bar to 1e-10 of the recorded
    oracle run at every step, the same Newton counts, the final P to 1e-8 per voxel."""
    d, setup = DECKS[deck]
    c = setup(d)
    s = gpulib.Solver(c["N"], c["mat"], c["kocks"], c["crystals"], float(d["time_step"]),
                      gpulib.G_REF_SHIFT)
    try:
        for k, p in c["mises"].items():
            s.set_mises(k, **p)
        pb, nw = run(s, d, int(d["step_last"]))
        ref = d["Pbar_oracle"]
        assert nw == d["newton_oracle"].tolist()
        rel = np.abs(pb - ref).max(axis=1) / np.abs(ref).max(axis=1)
        assert rel.max() < 1e-10, rel
        F, P = s.fields()
        Po = d["Pn1_oracle"]
        scale = np.maximum(np.abs(Po).max(axis=0), 1e-6 * np.abs(Po).max())
        assert (np.abs(P - Po).max(axis=0) / scale).max() < 1e-8
    finally:
        s.close()
