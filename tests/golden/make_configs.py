"""Oracle records of the named workloads' load histories, for the GPU parity tests.

  config1_n16_centered.npz  16^3, 8 Voronoi grains (seed 1), FCC Voce, uniaxial tension
                            2 % in 20 steps, the centered Green mapping (even N);
  config1_n15_ref.npz       the same RVE recipe at 15^3 with the reference's own mapping
                            (odd N, where the two mappings coincide);
  config2_n63_ref.npz       63^3, 64 grains (seed 2), uniaxial tension 5 % in 50 steps:
                            the first `CONFIG2_STEPS` load steps (odd N).

Each record holds P_bar after every step, the global Newton, P_bar-loop and CG counts of
every step, and the final F and P fields (config 2: every 97th voxel of them and the
field checksums).  Tolerances as the workloads state them: global NR 1e-6, CG 1e-10,
local 1e-10, at most 20 Newton iterations.  The reference (Fortran + MKL) cannot be
built here, so these are the oracle's outputs.

    python tests/golden/make_configs.py config1 | config2
"""
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from cpfft_gb300 import rve  # noqa: E402
from oracle import pyoracle as po  # noqa: E402

TOL_NR, TOL_CG, MAX_ITER = 1.0e-6, 1.0e-10, 20
CONFIG2_STEPS = 3
SUBSAMPLE = 97

# name, N, grains, seed, g_mapping, loading, steps run
CASES = {
    "config1": [("config1_n16_centered", 16, 8, 1, 1, (0.02, 20), 20),
                ("config1_n15_ref", 15, 8, 1, 0, (0.02, 20), 20)],
    "config2": [("config2_n63_ref", 63, 64, 2, 0, (0.05, 50), CONFIG2_STEPS)],
}


def run(name, N, grains, seed, gmap, loading, nsteps):
    r = rve.make_rve(N, grains, seed)
    load = rve.uniaxial_tension(*loading)
    o = po.Oracle(N, r.mat_list, r.kocks, r.crystals, 1.0, gmap)
    t0 = time.time()
    assert o.nr3_begin(TOL_CG) == 0
    pbar, newton, nbc, cg = [], [], [], []
    for s in range(1, nsteps + 1):
        rc, Pb, st = o.nr3_step(s, load.BC_all[s - 1], load.isNBC, TOL_NR, TOL_CG, MAX_ITER)
        assert rc >= 0, (name, s, rc)
        pbar.append(Pb)
        newton.append(st["newton_iters"])
        nbc.append(st["nbc_iters"])
        cg.append(st["cg_iters"])
        print(name, s, f"{time.time() - t0:.0f}s", st["newton_iters"], st["nbc_iters"],
              Pb[[0, 4, 8]], flush=True)
    f = o.fields()
    o.close()
    out = dict(N=N, grains=grains, seed=seed, g_mapping=gmap, loading=np.array(loading),
               steps=nsteps, tol=np.array([TOL_NR, TOL_CG]), max_iter=MAX_ITER,
               pbar=np.array(pbar), newton=np.array(newton), nbc=np.array(nbc),
               cg=np.array(cg))
    if N ** 3 <= 4096:
        out.update(F=f["Fn"], P=f["Pn"])
    else:
        out.update(F_sub=f["Fn"][:, ::SUBSAMPLE], P_sub=f["Pn"][:, ::SUBSAMPLE],
                   subsample=SUBSAMPLE, F_sum=f["Fn"].sum(axis=1), P_sum=f["Pn"].sum(axis=1),
                   P_absmax=np.abs(f["Pn"]).max(axis=1))
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)


if __name__ == "__main__":
    which = sys.argv[1] if len(sys.argv) > 1 else "config1"
    for case in CASES[which]:
        run(*case)
