"""The N>1 path on CPU: world_size-2 gloo ranks, each solving its own RVE replica with
no data-path collective; only the timing summary is reduced (max time, summed units),
as `bench.py --gpus N` does over NCCL."""
import os
import socket

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from cpfft_gb300 import replicas, rve


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _solve_replica(seed):
    """One load step of a 5^3 RVE with the CPU oracle (the per-rank work stand-in)."""
    from oracle import pyoracle as po
    r = rve.make_rve(5, 3, seed)
    load = rve.uniaxial_tension(0.02, 20)
    o = po.Oracle(5, r.mat_list, r.kocks, r.crystals, 1.0, 0, nthreads=1)
    try:
        o.nr3_begin(1e-10)
        rc, Pbar, st = o.nr3_step(1, load.BC_all[0], load.isNBC, 1e-6, 1e-10, 20)
        assert rc == 0
        return Pbar
    finally:
        o.close()


def _rank_main(rank, world, port, outdir):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        lo, hi = replicas.partition(4, world, rank)
        pbars = [_solve_replica(100 + k) for k in range(lo, hi)]
        units = float(len(pbars) * 5 ** 3)
        t_dev = 1.0 + rank          # rank 1 is the slowest
        t_e2e = 2.0 + 0.5 * rank
        tmax, temax, utot = replicas.reduce_timings(t_dev, t_e2e, units)
        np.savez(os.path.join(outdir, f"rank{rank}.npz"), lo=lo, hi=hi,
                 pbars=np.array(pbars), red=np.array([tmax, temax, utot]))
    finally:
        dist.destroy_process_group()


def test_partition_covers():
    for n in (0, 1, 5, 48):
        for world in (1, 2, 3, 8):
            seen = []
            for r in range(world):
                lo, hi = replicas.partition(n, world, r)
                seen.extend(range(lo, hi))
                assert hi - lo in (n // world, n // world + 1)
            assert seen == list(range(n))
    with pytest.raises(ValueError):
        replicas.partition(4, 2, 2)


def test_reduce_single_process():
    assert replicas.reduce_timings(1.5, 2.5, 10.0) == (1.5, 2.5, 10.0)


def test_two_rank_replicas(tmp_path, oracle):
    world = 2
    mp.spawn(_rank_main, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True)
    res = [np.load(tmp_path / f"rank{r}.npz") for r in range(world)]
    # every rank sees the same whole-job summary: slowest rank's times, summed units
    for d in res:
        assert np.allclose(d["red"], [2.0, 2.5, 4 * 5 ** 3])
    # the replicas' results equal single-process solves of the same RVEs
    assert (int(res[0]["lo"]), int(res[0]["hi"]), int(res[1]["lo"]), int(res[1]["hi"])) == (0, 2, 2, 4)
    ref = _solve_replica(102)
    assert np.array_equal(res[1]["pbars"][0], ref)
