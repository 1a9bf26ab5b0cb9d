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


def _config4_rank(rank, world, port, outdir):
    """bench.py's 48-RVE arm on one gloo rank, with the library's batch call replaced by a
    stand-in that takes 10 ms per load step and reports N^3 x 4 stress updates per step
    of each RVE (the arm's partition, barriers and reduction are what is under test)."""
    import contextlib
    import json
    import sys
    import time
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, root)
    import bench
    import cpfft_gb300 as cp
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    seen = []

    def batch_stub(rves, **kw):
        time.sleep(0.01 * rves[0]["nsteps"])
        seen.append([r["N"] for r in rves])
        return [{"voxel_updates": r["N"] ** 3 * 4 * r["nsteps"]} for r in rves]

    cp.load_library = lambda: None
    cp.batch_solve = batch_stub
    args = bench.make_parser().parse_args(["--workload", "config4", "--steps", "2",
                                           "--warmup", "1", "--batch-threads", "1"])
    out = os.path.join(outdir, f"c4_rank{rank}.txt")
    try:
        with open(out, "w") as f, contextlib.redirect_stdout(f):
            assert bench.config4_arm(args) == 0
        with open(os.path.join(outdir, f"c4_seen{rank}.json"), "w") as f:
            json.dump(seen, f)
    finally:
        dist.destroy_process_group()


def test_config4_partitioned_over_two_ranks(tmp_path):
    """`bench.py --workload config4` under two ranks: each solves its own 24 RVEs, and
    rank 0's line reports the units of all 48 over the slowest rank's time."""
    import json
    world = 2
    mp.spawn(_config4_rank, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True)
    seen = [json.load(open(tmp_path / f"c4_seen{r}.json")) for r in range(world)]
    Ns = (24, 32, 48, 64)
    for r, batches in enumerate(seen):
        assert all(b == [Ns[k % 4] for k in range(24 * r, 24 * r + 24)] for b in batches)
    assert open(tmp_path / "c4_rank1.txt").read() == ""
    line = json.loads(open(tmp_path / "c4_rank0.txt").read())
    all_units = sum(Ns[k % 4] ** 3 for k in range(48)) * 4 * 2    # 48 RVEs, 2 timed steps
    assert line["n_gpus"] == 2 and line["by_threads"]["1"]["voxel_updates"] == all_units
    assert 9.0 < line["ms_per_step"] < 500.0     # 10 ms a load step in the stand-in
