"""CPU, world_size 2 over gloo: the multi-rank path of bench.py. Every rank
draws its own population (no sample shared between ranks, no collective on
the data path), the job's time is the slowest rank's (all_reduce MAX) and the
whole-job rate counts every rank's samples."""
import os
import socket

import numpy as np
import pytest
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        bench.set_population(8)
        r, lr, w = bench.rank_info()
        assert (r, lr, w) == (rank, rank, world)
        an, prior, truth = bench.make_workload(seed_offset=rank)
        local = 1.0 + rank  # this rank's seconds per step
        slowest = bench.max_over_ranks(local, world, "cpu")
        rate = bench.job_rate(len(prior), world, slowest)
        np.savez(os.path.join(out_dir, f"r{rank}.npz"), timing=np.array([slowest, rate]),
                 prior=np.array([p.as_tuple() for p in prior]))
    finally:
        dist.destroy_process_group()


def test_two_ranks_shard_and_reduce(tmp_path):
    pytest.importorskip("torch")
    world = 2
    mp.spawn(_rank_main, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True)
    a, b = (np.load(tmp_path / f"r{i}.npz") for i in range(world))
    # both ranks agree on the job time (the slowest rank's) and the rate
    assert a["timing"][0] == b["timing"][0] == 2.0
    assert a["timing"][1] == b["timing"][1] == world * 8 / 2.0
    # disjoint populations of the same size
    pa, pb = a["prior"], b["prior"]
    assert pa.shape == pb.shape == (8, 6)
    assert not any(np.array_equal(x, y) for x in pa for y in pb)
