"""Ensembles over several ranks (one process per GPU in production): every rank
draws its own samples and solves them without exchange; the job's time is the
slowest rank's. Exercised here with two gloo ranks on the CPU."""
import os
import socket

import numpy as np
import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

from memilio_gb300 import replicas as R
from memilio_gb300 import workloads as W


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        base = W.mobility_graph(seed=1, N=5, out_degree=2)
        graphs = R.ensemble_for_rank(3, rank, base=base)
        # a rank-dependent "time": the job's time is the maximum
        t = R.max_over_ranks(1.0 + rank)
        out[rank] = (np.stack([g.params for g in graphs]), t,
                     R.job_throughput(sum(g.num_nodes for g in graphs) * 10.0, t, world))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_shard_samples_and_take_the_slowest():
    world = 2
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_rank, args=(world, _free_port(), out), nprocs=world, join=True)
        res = dict(out)
    p0, t0, v0 = res[0]
    p1, t1, v1 = res[1]
    assert t0 == t1 == 2.0  # both ranks see the slowest rank's time
    assert not np.allclose(p0, p1)  # independent samples per rank
    # rank 0 draws exactly the single-process ensemble
    base = W.mobility_graph(seed=1, N=5, out_degree=2)
    single = np.stack([g.params for g in W.ensemble(num_samples=3, base=base)])
    np.testing.assert_array_equal(p0, single)
    assert v0 == v1 == pytest.approx(2 * 3 * 5 * 10.0 / 2.0)


def test_single_process_needs_no_group():
    assert R.max_over_ranks(3.5) == 3.5
    assert R.job_throughput(100.0, 2.0, 1) == 50.0
