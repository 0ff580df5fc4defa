"""The N>1 path of bench.py on the CPU (gloo, world size 2): replicas run
their own seeded walkers and the timing is the slowest rank's, reduced with
a MAX all-reduce; the whole-job value is the units of all ranks over it."""
import os
import socket

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, out):
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        local = [1.0 + rank, 3.0 - rank, 0.5 * (rank + 1)]
        got = bench.slowest_rank_times(torch, local, torch.device("cpu"), world)
        from qmctorch_gb300.scf import Molecule
        mol = Molecule("H 0 0 -0.37; H 0 0 0.37", unit="angs", basis="sto-3g")
        pos = bench.seeded_positions(mol, 8, seed=rank)
        out[rank] = (got, pos)
    finally:
        dist.destroy_process_group()


def test_replica_timing_is_the_slowest_rank():
    world = 2
    port = _free_port()
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_worker, args=(world, port, out), nprocs=world, join=True)
        res = dict(out)
    for r in range(world):
        assert res[r][0] == [2.0, 3.0, 1.0]
    # every rank samples its own walkers
    assert not np.allclose(res[0][1], res[1][1])
    units_per_rank = 16384 * 100
    value = units_per_rank * world / max(res[0][0][0], res[1][0][0])
    assert value == pytest.approx(2 * units_per_rank / 2.0)
