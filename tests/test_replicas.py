"""Replica aggregation over two gloo ranks on CPU (the N > 1 bench path):
each rank runs its own crystal; the job rate is the summed work over the
slowest rank's time, and no simulation data crosses ranks."""
import os
import socket

import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    import torch.distributed as dist

    from phonomena_gb300 import crystal, replicas

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    spec = crystal.CrystalSpec(cells=(16, 16, 8), lattice=8, radius=(0.2, 0.4), tungsten_frac=0.5,
                               seed=replicas.rank_seed(rank))
    ids = crystal.material_ids(spec)
    ms = 10.0 * (rank + 1)
    work = float(spec.n_nodes * 100)
    m, w, rate = replicas.aggregate(ms, work, dist)
    out[rank] = (m, w, rate, int(ids.sum()))
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_aggregate():
    import torch.multiprocessing as mp

    port = _free_port()
    world = 2
    with mp.get_context("spawn").Manager() as mgr:
        out = mgr.dict()
        mp.start_processes(_worker, args=(world, port, out), nprocs=world, start_method="spawn", join=True)
        res = dict(out)
    nodes = 17 * 17 * 9
    for rank in range(world):
        m, w, rate, _ = res[rank]
        assert m == 20.0  # slowest rank
        assert w == world * nodes * 100
        assert rate == pytest.approx(w / 20.0)
    assert res[0][3] != res[1][3]  # each rank its own seeded crystal


def test_single_process_aggregate():
    from phonomena_gb300 import replicas

    assert replicas.aggregate(5.0, 100.0) == (5.0, 100.0, 20.0)
