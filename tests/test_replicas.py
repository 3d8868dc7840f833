"""The N>1 path: one replica per rank with work of its own and no collective
on the data path; only the timing is reduced (slowest rank, summed steps).
Runs as two gloo ranks on the CPU."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

from thunderrw_gb300 import replicas


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir):
    import torch
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    r, w, local = replicas.rank_env()
    assert (r, w, local) == (rank, world, rank)
    # each rank walks its own replica: its own sources and Philox key
    from oracle import oracle as O
    from thunderrw_gb300 import generators as G
    g = G.make_graph("rmat", 1 << 9, 8, seed=3)
    src = G.random_sources(g["row"], 16, seed=replicas.replica_seed(7, rank) & 0x7FFFFFFF).numpy()
    og = O.Graph(g["row"], g["adj"])
    res = O.walk(og, O.make_desc("ppr", "uniform", "uniform", length=1, tp=0.2,
                                 seed=replicas.replica_seed(11, rank)), src, per_query=50, want_lengths=False)
    seconds = 1.0 + rank  # the slowest rank sets the time
    t, s = replicas.reduce_timing(seconds, res["steps"], world)
    np.save(os.path.join(out_dir, "rank%d.npy" % rank), np.array([t, s, res["steps"], src[0]], dtype=np.float64))
    dist.barrier()
    dist.destroy_process_group()


@pytest.mark.timeout(300)
def test_two_gloo_replicas(tmp_path):
    world = 2
    mp.start_processes(_rank_main, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True,
                       start_method="spawn")
    r0, r1 = (np.load(str(tmp_path / ("rank%d.npy" % r))) for r in range(world))
    assert r0[0] == r1[0] == 2.0                      # max over ranks
    assert r0[1] == r1[1] == r0[2] + r1[2]            # summed steps
    assert r0[2] != r1[2] or r0[3] != r1[3]           # the replicas did different work


def test_replica_helpers():
    assert replicas.replica_seed(5, 0) == 5
    assert len({replicas.replica_seed(5, r) for r in range(8)}) == 8
    for total in (0, 1, 7, 100):
        for world in (1, 2, 3, 8):
            parts = [replicas.shard(total, r, world) for r in range(world)]
            assert parts[0][0] == 0 and parts[-1][1] == total
            assert all(a[1] == b[0] for a, b in zip(parts, parts[1:]))
            assert max(e - b for b, e in parts) - min(e - b for b, e in parts) <= 1
    assert replicas.reduce_timing(3.0, 10, 1) == (3.0, 10.0)
