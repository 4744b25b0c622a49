"""The N>1 path of bench.py on CPU ranks (gloo, world size 2): each rank
builds its own RVE (seed + rank), the figures combine as sum of
voxel-iterations over max time."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, out):
    import sys
    repo = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, os.path.join(repo, "m-themes_gb300"))
    import numpy as np
    import torch.distributed as dist
    from mth import replicas, synth
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    cfg = replicas.replica_config(synth.Config(cell_dim=(8, 8, 8), n_grains=3, seed=40), rank)
    g, _, _ = synth.microstructure(cfg)
    vox_it = float(g.size * (10 + rank))          # rank-dependent work
    secs = 1.0 + rank                              # rank-dependent time
    tot, mx, val = replicas.aggregate(vox_it, secs)
    out[rank] = (cfg.seed, int(g.sum()), tot, mx, val)
    dist.destroy_process_group()


@pytest.mark.timeout(120)
def test_replicas_aggregate_two_ranks():
    ctx = mp.get_context("spawn")
    with ctx.Manager() as m:
        out = m.dict()
        port = _free_port()
        procs = [ctx.Process(target=_worker, args=(r, 2, port, out)) for r in range(2)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(100)
            assert p.exitcode == 0
        r0, r1 = out[0], out[1]
    assert r0[0] == 40 and r1[0] == 41          # own seeds
    assert r0[1] != r1[1]                        # different RVEs
    assert r0[2] == r1[2] == 512 * 10 + 512 * 11
    assert r0[3] == r1[3] == 2.0
    assert abs(r0[4] - (512 * 21) / 2.0) < 1e-9


def _batch_worker(rank, world, port, out):
    import sys
    repo = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, os.path.join(repo, "m-themes_gb300"))
    import numpy as np
    import torch.distributed as dist
    from mth import replicas, synth
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    sizes = [int(np.prod(c.cell_dim)) for c in synth.batch_workload("batch64")]
    mine = replicas.batch_share(sizes, rank, world)
    vox_it = float(sum(sizes[i] for i in mine) * 100)   # 100 Green iterations per member
    tot, mx, val = replicas.aggregate(vox_it, 1.0 + 0.5 * rank)
    out[rank] = (mine, tot, mx, val)
    dist.destroy_process_group()


@pytest.mark.timeout(120)
def test_batch_partition_two_ranks():
    """A batch of independent RVEs split over two CPU ranks: disjoint,
    complete, balanced shares computed without communication; whole-job
    voxel-iterations summed, time the maximum."""
    import numpy as np
    import sys
    sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "m-themes_gb300"))
    from mth import synth
    sizes = [int(np.prod(c.cell_dim)) for c in synth.batch_workload("batch64")]
    ctx = mp.get_context("spawn")
    with ctx.Manager() as m:
        out = m.dict()
        port = _free_port()
        procs = [ctx.Process(target=_batch_worker, args=(r, 2, port, out)) for r in range(2)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(100)
            assert p.exitcode == 0
        r0, r1 = out[0], out[1]
    assert sorted(r0[0] + r1[0]) == list(range(len(sizes)))
    assert sum(sizes[i] for i in r0[0]) == sum(sizes[i] for i in r1[0])
    assert r0[1] == r1[1] == 100.0 * sum(sizes)
    assert r0[2] == r1[2] == 1.5
    assert abs(r0[3] - 100.0 * sum(sizes) / 1.5) < 1e-6


def test_batch_share_edges():
    import sys
    sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "m-themes_gb300"))
    from mth import replicas
    sizes = [27, 8, 64, 8, 27]
    assert replicas.batch_share(sizes, 0, 1) == [0, 1, 2, 3, 4]
    shares = [replicas.batch_share(sizes, r, 3) for r in range(3)]
    assert shares == [[2], [0, 1], [3, 4]]                 # 64 | 27+8 | 27+8
    assert [replicas.batch_share([5], r, 3) for r in range(3)] == [[0], [], []]
    with pytest.raises(ValueError):
        replicas.batch_share(sizes, 3, 3)
