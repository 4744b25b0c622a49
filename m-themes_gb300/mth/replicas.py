"""Multi-GPU runs: replicas only.

A single RVE shards only with an all-to-all per FFT, so N GPUs run N
independent RVEs (one per rank, seed + rank) with no data-path collective;
the only collectives are the barrier around the timed region and the
reduction of the per-rank figures: voxel-iterations are summed, times take
the maximum over ranks (weak scaling).  A batch of independent RVEs is
partitioned: each rank steps its share of the members as one batch."""
from __future__ import annotations

import copy


def replica_config(cfg, rank: int):
    """The RVE of one rank: the same workload with its own seed."""
    c = copy.deepcopy(cfg)
    c.seed = cfg.seed + rank
    return c


def aggregate(vox_iters: float, seconds: float, device=None):
    """(total voxel-iterations, max seconds, voxel-iterations/s) over the
    ranks of the default process group (a single process when none)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return vox_iters, seconds, vox_iters / seconds
    t = torch.tensor([vox_iters], dtype=torch.float64, device=device)
    m = torch.tensor([seconds], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    dist.all_reduce(m, op=dist.ReduceOp.MAX)
    return float(t.item()), float(m.item()), float(t.item()) / float(m.item())


def batch_share(sizes, rank: int, world: int):
    """Indices of the batch members rank `rank` of `world` runs: the members
    (voxel counts `sizes`) dealt largest first to the rank with the fewest
    voxels so far (ties: lower index, lower rank), so the shares are balanced
    and every rank computes the same partition without communicating."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("rank %d of world %d" % (rank, world))
    load = [0] * world
    own = [[] for _ in range(world)]
    for i in sorted(range(len(sizes)), key=lambda i: (-sizes[i], i)):
        r = min(range(world), key=lambda q: (load[q], q))
        own[r].append(i)
        load[r] += sizes[i]
    return sorted(own[rank])
