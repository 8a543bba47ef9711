"""Scenes of a batch across ranks (one GPU per rank).

The batched form's scenes are independent, so several GPUs split them with no
data exchange during stepping: :func:`partition_scenes` balances the ranks'
fluid particle counts greedily (largest scene first onto the least-loaded
rank), and :func:`gather_scene_stats` -- the only collective -- collects the
per-scene statistics on one rank in global scene order.  The reference runs one
scene per process (``main.py:8-12``); this is the layer above it that a batch
of scenes needs.
"""


def partition_scenes(counts, world_size):
    """Scene indices of each rank: longest-processing-time greedy on `counts`
    (ties: lower scene index first, then the lower rank).  Deterministic; every
    scene is assigned exactly once; each rank's list is ascending."""
    if world_size < 1:
        raise ValueError("world_size must be positive")
    order = sorted(range(len(counts)), key=lambda i: (-int(counts[i]), i))
    load = [0] * world_size
    parts = [[] for _ in range(world_size)]
    for i in order:
        r = min(range(world_size), key=lambda k: (load[k], k))
        parts[r].append(i)
        load[r] += int(counts[i])
    return [sorted(p) for p in parts]


def gather_scene_stats(local_stats, scene_ids, n_scenes, dist=None, dst=0):
    """Per-scene statistics of all ranks in global scene order on rank `dst`
    (None on the other ranks).  `local_stats[i]` belongs to scene
    `scene_ids[i]`.  Without `dist` (one process) the local list is returned."""
    if dist is None:
        out = [None] * n_scenes
        for sid, st in zip(scene_ids, local_stats):
            out[sid] = st
        return out
    rank, ws = dist.get_rank(), dist.get_world_size()
    payload = list(zip([int(s) for s in scene_ids], local_stats))
    gathered = [None] * ws if rank == dst else None
    dist.gather_object(payload, gathered, dst=dst)
    if rank != dst:
        return None
    out = [None] * n_scenes
    for part in gathered:
        for sid, st in part:
            if out[sid] is not None:
                raise RuntimeError("scene %d reported by two ranks" % sid)
            out[sid] = st
    if any(o is None for o in out):
        raise RuntimeError("scenes missing from the gather: %s" % [i for i, o in enumerate(out) if o is None])
    return out


def max_over_ranks(value, dist=None):
    """The largest `value` over all ranks (the bench's job time), on every rank."""
    if dist is None:
        return float(value)
    import torch
    backend = dist.get_backend()
    dev = torch.device("cuda", torch.cuda.current_device()) if backend == "nccl" else torch.device("cpu")
    t = torch.tensor([float(value)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())
