"""Sharding a batch of worlds over ranks (one GPU per rank).

Worlds never interact (contact.go:204-207), so N GPUs each take a disjoint
subset of the worlds and step them with no data-path collective.  The only
communication is a host-side gather of results (state, statistics) after a
rollout.  The partition balances the narrowphase cost, which grows as n^2 in
the bodies of a world.
"""
import numpy as np


def partition(counts, world_size):
    """World ids per rank, balancing sum(n^2) greedily (largest first).
    Deterministic: every rank computes the same partition."""
    counts = np.asarray(counts)
    order = np.argsort(-counts.astype(np.int64) ** 2, kind="stable")
    load = np.zeros(world_size, np.int64)
    parts = [[] for _ in range(world_size)]
    for w in order:
        r = int(np.argmin(load))
        parts[r].append(int(w))
        load[r] += int(counts[w]) ** 2
    return [sorted(p) for p in parts]


def gather_bodies(local_state, local_worlds, scene, group=None):
    """Assemble the full body state from every rank's shard (torch.distributed
    all_gather_object on the host).  local_state: dict of arrays for the
    rank's worlds in `local_worlds` order."""
    import torch.distributed as dist
    ws = dist.get_world_size(group)
    items = [None] * ws
    dist.all_gather_object(items, (local_worlds, {k: np.asarray(v) for k, v in local_state.items()}), group=group)
    out = {}
    for worlds, state in items:
        offs = 0
        for w in worlds:
            sl = scene.world_slice(w)
            n = sl.stop - sl.start
            for k, v in state.items():
                if k not in out:
                    out[k] = np.zeros((scene.num_bodies,) + v.shape[1:], v.dtype)
                out[k][sl] = v[offs:offs + n]
            offs += n
    return out
