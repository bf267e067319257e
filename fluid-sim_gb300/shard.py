"""Host-side partition of a batch of independent scenes over ranks.

A scene's step does not shard (its MIC(0) wavefronts serialise across any
cut), but a batch of scenes does: each rank (one GPU) advances a subset, and
the only exchange is a host gather of per-scene results (losses, statistics,
gradients).  Scenes are assigned longest-first to the least-loaded rank
(load = cells), the same rule the batch applies to its host workers.
"""
from __future__ import annotations


def partition(loads, world):
    """Indices of the scenes each of `world` ranks runs (LPT assignment by load)."""
    if world < 1:
        raise ValueError("world must be >= 1")
    order = sorted(range(len(loads)), key=lambda k: (-loads[k], k))
    parts = [[] for _ in range(world)]
    total = [0] * world
    for k in order:
        r = min(range(world), key=lambda i: (total[i], i))
        parts[r].append(k)
        total[r] += loads[k]
    return [sorted(p) for p in parts]


def gather(values_by_scene, parts, rank, world, group=None):
    """Every rank passes {scene index: value} for its own scenes; returns the
    values of all scenes in scene order (torch.distributed all_gather_object;
    with world == 1 no process group is needed)."""
    mine = {k: values_by_scene[k] for k in parts[rank]}
    if world == 1:
        merged = mine
    else:
        import torch.distributed as dist
        out = [None] * world
        dist.all_gather_object(out, mine, group=group)
        merged = {}
        for d in out:
            merged.update(d)
    n = sum(len(p) for p in parts)
    if sorted(merged) != list(range(n)):
        raise RuntimeError("gather: scenes missing or duplicated across ranks")
    return [merged[k] for k in range(n)]
