"""Scene sharding across ranks (one process per GPU).

Scenes are independent, so a batch shards by scene with no exchange during
stepping: each rank builds one context over its own scenes.  Collectives are
used only around the run: the timing barrier, the max-over-ranks time, and
gathering the recorder histories to rank 0 afterwards.
"""
from __future__ import annotations

import numpy as np


def assign(costs, world):
    """Balanced assignment of scenes to ranks: longest-processing-time-first
    over the per-scene costs (air cells), ties broken by scene index.
    Returns a list (per rank) of ascending scene indices."""
    order = sorted(range(len(costs)), key=lambda i: (-costs[i], i))
    load = [0.0] * world
    owned = [[] for _ in range(world)]
    for i in order:
        r = min(range(world), key=lambda k: (load[k], k))
        owned[r].append(i)
        load[r] += costs[i]
    return [sorted(o) for o in owned]


def local_scenes(costs, rank, world):
    """Scene indices of `rank`; a single scene is replicated on every rank."""
    if len(costs) == 1:
        return [0]
    return assign(costs, world)[rank]


def gather_histories(local, owned_all, n_scenes, dist=None, device="cpu"):
    """Recorder histories of every scene on rank 0.

    local: list of [T][n_rec_s] arrays for this rank's scenes (in the order of
    its owned list); owned_all: assign(...) result.  Returns the list over all
    scenes on rank 0 (None elsewhere).  Histories are padded to a common
    shape for the collective and cut back afterwards."""
    import torch

    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return list(local)
    rank, world = dist.get_rank(), dist.get_world_size()
    T = max((h.shape[0] for h in local), default=0)
    R = max((h.shape[1] for h in local), default=0)
    meta = torch.tensor([T, R, len(local)], dtype=torch.int64, device=device)
    metas = [torch.zeros_like(meta) for _ in range(world)]
    dist.all_gather(metas, meta)
    Tm = int(max(m[0] for m in metas))
    Rm = int(max(m[1] for m in metas))
    Nm = int(max(m[2] for m in metas))
    buf = torch.zeros((Nm, Tm, Rm), dtype=torch.float64, device=device)
    shapes = torch.zeros((Nm, 2), dtype=torch.int64, device=device)
    for k, h in enumerate(local):
        buf[k, : h.shape[0], : h.shape[1]] = torch.as_tensor(np.asarray(h, np.float64))
        shapes[k, 0], shapes[k, 1] = h.shape[0], h.shape[1]
    bufs = [torch.zeros_like(buf) for _ in range(world)]
    shps = [torch.zeros_like(shapes) for _ in range(world)]
    dist.all_gather(bufs, buf)
    dist.all_gather(shps, shapes)
    if rank != 0:
        return None
    out = [None] * n_scenes
    for r in range(world):
        for k, s in enumerate(owned_all[r]):
            t, n = int(shps[r][k, 0]), int(shps[r][k, 1])
            out[s] = bufs[r][k, :t, :n].cpu().numpy()
    return out
