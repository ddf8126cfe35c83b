"""Box-wise sharding of an ensemble over the ranks of a job.

The ensemble's boxes are independent (no exchange between them), so N
ranks share them out: longest-processing-time assignment by site count
(largest box to the least-loaded rank), then one gather of the per-box
statistics at the end.  No counterpart in the reference, which runs one
box per job.  Host code only: no device work here.
"""

import numpy as np


def box_sites(p):
    """Sites of one box (a BoxParam or a 3-sequence of extents)."""
    n = p.ntotal if hasattr(p, "ntotal") else p
    return int(n[0]) * int(n[1]) * int(n[2])


def shard_boxes(params, world):
    """Indices of the boxes each rank owns: a list of `world` sorted
    lists, together a partition of range(len(params)).  Deterministic:
    ties go to the lower rank, boxes of equal size in index order."""
    if world < 1:
        raise ValueError("world must be >= 1")
    sizes = [box_sites(p) for p in params]
    order = sorted(range(len(sizes)), key=lambda i: (-sizes[i], i))
    load = [0] * world
    owned = [[] for _ in range(world)]
    for i in order:
        r = min(range(world), key=lambda k: (load[k], k))
        owned[r].append(i)
        load[r] += sizes[i]
    return [sorted(o) for o in owned]


def gather_box_stats(pg, nbox, local_idx, local_stats):
    """All ranks' per-box statistics in box order (a list of nbox entries)
    on every rank.  pg is torch.distributed (initialised) or None for a
    single rank."""
    pairs = list(zip(local_idx, local_stats))
    if pg is None:
        gathered = [pairs]
    else:
        gathered = [None] * pg.get_world_size()
        pg.all_gather_object(gathered, pairs)
    out = [None] * nbox
    for part in gathered:
        for i, st in part:
            if out[i] is not None:
                raise RuntimeError("box %d reported by two ranks" % i)
            out[i] = st
    missing = [i for i, v in enumerate(out) if v is None]
    if missing:
        raise RuntimeError("boxes without statistics: %s" % missing)
    return out


def load_imbalance(params, shards):
    """max / mean sites per rank of a sharding."""
    loads = np.array([sum(box_sites(params[i]) for i in s) for s in shards],
                     dtype=np.float64)
    return float(loads.max() / loads.mean()) if loads.mean() > 0 else 1.0
