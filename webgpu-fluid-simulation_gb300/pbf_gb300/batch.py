"""Host-side placement of independent scenes on ranks.

Batched scenes do not interact, so N GPUs split a batch by scene: each rank
steps its own subset in one batch handle (no collective on the data path)
and the per-scene results are gathered on the host afterwards.
"""


def partition_scenes(counts, world):
    """Greedy longest-first partition of scenes over `world` ranks by
    particle count (each scene goes to the currently lightest rank).
    Returns one sorted list of scene indices per rank."""
    order = sorted(range(len(counts)), key=lambda i: (-int(counts[i]), i))
    load = [0] * world
    parts = [[] for _ in range(world)]
    for i in order:
        r = min(range(world), key=lambda k: (load[k], k))
        parts[r].append(i)
        load[r] += int(counts[i])
    return [sorted(p) for p in parts]


def imbalance(counts, parts):
    """Largest rank load over the mean rank load (1.0 = perfect balance)."""
    loads = [sum(int(counts[i]) for i in p) for p in parts]
    mean = sum(loads) / max(len(loads), 1)
    return max(loads) / mean if mean else 1.0


def gather_scene_results(local, dist=None):
    """Merge {scene index: result} dicts of all ranks (torch.distributed
    all_gather_object when a process group is up; identity otherwise).
    Raises if two ranks report the same scene."""
    if dist is None or not dist.is_available() or not dist.is_initialized():
        return dict(local)
    parts = [None] * dist.get_world_size()
    dist.all_gather_object(parts, dict(local))
    merged = {}
    for p in parts:
        for k, v in p.items():
            if k in merged:
                raise RuntimeError("scene %d reported by two ranks" % k)
            merged[k] = v
    return merged
