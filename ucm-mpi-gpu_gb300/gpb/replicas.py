"""Several GPUs as independent replicas over one patch list.

Patches are independent: each builds its own affinity matrix and eigenproblem,
so ranks never exchange device data.  This is how the reference spreads them,
one MPI rank per patch (main.cpp:253-301), with the result planes sent back to
rank 0 (MpiSendMat / MpiRecvMatVec, main.cpp:309-344).  Here a rank takes a
share of the list balanced by predicted cost (longest-processing-time first
on the pixel count), runs it as one batch on its own GPU, and rank 0 gathers
the results over torch.distributed (any backend that carries Python objects;
gloo on the host).
"""
import heapq


def partition(sizes, world):
    """Patch indices per rank, balancing the summed pixel counts: patches in
    decreasing size go to the currently lightest rank (ties: lower rank,
    lower index).  sizes: (height, width) per patch."""
    if world < 1:
        raise ValueError("world must be >= 1")
    order = sorted(range(len(sizes)), key=lambda i: (-int(sizes[i][0]) * int(sizes[i][1]), i))
    heap = [(0, r) for r in range(world)]
    shares = [[] for _ in range(world)]
    for i in order:
        load, r = heapq.heappop(heap)
        shares[r].append(i)
        heapq.heappush(heap, (load + int(sizes[i][0]) * int(sizes[i][1]), r))
    return [sorted(s) for s in shares]


def run_share(compute, patches, rank, world):
    """This rank's (index, result) pairs: compute(list of patches) -> list of
    results, called once on the rank's share (one batch)."""
    mine = partition([p.shape[:2] for p in patches], world)[rank]
    if not mine:
        return []
    outs = compute([patches[i] for i in mine])
    return list(zip(mine, outs))


def gather(pairs, n, rank, world, group=None):
    """Rank 0 receives every rank's (index, result) pairs and returns the n
    results in patch order; the other ranks return None."""
    import torch.distributed as dist
    if world == 1:
        out = [None] * n
        for i, r in pairs:
            out[i] = r
        return out
    bucket = [None] * world if rank == 0 else None
    dist.gather_object(pairs, bucket, dst=0, group=group)
    if rank != 0:
        return None
    out = [None] * n
    for part in bucket:
        for i, r in part:
            out[i] = r
    missing = [i for i, r in enumerate(out) if r is None]
    if missing:
        raise RuntimeError("patches without a result: %s" % missing[:8])
    return out


def balance(sizes, shares):
    """Largest over smallest summed pixel count of the shares (1.0 = even)."""
    loads = [sum(int(sizes[i][0]) * int(sizes[i][1]) for i in s) for s in shares]
    return max(loads) / max(1, min(loads))


__all__ = ["partition", "run_share", "gather", "balance"]
