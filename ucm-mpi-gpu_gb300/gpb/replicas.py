"""Several GPUs as independent replicas over one patch list.

Patches are independent: each builds its own affinity matrix and eigenproblem,
so ranks never exchange device data.  This is how the reference spreads them,
one MPI rank per patch (main.cpp:253-301), with the result planes sent back to
rank 0 (MpiSendMat / MpiRecvMatVec, main.cpp:309-344).  Here a rank takes a
share of the list balanced by predicted cost (longest-processing-time first),
runs it as one batch on its own GPU, and rank 0 gathers the results over
torch.distributed (any backend that carries Python objects; gloo on the host).

Predicted cost: pixels^1.41 * (regions + 1)^0.23, fitted (least squares in
logs) to the measured solve time of 115 patches solved one at a time on a
GB300 (tests/golden/replica_costs.npz): larger patches need more outer
iterations than their pixel count says, and patches with more coarse colour
regions have more clustered small eigenvalues.
"""
import heapq


COST_EXP_PIXELS, COST_EXP_REGIONS = 1.41, 0.23


def regions(bgr, down=4, q=32, min_px=8):
    """Coarse colour regions of a BGR patch: 4 x 4 block means quantised to
    32 levels per channel, connected components of each colour with at least
    min_px blocks."""
    import numpy as np
    from scipy import ndimage
    H, W, _ = bgr.shape
    h, w = H // down, W // down
    if h == 0 or w == 0:
        return 1
    b = bgr[:h * down, :w * down].reshape(h, down, w, down, 3).mean((1, 3))
    lab = (b[..., 0] // q) * 64 + (b[..., 1] // q) * 8 + (b[..., 2] // q)
    n = 0
    for v in np.unique(lab):
        cc, k = ndimage.label(lab == v)
        if k:
            n += int((np.bincount(cc.ravel())[1:] >= min_px).sum())
    return n


def predicted_cost(bgr):
    """Relative solve cost of one BGR patch (see the module docstring)."""
    H, W = bgr.shape[:2]
    return float(H * W) ** COST_EXP_PIXELS * float(regions(bgr) + 1) ** COST_EXP_REGIONS


def partition(sizes, world, costs=None):
    """Patch indices per rank, balancing the summed costs (default: pixel
    counts): patches in decreasing cost go to the currently lightest rank
    (ties: lower rank, lower index).  sizes: (height, width) per patch."""
    if world < 1:
        raise ValueError("world must be >= 1")
    cost = list(costs) if costs is not None else [int(h) * int(w) for h, w in sizes]
    order = sorted(range(len(sizes)), key=lambda i: (-cost[i], i))
    heap = [(0, r) for r in range(world)]
    shares = [[] for _ in range(world)]
    for i in order:
        load, r = heapq.heappop(heap)
        shares[r].append(i)
        heapq.heappush(heap, (load + cost[i], r))
    return [sorted(s) for s in shares]


def run_share(compute, patches, rank, world, costs=None):
    """This rank's (index, result) pairs: compute(list of patches) -> list of
    results, called once on the rank's share (one batch).  costs: per patch
    (e.g. predicted_cost of each BGR patch), the same on every rank."""
    mine = partition([p.shape[:2] for p in patches], world, costs)[rank]
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
