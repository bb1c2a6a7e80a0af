"""Replicas across GPUs: one process per GPU, independent systems.

The path does not shard within one grid (the global ILU(0) would become
block-Jacobi and the preconditioner would change), so several GPUs serve
independent systems -- ensemble realizations or requests -- with no
data-path collective.  `assign` balances systems over ranks by their device
footprint (largest first to the least loaded rank); `reduce_timing` is the
only collective: the maximum of the ranks' times and the sum of their work,
once per measurement.
"""
import heapq


def assign(footprints, world):
    """Indices of the systems each rank takes: longest-processing-time-first
    bin packing by footprint (bytes, or any additive cost)."""
    if world < 1:
        raise ValueError("world must be >= 1")
    order = sorted(range(len(footprints)), key=lambda i: (-footprints[i], i))
    heap = [(0, r) for r in range(world)]
    out = [[] for _ in range(world)]
    for i in order:
        load, r = heapq.heappop(heap)
        out[r].append(i)
        heapq.heappush(heap, (load + footprints[i], r))
    for r in range(world):
        out[r].sort()
    return out


def reduce_timing(ms, work, device=None):
    """All ranks: (max of ms, sum of work) over the process group; the
    identity without one."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(ms), float(work)
    dev = device if device is not None else "cpu"
    t = torch.tensor([float(ms)], dtype=torch.float64, device=dev)
    w = torch.tensor([float(work)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.all_reduce(w, op=dist.ReduceOp.SUM)
    return float(t.item()), float(w.item())
