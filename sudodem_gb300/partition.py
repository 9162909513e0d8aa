"""Sharding independent specimens across GPUs (one process per GPU).

Specimens never exchange data, so a multi-GPU run is a partition of the specimen list: each
rank steps its own batch and only the per-rank totals are combined at the end.  The
partition balances the summed particle counts (longest-processing-time greedy: specimens by
decreasing size, each to the least-loaded rank; ties to the lower rank), and every rank
computes the same partition from the sizes alone.
"""
import heapq


def partition_scenes(sizes, world_size):
    """Lists of specimen indices per rank (ascending within a rank)."""
    if world_size < 1:
        raise ValueError("world_size must be >= 1")
    order = sorted(range(len(sizes)), key=lambda i: (-sizes[i], i))
    heap = [(0, r) for r in range(world_size)]
    parts = [[] for _ in range(world_size)]
    for i in order:
        load, r = heapq.heappop(heap)
        parts[r].append(i)
        heapq.heappush(heap, (load + sizes[i], r))
    return [sorted(p) for p in parts]


def rank_share(sizes, rank, world_size):
    return partition_scenes(sizes, world_size)[rank]
