"""Partition a variable-size batch of independent systems across ranks.

The batched solve has no data exchange between systems, so N GPUs split the
batch and each solves its share with one batched launch; only the per-system
status (info, iter) and the timing are combined afterwards.  Assignment is
greedy longest-processing-time first: systems in decreasing cost (n^3 for the
factorisation plus n^2 nrhs for the solves) go to the least-loaded rank, which
keeps the largest load within one system's cost of the average.
"""
import heapq

import numpy as np


def system_costs(n, nrhs, kind):
    """Flop estimate per system: 2n^3/3 (LU, kind 0) or n^3/3 (Cholesky,
    kind 1) plus 2 n^2 nrhs for the two triangular solves."""
    n = np.asarray(n, dtype=np.float64)
    nrhs = np.asarray(nrhs, dtype=np.float64)
    kind = np.asarray(kind)
    return np.where(kind == 0, 2.0 / 3.0, 1.0 / 3.0) * n ** 3 + 2.0 * n * n * nrhs


def partition_systems(costs, world_size):
    """Return (parts, loads): parts[r] is the sorted array of system indices
    of rank r, loads[r] the sum of their costs."""
    if world_size < 1:
        raise ValueError("world_size must be >= 1")
    costs = np.asarray(costs, dtype=np.float64)
    order = np.argsort(-costs, kind="stable")
    heap = [(0.0, r) for r in range(world_size)]
    parts = [[] for _ in range(world_size)]
    for i in order:
        load, r = heapq.heappop(heap)
        parts[r].append(int(i))
        heapq.heappush(heap, (load + float(costs[i]), r))
    loads = np.zeros(world_size)
    for load, r in heap:
        loads[r] = load
    return [np.array(sorted(p), dtype=np.int64) for p in parts], loads
