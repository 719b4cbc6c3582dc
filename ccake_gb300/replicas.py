"""Events across GPUs: one process per GPU, each running its own event server
on its share of the events (independent events, no data-path collective).

`assign_events` splits the events by device bytes (longest-processing-time
first: largest event to the least-loaded rank), deterministically, so every
rank computes the same assignment without communication. `run_replicated`
runs a rank's share and gathers the per-event results on rank 0 (one
`gather_object` after the work; the only collective).
"""
from __future__ import annotations

import heapq


def assign_events(sizes, n_ranks):
    """Rank of each event: events in decreasing size go to the rank with the
    smallest total so far (ties to the lower rank; equal sizes keep their
    order)."""
    if n_ranks < 1:
        raise ValueError("n_ranks must be >= 1")
    order = sorted(range(len(sizes)), key=lambda i: (-sizes[i], i))
    heap = [(0, r) for r in range(n_ranks)]
    owner = [0] * len(sizes)
    for i in order:
        load, r = heapq.heappop(heap)
        owner[i] = r
        heapq.heappush(heap, (load + sizes[i], r))
    return owner


def run_replicated(events, sizes, rank, world, run_share, dist=None):
    """Runs this rank's events with run_share(list of (index, event)) -> list
    of (index, result) and returns, on rank 0, the results of all events in
    event order (None on the other ranks). With world == 1 no process group
    is needed."""
    owner = assign_events(sizes, world)
    mine = [(i, ev) for i, ev in enumerate(events) if owner[i] == rank]
    local = run_share(mine)
    if world == 1:
        gathered = [local]
    else:
        gathered = [None] * world if rank == 0 else None
        dist.gather_object(local, gathered, dst=0)
    if rank != 0:
        return None
    out = [None] * len(events)
    for part in gathered:
        for i, res in part:
            out[i] = res
    return out
