"""Events across ranks (ccake_gb300.replicas): the assignment, and a
world-size-2 gloo run on the CPU with a stand-in for the per-GPU server."""
import os
import socket

import pytest

from ccake_gb300 import replicas


def test_assignment_is_deterministic_and_balanced():
    sizes = [10, 400, 35, 120, 120, 8, 300, 55, 90, 260]
    a = replicas.assign_events(sizes, 3)
    assert a == replicas.assign_events(sizes, 3)
    assert sorted(set(a)) == [0, 1, 2]
    loads = [sum(s for s, r in zip(sizes, a) if r == k) for k in range(3)]
    # longest-processing-time first is within 4/3 of the optimum
    assert max(loads) <= (4 / 3) * max(max(sizes), sum(sizes) / 3) + 1e-9
    assert replicas.assign_events(sizes, 1) == [0] * len(sizes)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, sizes, q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)

    def run_share(share):   # stand-in for a rank's event server
        return [(i, {"rank": rank, "particles": ev}) for i, ev in share]

    out = replicas.run_replicated(sizes, sizes, rank, world, run_share, dist)
    dist.barrier()
    dist.destroy_process_group()
    q.put((rank, out))


def test_two_ranks_over_gloo():
    import torch.multiprocessing as mp
    sizes = [50_000, 10_000, 400_000, 120_000, 35_000, 200_000, 15_000]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, sizes, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = dict(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert res[1] is None
    out = res[0]
    owner = replicas.assign_events(sizes, 2)
    assert [o["particles"] for o in out] == sizes
    assert [o["rank"] for o in out] == owner
    assert set(owner) == {0, 1}
