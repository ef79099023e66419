"""bench.py with N>1 ranks: every rank scores its own replica (no data-path
collective); the whole-job value is all ranks' cells over the slowest rank's
time.  Two gloo ranks on the CPU."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench
    w, r, _ = bench._dist()
    assert (w, r) == (world, rank)
    # rank r: 10^9 (r+1) cells in (r+1) seconds
    v = bench.aggregate_gcups(w, 1e9 * (r + 1), float(r + 1))
    seed = bench.replica_seed(r)
    import torch.distributed as dist
    seeds = [None] * w
    dist.all_gather_object(seeds, seed)
    out.put((r, v, seeds))
    dist.destroy_process_group()


def test_two_rank_aggregate_and_distinct_replicas():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    res = sorted(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    # (1e9 + 2e9) cells / max(1 s, 2 s) = 1.5 GCUPS on every rank
    assert [r[1] for r in res] == [1.5, 1.5]
    seeds = res[0][2]
    assert len(set(seeds)) == 2 and res[1][2] == seeds
