"""One all-pairs matrix split over several ranks (mestrado_gb300/shard.py):
the row blocks cover every pair of the upper triangle exactly once and
balance the DP cells; the blocks reassemble into the full symmetric matrix;
and two gloo ranks on the CPU, each scoring its block through a stand-in
scorer (the oracle) and exchanging blocks by one all-gather, both end with
the matrix a single rank computes."""
import os
import socket
import sys

import numpy as np
import pytest

import oracle_py as O
from mestrado_gb300 import shard, synth

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


class OracleScorer:
    """The per-rank device call (Context.score_block) stood in by the oracle."""

    def score_block(self, xseqs, yseqs):
        D = O.score_all(list(xseqs) + list(yseqs))
        return np.ascontiguousarray(D[: len(xseqs), len(xseqs):], dtype=np.float32)


@pytest.mark.parametrize("world", [1, 2, 3, 5, 8])
def test_tiles_cover_the_triangle_once_and_balance_cells(world):
    S = synth.config(2).subset(range(400))
    L = np.array([len(s) for s in S], dtype=np.float64)
    b = shard.tile_plan(L, world)
    n = len(L)
    assert b[0] == 0 and b[-1] == n and np.all(np.diff(b) >= 0) and len(b) == world + 1
    cover = np.zeros((n, n), dtype=np.int32)
    for r0, r1 in zip(b[:-1], b[1:]):
        cover[r0:r1, r0:] += 1
    assert np.array_equal(np.triu(cover), np.triu(np.ones((n, n), dtype=np.int32)))
    cells = shard.block_cells(L, b)
    total = (L.sum() ** 2 - (L * L).sum()) / 2
    assert abs(cells.sum() - total) <= 1e-6 * total
    # each block within one row's cells of an even share
    row_max = float((L * L.sum()).max())
    assert np.all(np.abs(cells - total / world) <= row_max)


def test_assemble_equals_full_matrix():
    S = synth.family(37, 90, ps=0.1, pi=0.01, seed=3)
    seqs = [S[i] for i in range(len(S))]
    D = O.score_all(seqs)
    for world in (1, 2, 4, 7):
        b = shard.tile_plan([len(s) for s in seqs], world)
        blocks = [OracleScorer().score_block(seqs[r0:r1], seqs[r0:]) for r0, r1 in zip(b[:-1], b[1:])]
        assert np.array_equal(shard.assemble(blocks, b, len(seqs)), D)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import torch.distributed as dist
    from mestrado_gb300 import shard as sh, synth as sy
    dist.init_process_group("gloo", rank=rank, world_size=world)
    S = sy.family(29, 70, ps=0.1, pi=0.01, seed=8)
    D = sh.sharded_score_all(OracleScorer(), S, rank, world, device="cpu")
    out.put((rank, D))
    dist.destroy_process_group()


def test_two_gloo_ranks_assemble_the_single_rank_matrix():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    res = sorted((q.get(timeout=180) for _ in ps), key=lambda t: t[0])
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    S = synth.family(29, 70, ps=0.1, pi=0.01, seed=8)
    D = O.score_all([S[i] for i in range(len(S))])
    for _, Dr in res:
        assert np.array_equal(Dr, D)
        assert np.array_equal(Dr, Dr.T)
