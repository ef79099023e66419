"""One all-pairs distance matrix split over several GPUs (one process each).

The reference distributes the sequences by rows over its MPI ranks and passes
column blocks around a ring, each rank scoring its rows against every block
(SpeciesBlock.cpp:242-403, the ring at :377-402).  Here the pair space is
split once: rank k scores the row block [r_k, r_{k+1}) against the columns
[r_k, n) -- its rows' part of the upper triangle, the diagonal included --
with one nwg_score_block call (column offset r_k), and the blocks are
exchanged by one all-gather and mirrored into the full symmetric matrix.
Pairs are independent, so there is no other exchange.  The row boundaries
balance the DP cells, sum_{i in block} L_i * sum_{j >= i} L_j, across ranks.

tile_plan and assemble are pure host logic (tested with two gloo ranks on
the CPU); sharded_score_all runs the split on the ranks' GPUs with any
torch.distributed backend (NCCL on a multi-GPU node).
"""
from __future__ import annotations

import numpy as np


def tile_plan(lengths, world: int) -> np.ndarray:
    """Row boundaries r_0 = 0 <= r_1 <= ... <= r_world = n of a cell-balanced
    split of the upper triangle (diagonal included) into `world` row blocks."""
    L = np.asarray(lengths, dtype=np.float64)
    n = len(L)
    if world < 1:
        raise ValueError("world must be >= 1")
    suffix = np.cumsum(L[::-1])[::-1]                 # sum_{j >= i} L_j
    cost = np.cumsum(L * suffix)                      # cells of rows [0, i]
    total = cost[-1] if n else 0.0
    bounds = [0]
    for k in range(1, world):
        bounds.append(int(np.searchsorted(cost, total * k / world, side="left")) + 1 if n else 0)
    bounds.append(n)
    b = np.maximum.accumulate(np.clip(np.array(bounds, dtype=np.int64), 0, n))
    return b


def block_cells(lengths, bounds) -> np.ndarray:
    """DP cells of each rank's block: pairs (i, j), i in the block, j > i."""
    L = np.asarray(lengths, dtype=np.float64)
    after = np.concatenate([np.cumsum(L[::-1])[::-1][1:], [0.0]])   # sum_{j > i} L_j
    per_row = L * after
    return np.array([per_row[r0:r1].sum() for r0, r1 in zip(bounds[:-1], bounds[1:])])


def assemble(blocks, bounds, n: int) -> np.ndarray:
    """The full symmetric n x n matrix from each rank's block
    (rows [r_k, r_{k+1}) x columns [r_k, n)); the lower triangle of each block
    row is mirrored from the blocks above it."""
    D = np.zeros((n, n), dtype=np.float32)
    for (r0, r1), B in zip(zip(bounds[:-1], bounds[1:]), blocks):
        B = np.asarray(B, dtype=np.float32).reshape(r1 - r0, n - r0)
        D[r0:r1, r0:] = B
    iu = np.triu_indices(n, 1)
    D[(iu[1], iu[0])] = D[iu]
    return D


def sharded_score_all(ctx, seqs, rank: int, world: int, device=None):
    """Score one all-pairs matrix split over `world` ranks: this rank's block
    on its own GPU through ctx (nwg_score_block), then one all-gather of the
    blocks (torch.distributed, initialised by the caller); returns the full
    matrix on every rank (numpy, float32)."""
    import torch
    import torch.distributed as dist

    n = len(seqs)
    seqs = [seqs[i] for i in range(n)]
    lengths = [len(s) for s in seqs]
    b = tile_plan(lengths, world)
    r0, r1 = int(b[rank]), int(b[rank + 1])
    if r1 > r0:
        B = ctx.score_block(seqs[r0:r1], seqs[r0:])
    else:
        B = np.zeros((0, n - r0), dtype=np.float32)
    if world == 1:
        return assemble([B], b, n)
    sizes = [(int(b[k + 1]) - int(b[k])) * (n - int(b[k])) for k in range(world)]
    cap = max(sizes) if sizes else 0
    dev = device if device is not None else ("cuda" if torch.cuda.is_available() else "cpu")
    mine = torch.zeros(cap, dtype=torch.float32, device=dev)
    if B.size:
        mine[: B.size] = torch.from_numpy(np.ascontiguousarray(B, dtype=np.float32).ravel()).to(dev)
    parts = [torch.empty(cap, dtype=torch.float32, device=dev) for _ in range(world)]
    dist.all_gather(parts, mine)
    blocks = [p[: sizes[k]].cpu().numpy() for k, p in enumerate(parts)]
    return assemble(blocks, b, n)
