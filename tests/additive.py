"""Additive (tree) metrics for neighbor-joining property tests.

A random binary tree with integer branch lengths gives a distance matrix of
path lengths.  Neighbor joining is consistent on such a matrix: every pair
minimising q = d(i,j)(n-2) - T_i - T_j is a cherry of the tree (Studier and
Keppler 1988), so the joins recover the tree's topology whatever the
tie-break.  With integer lengths every value the join loop forms (matrix
updates (D_ik + D_jk - D_ij)/2, row sums, q) is exact in float and double, so
the property holds for the reference's arithmetic too.
"""
import numpy as np


def random_tree_metric(n: int, seed: int, max_len: int = 20):
    """(D, splits): the n x n float32 path-length matrix of a random binary
    tree (clusters merged at random, branch lengths 1..max_len) and the set of
    its non-trivial splits."""
    rng = np.random.default_rng(seed)
    D = np.zeros((n, n), dtype=np.float32)
    clusters = [(np.array([k]), np.zeros(1, dtype=np.int64)) for k in range(n)]
    splits = set()
    while len(clusters) > 1:
        a, b = sorted(rng.choice(len(clusters), size=2, replace=False))
        (la, da), (lb, db) = clusters[a], clusters[b]
        ea, eb = rng.integers(1, max_len + 1, size=2)
        block = (da + ea)[:, None] + (db + eb)[None, :]
        D[np.ix_(la, lb)] = block
        D[np.ix_(lb, la)] = block.T
        leaves = np.concatenate([la, lb])
        depths = np.concatenate([da + ea, db + eb])
        clusters = [c for k, c in enumerate(clusters) if k not in (a, b)] + [(leaves, depths)]
        splits.add(_split(leaves, n))
    return D, {s for s in splits if s is not None}


def _split(leaves, n):
    s = frozenset(int(v) for v in leaves)
    if 0 in s:
        s = frozenset(range(n)) - s
    return s if 1 < len(s) < n - 1 else None


def join_splits(joins, n: int):
    """The non-trivial splits of the tree a join list builds (node n + k joins
    joins[k].i and joins[k].j)."""
    under = {k: [k] for k in range(n)}
    splits = set()
    for k, J in enumerate(joins):
        under[n + k] = under.pop(int(J["i"])) + under.pop(int(J["j"]))
        s = _split(under[n + k], n)
        if s is not None:
            splits.add(s)
    return splits
