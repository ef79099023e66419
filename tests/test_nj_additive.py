"""Neighbor joining on tree metrics: the joins recover the tree (NJ's
consistency), in the oracle on the CPU and in every launch form of the device,
which also equals the oracle join for join."""
import numpy as np
import pytest

import oracle_py as O
from additive import join_splits, random_tree_metric


@pytest.mark.parametrize("n,seed", [(4, 1), (5, 2), (10, 3), (64, 4), (200, 5)])
def test_oracle_nj_recovers_tree_metrics(n, seed):
    D, splits = random_tree_metric(n, seed)
    assert np.array_equal(D, D.T) and not np.diag(D).any()
    joins, _ = O.nj(D)
    assert len(joins) == n - 1
    assert join_splits(joins, n) == splits


@pytest.mark.gpu
@pytest.mark.parametrize("n,seed", [(100, 6), (500, 7), (1500, 8), (2100, 9)])
def test_device_nj_recovers_tree_metrics(ctx, n, seed):
    # one size per launch form: one CTA, a cluster's shared memory, a cluster
    # over L2, the whole GPU
    D, splits = random_tree_metric(n, seed)
    joins, st = ctx.nj(D, stats=True)
    oj, ost = O.nj(D)
    for a, b in zip(joins, oj):
        assert (a["i"], a["j"], a["node"], a["len_i"], a["len_j"], a["q"]) == \
            (b["i"], b["j"], b["node"], b["len_i"], b["len_j"], b["q"])
    assert st["tie_steps"] == ost["tie_steps"] and st["ambiguous_steps"] == ost["ambiguous_steps"]
    assert join_splits(joins, n) == splits
