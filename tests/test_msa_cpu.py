"""The oracle's progressive alignment (this library's definition; the
reference's computeMSA is an empty loop): two sequences give the pairwise
traceback exactly, every row is its sequence with gaps, and columns are never
all gaps."""
import numpy as np
import pytest

import oracle_py as O
from mestrado_gb300 import synth


def _rand(seed, n, lo, hi):
    rng = np.random.default_rng(seed)
    letters = np.frombuffer(b"ARNDCQEGHILKMFPSTWYV", dtype=np.uint8)
    return [letters[rng.integers(0, 20, rng.integers(lo, hi + 1))].tobytes() for _ in range(n)]


@pytest.mark.parametrize("seed", range(6))
def test_two_sequences_equal_pairwise_traceback(seed):
    x, y = _rand(seed, 2, 1, 120)
    rows = O.msa([x, y], [0], [1])
    ax, ay, _ = O.traceback(x, y)
    assert rows == [ax, ay]


def _caterpillar(n):
    left, right = [0], [1]
    for k in range(1, n - 1):
        left.append(k + 1)
        right.append(n + k - 1)
    return left, right


@pytest.mark.parametrize("tree", ["balanced", "caterpillar"])
def test_rows_are_the_sequences_with_gaps(tree):
    seqs = _rand(11, 17, 5, 80)
    n = len(seqs)
    if tree == "caterpillar":
        left, right = _caterpillar(n)
    else:
        from mestrado_gb300._native import JOIN_DTYPE
        D = O.score_all(seqs)
        j, _ = O.nj(D)
        left, right = j["i"], j["j"]
    rows = O.msa(seqs, left, right)
    L = len(rows[0])
    assert all(len(r) == L for r in rows)
    for r, s in zip(rows, seqs):
        assert r.replace(b"-", b"") == s
    cols = np.frombuffer(b"".join(rows), dtype=np.uint8).reshape(n, L)
    assert not np.any(np.all(cols == ord("-"), axis=0))
