"""Progressive alignment on the device against the oracle's restatement
(nwo_msa): pairs (which must equal the cherry traceback), neighbor-joining
and caterpillar trees, bands longer than one strip, other gap penalties, and
configuration 0 along the reference's own tree."""
import os

import numpy as np
import pytest

import oracle_py as O
from mestrado_gb300 import Context, synth
from fasta import read_fasta
from test_nj_cpu import golden_joins

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _rand(seed, n, lo, hi):
    rng = np.random.default_rng(seed)
    letters = np.frombuffer(b"ARNDCQEGHILKMFPSTWYV", dtype=np.uint8)
    return [letters[rng.integers(0, 20, rng.integers(lo, hi + 1))].tobytes() for _ in range(n)]


def _caterpillar(n):
    left, right = [0], [1]
    for k in range(1, n - 1):
        left.append(k + 1)
        right.append(n + k - 1)
    return left, right


@pytest.mark.parametrize("seed", range(5))
def test_pairs_equal_cherry_traceback(ctx, seed):
    x, y = _rand(seed, 2, 1, 600)
    rows = ctx.msa([x, y], [0], [1])
    assert rows == O.msa([x, y], [0], [1])
    from mestrado_gb300 import encode
    codes, off = encode([x, y])
    (ax, ay, _), = ctx.align_pairs(codes, off, [0], [1])
    assert rows == [ax, ay]


@pytest.mark.parametrize("seed,n,lo,hi,tree", [(1, 17, 5, 80, "nj"), (2, 30, 50, 200, "nj"),
                                               (3, 12, 20, 120, "caterpillar"), (4, 6, 260, 700, "nj"),
                                               (5, 9, 300, 560, "caterpillar")])
def test_trees_match_oracle(ctx, seed, n, lo, hi, tree):
    seqs = _rand(seed, n, lo, hi)
    if tree == "nj":
        j = ctx.nj(ctx.score_all(seqs))
        left, right = j["i"], j["j"]
    else:
        left, right = _caterpillar(n)
    rows = ctx.msa(seqs, left, right)
    assert rows == O.msa(seqs, left, right)
    for r, s in zip(rows, seqs):
        assert r.replace(b"-", b"") == s


def test_other_penalties_match_oracle():
    seqs = [synth.family(14, 150, ps=0.1, pi=0.02, seed=8)[i] for i in range(14)]
    with Context(4, 1) as c:
        j = c.nj(c.score_all(seqs))
        assert c.msa(seqs, j["i"], j["j"]) == O.msa(seqs, j["i"], j["j"], go=4, ge=1)


def test_config0_along_reference_tree(ctx):
    names, seqs = read_fasta(os.path.join(GOLD, "cfg0", "input.fasta"))
    ref = golden_joins("cfg0")
    rows, st = ctx.msa(seqs, ref["i"], ref["j"], stats=True)
    assert rows == O.msa(seqs, ref["i"], ref["j"])
    assert st["cells"] > 0 and st["kernel_ms"] > 0
