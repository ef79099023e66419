"""Traceback kernels against the oracle restatement of the match/back kernels."""
import os

import numpy as np
import pytest

import oracle_py as O
from mestrado_gb300 import cherries, encode, synth
from fasta import read_fasta

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _rand_set(seed, n, lo, hi, alphabet=b"ARNDCQEGHILKMFPSTWYV"):
    rng = np.random.default_rng(seed)
    letters = np.frombuffer(alphabet, dtype=np.uint8)
    lens = rng.integers(lo, hi + 1, size=n)
    return [letters[rng.integers(0, len(letters), L)].tobytes() for L in lens]


def _check(ctx, seqs, px, py):
    codes, off = encode(seqs)
    out = ctx.align_pairs(codes, off, px, py)
    for (ax, ay, s), i, j in zip(out, px, py):
        rx, ry, rs = O.traceback(seqs[i], seqs[j])
        assert (ax, ay, s) == (rx, ry, rs), (i, j)


def test_random_pairs_short_and_multiband(ctx):
    seqs = _rand_set(5, 30, 1, 700) + _rand_set(6, 4, 1, 20, alphabet=b"ARNDCQEGHILKMFPSTWYVBZX*")
    rng = np.random.default_rng(2)
    px, py = rng.integers(0, len(seqs), 80), rng.integers(0, len(seqs), 80)
    _check(ctx, seqs, px, py)


def test_related_and_identical_pairs(ctx):
    S = synth.family(20, 300, ps=0.1, pi=0.03, seed=8)
    seqs = [S[i] for i in range(len(S))] + [S[0]]
    px = np.arange(0, 20)
    py = np.array(list(range(1, 20)) + [20])
    _check(ctx, seqs, px, py)


@pytest.mark.parametrize("case", ["cfg0", "nj300"])
def test_cherries_of_reference_tree(ctx, case):
    names, seqs = read_fasta(os.path.join(GOLD, case, "input.fasta"))
    rows = [l.split() for l in open(os.path.join(GOLD, case, "joins.txt"))]
    left = np.array([int(r[1]) for r in rows], dtype=np.int32)
    right = np.array([int(r[2]) for r in rows], dtype=np.int32)
    node, l, r = cherries(left, right, len(seqs))
    _check(ctx, seqs, l, r)


def test_device_alignments_rescore_to_their_score(ctx):
    # independent of the flag rules: the path found reproduces the DP score
    from rescore import rescore
    from mestrado_gb300 import encode
    rng = np.random.default_rng(12)
    letters = np.frombuffer(b"ARNDCQEGHILKMFPSTWYV", dtype=np.uint8)
    seqs = [letters[rng.integers(0, 20, rng.integers(1, 700))].tobytes() for _ in range(80)]
    codes, off = encode(seqs)
    px = np.arange(0, 80, 2, dtype=np.int32)
    py = np.arange(1, 80, 2, dtype=np.int32)
    sub = O.blosum()
    for (ax, ay, sc), i, j in zip(ctx.align_pairs(codes, off, px, py), px, py):
        assert ax.replace(b"-", b"") == seqs[i] and ay.replace(b"-", b"") == seqs[j]
        assert rescore(ax, ay, sub) == sc


@pytest.mark.parametrize("lanes", [32, 16, 8])
def test_every_front_width_matches_oracle(lanes):
    # 1, 2 or 4 pairs per warp, bands of 256, 128 or 64 rows: fronts of one
    # warp with different band counts and X lengths, single- and multi-band,
    # related pairs (long diagonal runs) and tiny ones
    from mestrado_gb300 import Context
    seqs = _rand_set(40 + lanes, 40, 1, 700) + _rand_set(41, 6, 1, 9)
    S = synth.family(12, 260, ps=0.1, pi=0.03, seed=lanes)
    seqs += [S[i] for i in range(len(S))]
    rng = np.random.default_rng(lanes)
    n = len(seqs)
    px = np.concatenate([rng.integers(0, n, 70), np.arange(n - 12, n - 1)]).astype(np.int32)
    py = np.concatenate([rng.integers(0, n, 70), np.arange(n - 11, n)]).astype(np.int32)
    with Context(10, 2) as c:
        c.set_trace_lanes(lanes)
        _check(c, seqs, px, py)


def test_trace_lanes_rejects_other_widths(ctx):
    from mestrado_gb300._native import NWGError
    with pytest.raises(NWGError):
        ctx.set_trace_lanes(4)


@pytest.mark.parametrize("go,ge", [(3, 5), (10, 10), (0, 0), (15, 1)])
@pytest.mark.parametrize("lanes", [32, 16])
def test_gap_models_match_oracle(go, ge, lanes):
    # go >= ge takes the one-max F chain (F from max(E, diag + S) of the row
    # above), go < ge the direct recurrence; both give the reference's flags
    from mestrado_gb300 import Context
    seqs = _rand_set(60 + go, 24, 1, 500) + _rand_set(61, 4, 1, 12)
    S = synth.family(10, 200, ps=0.1, pi=0.03, seed=go + 3)
    seqs += [S[i] for i in range(len(S))]
    rng = np.random.default_rng(go * 7 + ge)
    n = len(seqs)
    px = rng.integers(0, n, 40).astype(np.int32)
    py = rng.integers(0, n, 40).astype(np.int32)
    codes, off = encode(seqs)
    with Context(go, ge) as c:
        c.set_trace_lanes(lanes)
        out = c.align_pairs(codes, off, px, py)
    for (ax, ay, s), i, j in zip(out, px, py):
        assert (ax, ay, s) == O.traceback(seqs[i], seqs[j], go, ge), (i, j)
