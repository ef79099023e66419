"""The oracle itself: hand-derived known answers and the golden fixtures made
by the reference's own neighbor-joining code (CPU only)."""
import hashlib
import json
import os

import numpy as np
import pytest

import oracle_py as O
from mestrado_gb300 import synth

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def test_known_answers_score():
    # Worked by hand from NeedlemanWunsch.cu:22-161 with go=10, ge=2, BLOSUM62.
    assert O.score_pair(b"A", b"A") == 4
    # trailing end gap (original orientation) costs ge, no open: 4 - 2
    assert O.score_pair(b"AW", b"A") == 2
    # leading W either gapped (-10 + 4) or mismatched with a cheap trailing gap (-3 - 2)
    assert O.score_pair(b"WA", b"A") == -5
    # three trailing end gaps: 4 - 3*2
    assert O.score_pair(b"AAAA", b"A") == -2
    assert O.score_pair(b"W", b"W") == 11


def _gotoh_textbook(x: bytes, y: bytes, go=10, ge=2):
    """Independent small-case restatement: full matrices, reversed inputs."""
    sub = O.blosum().reshape(24, 24)
    order = "ARNDCQEGHILKMFPSTWYVBZX*"
    X = [order.index(ch) for ch in x.decode()[::-1]]
    Y = [order.index(ch) for ch in y.decode()[::-1]]
    n, m = len(X), len(Y)
    NEG = -32768 + ge
    H = [[0] * (n + 1) for _ in range(m + 1)]
    E = [[NEG] * (n + 1) for _ in range(m + 1)]
    F = [[NEG] * (n + 1) for _ in range(m + 1)]
    for c in range(1, n + 1):
        H[0][c] = -ge * c
    for r in range(1, m + 1):
        H[r][0] = -ge * r
        for c in range(1, n + 1):
            F[r][c] = max(F[r - 1][c] - ge, H[r - 1][c] - go)
            E[r][c] = max(E[r][c - 1] - ge, H[r][c - 1] - go)
            H[r][c] = max(E[r][c], F[r][c], H[r - 1][c - 1] + int(sub[Y[r - 1], X[c - 1]]))
    return H[m][n]


@pytest.mark.parametrize("seed", range(6))
def test_score_matches_textbook_dp(seed):
    rng = np.random.default_rng(seed)
    letters = np.frombuffer(b"ARNDCQEGHILKMFPSTWYVBZX*", dtype=np.uint8)
    for _ in range(20):
        lx, ly = rng.integers(1, 40, size=2)
        x = letters[rng.integers(0, 24, lx)].tobytes()
        y = letters[rng.integers(0, 24, ly)].tobytes()
        assert O.score_pair(x, y) == _gotoh_textbook(x, y)
        assert O.score_pair(x, y) == O.score_pair(y, x)


@pytest.mark.parametrize("go,ge", [(5, 1), (11, 1), (20, 5), (2, 3), (0, 0)])
def test_score_matches_textbook_dp_other_penalties(go, ge):
    # the gap model beyond 10/2, including an extension dearer than an
    # opening and no gap cost at all
    rng = np.random.default_rng(go * 31 + ge)
    letters = np.frombuffer(b"ARNDCQEGHILKMFPSTWYVBZX*", dtype=np.uint8)
    for _ in range(30):
        lx, ly = rng.integers(1, 40, size=2)
        x = letters[rng.integers(0, 24, lx)].tobytes()
        y = letters[rng.integers(0, 24, ly)].tobytes()
        assert O.score_pair(x, y, go, ge) == _gotoh_textbook(x, y, go, ge)


def test_traceback_known_answers():
    assert O.traceback(b"A", b"A") == (b"A", b"A", 4)
    assert O.traceback(b"AW", b"A") == (b"AW", b"A-", 2)
    ax, ay, s = O.traceback(b"A", b"AA")
    assert (ax, ay) == (b"A-", b"AA")


def test_traceback_is_an_alignment():
    S = synth.family(12, 80, ps=0.2, pi=0.05, seed=3)
    for i in range(0, 12, 2):
        x, y = S[i], S[i + 1]
        ax, ay, s = O.traceback(x, y)
        assert len(ax) == len(ay)
        assert ax.replace(b"-", b"") == x[: len(ax.replace(b"-", b""))]
        assert ay.replace(b"-", b"") == y[: len(ay.replace(b"-", b""))]
        assert s == O.score_pair(x, y)


def _load_joins(path):
    rows = []
    for line in open(path):
        k, l, r, ll, lr = line.split()
        rows.append((int(k), int(l), int(r), float.fromhex(ll), float.fromhex(lr)))
    return rows


def golden_matrix(case, seqs):
    """The matrix a golden case's joins were made on: the sequences' scores,
    or for tree500 the tree metric of tests/additive.py (seed 22)."""
    if case == "tree500":
        from additive import random_tree_metric
        return random_tree_metric(len(seqs), 22)[0]
    return O.score_all(seqs, threads=os.cpu_count() or 2)


@pytest.mark.parametrize("case", ["cfg0", "nj300", "nj1200", "dup200", "tree500"])
def test_oracle_nj_matches_reference_golden(case):
    # dup200 (every sequence twice) and tree500 (integer tree metric) pin the
    # tie-break: 91 and 16 of their joins are exact ties in q
    d = os.path.join(GOLD, case)
    meta = json.load(open(os.path.join(d, "meta.json")))
    from fasta import read_fasta
    names, seqs = read_fasta(os.path.join(d, "input.fasta"))
    D = golden_matrix(case, seqs)
    assert hashlib.sha256(D.tobytes()).hexdigest() == meta["D_sha256"]
    joins, st = O.nj(D)
    if case in ("dup200", "tree500"):
        assert st["tie_steps"] > 10
    ref = _load_joins(os.path.join(d, "joins.txt"))
    assert len(ref) == len(joins)
    for r, j in zip(ref, joins):
        assert (r[0], r[1], r[2]) == (j["node"], j["i"], j["j"])
        assert r[3] == j["len_i"] and r[4] == j["len_j"]
    assert st["ambiguous_steps"] == 0 and st["pq_trigger_open"] == 0


def test_golden_inputs_regenerate():
    # the generator's integer-only path is platform independent
    meta = json.load(open(os.path.join(GOLD, "cfg0", "meta.json")))
    S = synth.config(0)
    assert hashlib.sha256(S.residues).hexdigest() == meta["residues_sha256"]
