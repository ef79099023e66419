"""The oracle's score and traceback restatements against the reference's own
kernel text: NeedlemanWunschGlobalScoreKernel, NeedlemanWunschGlobalMatchKernel
and NeedlemanWunschGlobalBackKernel (NeedlemanWunsch.cu:22-494), compiled
unchanged for the host through oracle/ref_shim/ref_kernels.cpp (make refkern)
and run one pair at a time, with the shim's patches for the shipped defects
(full matrix load, one thread per block) listed in that file.  The matrix is
the reference's own definitions.cuh table.

* scores: every pair of configuration 0 (the diagonal included), 2,000 random
  pairs of lengths 1-900 over the full 24-letter alphabet under five gap
  models (go < ge included), and edge lengths;
* tracebacks: every cherry of configuration 0's guide tree (the reference's
  own buildAlign list, tests/golden/cfg0/cherries.txt) and 300 random pairs.

CPU only; skipped where the reference checkout is absent."""
import ctypes
import os
import subprocess

import numpy as np
import pytest

import oracle_py as O
from mestrado_gb300 import synth
from refsrc import REF, present

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLD = os.path.join(ROOT, "tests", "golden")
P = ctypes.POINTER

pytestmark = pytest.mark.skipif(not present("NeedlemanWunsch.cu"), reason="reference sources not present")

GAPS = [(10, 2), (5, 1), (12, 3), (3, 5), (0, 1)]


@pytest.fixture(scope="module")
def refk():
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "refkern", f"REF={REF}"], check=True)
    L = ctypes.CDLL(os.path.join(ROOT, "oracle", "_ref", "libref_nwkern.so"))
    L.refk_score_pair.argtypes = [P(ctypes.c_int8), ctypes.c_int, P(ctypes.c_int8), ctypes.c_int,
                                  ctypes.c_int, ctypes.c_int]
    L.refk_score_pair.restype = ctypes.c_int
    L.refk_traceback.argtypes = [P(ctypes.c_int8), ctypes.c_int, P(ctypes.c_int8), ctypes.c_int, ctypes.c_int,
                                 ctypes.c_int, ctypes.c_char_p, ctypes.c_char_p, P(ctypes.c_int)]
    L.refk_traceback.restype = ctypes.c_int
    return L


def _ptr(a):
    return a.ctypes.data_as(P(ctypes.c_int8))


def _ref_scores(L, codes, off, pi, pj, go, ge):
    out = np.empty(len(pi), dtype=np.int64)
    for k, (i, j) in enumerate(zip(pi, pj)):
        x, y = codes[off[i]:off[i + 1]], codes[off[j]:off[j + 1]]
        out[k] = L.refk_score_pair(_ptr(x), len(x), _ptr(y), len(y), go, ge)
    return out


def _ref_traceback(L, sx, sy, go=10, ge=2):
    (cx, _), (cy, _) = O.encode([sx]), O.encode([sy])
    bx = ctypes.create_string_buffer(len(sx) + len(sy) + 1)
    by = ctypes.create_string_buffer(len(sx) + len(sy) + 1)
    sc = ctypes.c_int(0)
    k = L.refk_traceback(_ptr(cx), len(sx), _ptr(cy), len(sy), go, ge, bx, by, ctypes.byref(sc))
    assert k == len(bx.value) == len(by.value)
    return bx.value, by.value, sc.value


def _rand_set(seed, n, lo, hi, alphabet=b"ARNDCQEGHILKMFPSTWYVBZX*"):
    rng = np.random.default_rng(seed)
    letters = np.frombuffer(alphabet, dtype=np.uint8)
    lens = rng.integers(lo, hi + 1, size=n)
    return [letters[rng.integers(0, len(letters), L)].tobytes() for L in lens]


def test_config0_scores_equal_reference_kernel(refk):
    S = synth.config(0)
    codes, off = O.encode(S)
    n = len(S)
    pi, pj = np.triu_indices(n)
    ref = _ref_scores(refk, codes, off, pi, pj, 10, 2)
    D = O.score_all(S)
    assert np.array_equal(D[pi, pj], ref.astype(np.float32))
    assert np.array_equal(D, np.load(os.path.join(GOLD, "cfg0", "D.npy")))


@pytest.mark.parametrize("go,ge", GAPS)
def test_random_pairs_equal_reference_kernel(refk, go, ge):
    S = _rand_set(1000 + go * 10 + ge, 120, 1, 900)
    codes, off = O.encode(S)
    rng = np.random.default_rng(go * 100 + ge)
    count = 2000 if (go, ge) == (10, 2) else 400
    pi, pj = rng.integers(0, len(S), count), rng.integers(0, len(S), count)
    ref = _ref_scores(refk, codes, off, pi, pj, go, ge)
    ours = O.score_list(codes, off, pi, pj, go=go, ge=ge, threads=os.cpu_count())
    assert np.array_equal(ours, ref)


def test_edge_lengths_equal_reference_kernel(refk):
    # one residue, strip boundaries of the reference's 12-row (score) and
    # 8-row (match) strips, identical sequences
    base = _rand_set(77, 1, 40, 40)[0]
    S = [b"A", b"W", b"*", base[:11], base[:12], base[:13], base[:7], base[:8], base[:9], base[:24], base, base]
    codes, off = O.encode(S)
    pi, pj = np.meshgrid(np.arange(len(S)), np.arange(len(S)))
    pi, pj = pi.ravel(), pj.ravel()
    ref = _ref_scores(refk, codes, off, pi, pj, 10, 2)
    assert np.array_equal(O.score_list(codes, off, pi, pj), ref)
    for i, j in zip(pi, pj):
        assert O.traceback(S[i], S[j]) == _ref_traceback(refk, S[i], S[j])


def test_config0_cherries_equal_reference_kernels(refk):
    S = synth.config(0)
    rows = [tuple(int(v) for v in line.split()) for line in open(os.path.join(GOLD, "cfg0", "cherries.txt"))
            if line.strip()]
    assert len(rows) > 5
    for _, a, b in rows:
        assert O.traceback(S[a], S[b]) == _ref_traceback(refk, S[a], S[b])


@pytest.mark.parametrize("go,ge", [(10, 2), (4, 1), (3, 5)])
def test_random_tracebacks_equal_reference_kernels(refk, go, ge):
    S = _rand_set(2000 + go, 60, 1, 400)
    rng = np.random.default_rng(go)
    for _ in range(100):
        i, j = rng.integers(0, len(S), 2)
        assert O.traceback(S[i], S[j], go, ge) == _ref_traceback(refk, S[i], S[j], go, ge)
