"""Parity on the headline workload, configuration 2 at full size: 10,000
sequences in 50 families (root lengths lognormal, median 350, sigma 0.6;
lengths 97 to 1,738 with the generator's seed), 50,005,000 pairs with the
diagonal.  The batched persistent form (int16x2 lanes, autotuned templates,
CUDA graph) must give the plain form's matrix entry for entry, and both must
equal the oracle on

* every pair of the family with the longest sequences (19,900 pairs of about
  1,600 residues each: the longest bands and the largest scores), and
* a length-stratified sample: 400 random pairs from each pair of length
  deciles (55 decile pairs, 22,000 pairs), plus every 50th diagonal entry.

Every sequence of this workload is shorter than 2,976 residues, so all of its
int16 pairs are inside the guarded range by length alone; the optimistic
int16 region and the int32 re-run are covered by
test_score_gpu.py::test_overflow_guard_routes_to_int32."""
import os

import numpy as np
import pytest

import oracle_py as O
from mestrado_gb300 import MODE_BATCHED, MODE_PLAIN, encode, synth

pytestmark = pytest.mark.gpu


def test_config2_full_matrix_batched_equals_plain_and_oracle(ctx):
    S = synth.config(2)
    n = len(S)
    assert n == 10000
    codes, off = encode(S)
    L = np.diff(off)
    Db, st = ctx.score_all(codes=codes, offsets=off, mode=MODE_BATCHED, stats=True)
    assert st["pairs"] == n * (n + 1) // 2
    assert np.array_equal(Db, Db.T)
    Dp = ctx.score_all(codes=codes, offsets=off, mode=MODE_PLAIN)
    assert np.array_equal(Db, Dp)
    del Dp

    fam = np.arange(n) // 200
    longest = int(np.argmax([L[fam == f].mean() for f in range(50)]))
    idx = np.where(fam == longest)[0]
    a, b = np.triu_indices(len(idx), 1)
    pi, pj = [idx[a]], [idx[b]]
    rng = np.random.default_rng(2)
    order = np.argsort(L, kind="stable")
    dec = np.array_split(order, 10)
    for i in range(10):
        for j in range(i, 10):
            pi.append(rng.choice(dec[i], 400))
            pj.append(rng.choice(dec[j], 400))
    diag = np.arange(0, n, 50)
    pi.append(diag)
    pj.append(diag)
    pi, pj = np.concatenate(pi), np.concatenate(pj)
    assert len(pi) >= 19900 + 22000
    ref = O.score_list(codes, off, pi, pj, threads=os.cpu_count())
    got = Db[pi, pj]
    bad = np.nonzero(got != ref.astype(np.float32))[0]
    assert bad.size == 0, [(int(pi[k]), int(pj[k]), float(got[k]), int(ref[k])) for k in bad[:5]]
