"""Configuration 3 end to end on the device: 8,000 sequences -> batched
distance matrix -> neighbor joining -> cherry traceback, checked against the
tree the reference's own buildTree made on the same matrix (golden fixture)."""
import hashlib
import json
import os
import time

import numpy as np
import pytest

import oracle_py as O
from mestrado_gb300 import cherries, encode, newick, synth
from test_nj_cpu import golden_joins

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "cfg3")


def test_config3_pipeline_matches_reference_tree(ctx):
    meta = json.load(open(os.path.join(GOLD, "meta.json")))
    S = synth.config(3)
    assert hashlib.sha256(S.residues).hexdigest() == meta["residues_sha256"]
    n = len(S)
    t0 = time.perf_counter()
    D = ctx.score_all(S)
    t1 = time.perf_counter()
    assert hashlib.sha256(D.tobytes()).hexdigest() == meta["D_sha256"]
    joins, st = ctx.nj(D, stats=True)
    t2 = time.perf_counter()
    ref = golden_joins("cfg3")
    assert len(joins) == len(ref) == n - 1
    bad = [k for k, (a, b) in enumerate(zip(joins, ref))
           if (a["node"], a["i"], a["j"], a["len_i"], a["len_j"]) != (b["node"], b["i"], b["j"], b["len_i"], b["len_j"])]
    assert not bad, f"{len(bad)} joins differ, first at step {bad[0]}"
    assert st["ambiguous_steps"] == 0 and st["pq_trigger_open"] == 0
    names = [f">s{i}" for i in range(n)]
    assert newick(joins, names) == open(os.path.join(GOLD, "tree.nwk")).read()
    node, left, right = cherries(joins["i"], joins["j"], n)
    refc = [tuple(int(v) for v in line.split()) for line in open(os.path.join(GOLD, "cherries.txt"))]
    assert refc == list(zip(node.tolist(), left.tolist(), right.tolist()))[: len(refc)]
    codes, off = encode(S)
    t3 = time.perf_counter()
    out = ctx.align_pairs(codes, off, left, right)
    t4 = time.perf_counter()
    for k in range(0, len(out), max(1, len(out) // 150)):
        assert out[k] == O.traceback(S[int(left[k])], S[int(right[k])])
    print(f"\nconfig 3: score {1e3*(t1-t0):.0f} ms, nj {1e3*(t2-t1):.0f} ms (device {st['device_ms']:.0f} ms, "
          f"{st['rebuilds']} rebuilds, {st['tie_steps']} tie steps), traceback of {len(out)} cherries "
          f"{1e3*(t4-t3):.0f} ms")
