"""The oracle's model of the reference's join loop (oracle/nj_model.cpp: bins,
bin heaps, candidate list, the eight kept candidates, prediction array) against
the reference's own buildTree, CPU only:

* every golden join list made by the reference (tests/golden/*/joins.txt),
  branch lengths bit for bit, including dup300 (100 sequences three times),
  where the reference's heap order and its cut to eight candidates decide 58
  joins and the exact argmin departs from its tree at join 22;
* fresh tie-heavy matrices handed to the compiled reference (duplicated
  sequences, two to six copies; skipped where the reference checkout is
  absent);
* where the exact-argmin restatement counts no ambiguous step, both give the
  same joins (random families, integer matrices)."""
import hashlib
import json
import os
import subprocess
import tempfile

import numpy as np
import pytest

import oracle_py as O
from additive import random_tree_metric
from fasta import read_fasta
from mestrado_gb300 import newick, synth
from mestrado_gb300._native import JOIN_DTYPE
from refsrc import REF, present
from test_nj_cpu import golden_joins

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLD = os.path.join(ROOT, "tests", "golden")


def _same(j, ref):
    assert len(j) == len(ref)
    for t, (a, b) in enumerate(zip(j, ref)):
        assert (a["node"], a["i"], a["j"]) == (b["node"], b["i"], b["j"]), f"join {t}"
        assert a["len_i"] == b["len_i"] and a["len_j"] == b["len_j"], f"join {t}"


@pytest.mark.parametrize("case", ["cfg0", "nj300", "nj1200", "dup200", "dup300", "tree500"])
def test_model_equals_reference_golden(case):
    d = os.path.join(GOLD, case)
    names, seqs = read_fasta(os.path.join(d, "input.fasta"))
    if case == "tree500":
        D = random_tree_metric(len(seqs), 22)[0]
    else:
        D = O.score_all(seqs, threads=os.cpu_count() or 2)
    meta = json.load(open(os.path.join(d, "meta.json")))
    assert hashlib.sha256(np.ascontiguousarray(D).tobytes()).hexdigest() == meta["D_sha256"]
    joins, _ = O.nj_model(D)
    _same(joins, golden_joins(case))
    j = np.zeros(len(joins), dtype=np.dtype(JOIN_DTYPE))
    for k in joins.dtype.names:
        j[k] = joins[k]
    assert newick(j, names) == open(os.path.join(d, "tree.nwk")).read()


def _copies(k, c, seed, L=80):
    S = synth.family(k, L, ps=0.05, pi=0.005, seed=seed).subset([i for i in range(k) for _ in range(c)])
    return S, O.score_all(S, threads=os.cpu_count() or 2)


@pytest.fixture(scope="module")
def ref_nj():
    if not present():
        pytest.skip("reference sources not present")
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref", f"REF={REF}"], check=True)
    return os.path.join(ROOT, "oracle", "_ref", "ref_nj")


def _run_ref(exe, S, D):
    with tempfile.TemporaryDirectory() as td:
        fasta = os.path.join(td, "input.fasta")
        S.to_fasta(fasta)
        dpath = os.path.join(td, "D.f32")
        np.ascontiguousarray(D, dtype=np.float32).tofile(dpath)
        subprocess.run([exe, fasta, os.path.join(td, "out")], check=True, cwd=td,
                       env=dict(os.environ, NWG_REF_D=dpath), stdout=subprocess.DEVNULL)
        rows = [r.split() for r in open(os.path.join(td, "out.joins")) if r.strip()]
    return [(int(r[0]), int(r[1]), int(r[2]), float.fromhex(r[3]), float.fromhex(r[4])) for r in rows]


@pytest.mark.parametrize("k,c,seed", [(100, 3, 31), (60, 4, 5), (40, 6, 7), (150, 3, 9), (200, 5, 8), (10, 3, 2),
                                      (300, 2, 4), (90, 2, 12)])
def test_model_equals_reference_on_duplicates(ref_nj, k, c, seed):
    S, D = _copies(k, c, seed)
    ref = _run_ref(ref_nj, S, D)
    joins, _ = O.nj_model(D)
    assert len(joins) == len(ref)
    for t, (a, r) in enumerate(zip(joins, ref)):
        assert (int(a["node"]), int(a["i"]), int(a["j"]), float(a["len_i"]), float(a["len_j"])) == r, f"join {t}"


@pytest.mark.parametrize("kind,seed", [("family", 1), ("family", 2), ("family", 3), ("integer", 4), ("integer", 5)])
def test_model_equals_exact_argmin_where_unambiguous(kind, seed):
    rng = np.random.default_rng(seed)
    if kind == "family":
        S = synth.family(int(rng.integers(40, 400)), 120, ps=0.1, pi=0.01, seed=seed)
        D = O.score_all(S, threads=os.cpu_count() or 2)
    else:
        n = int(rng.integers(40, 300))
        M = rng.integers(0, 1000, size=(n, n)).astype(np.float32)
        D = np.triu(M, 1) + np.triu(M, 1).T
    ex, st = O.nj(D)
    assert st["ambiguous_steps"] == 0
    joins, _ = O.nj_model(D)
    for a, b in zip(joins, ex):
        assert (a["i"], a["j"], a["q"], a["ti"], a["tj"], a["len_i"], a["len_j"]) == \
               (b["i"], b["j"], b["q"], b["ti"], b["tj"], b["len_i"], b["len_j"])


def test_exact_argmin_flags_where_reference_departs():
    # dup300: the exact argmin counts ambiguous steps, and its tree departs
    # from the reference's (golden) at join 22, where the model follows it
    d = os.path.join(GOLD, "dup300")
    _, seqs = read_fasta(os.path.join(d, "input.fasta"))
    D = O.score_all(seqs, threads=os.cpu_count() or 2)
    ex, st = O.nj(D)
    ref = golden_joins("dup300")
    assert st["ambiguous_steps"] > 0
    first = next(t for t in range(len(ref)) if (ex[t]["i"], ex[t]["j"]) != (ref[t]["i"], ref[t]["j"]))
    assert first == 22
    joins, _ = O.nj_model(D)
    _same(joins, ref)
