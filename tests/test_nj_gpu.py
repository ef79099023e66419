"""Device neighbor joining against the reference's own buildTree (golden join
lists made by SpeciesBlock.cpp compiled through the one-rank MPI shim) and
against the oracle restatement."""
import hashlib
import json
import os

import numpy as np
import pytest

import oracle_py as O
from mestrado_gb300 import newick, synth
from fasta import read_fasta
from test_nj_cpu import golden_joins

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _same(j, ref):
    assert len(j) == len(ref)
    for a, b in zip(j, ref):
        assert (a["node"], a["i"], a["j"]) == (b["node"], b["i"], b["j"])
        assert a["len_i"] == b["len_i"] and a["len_j"] == b["len_j"]


@pytest.mark.parametrize("case", ["cfg0", "nj300", "nj1200", "dup200", "tree500"])
def test_device_nj_matches_reference_tree(ctx, case):
    # dup200 and tree500: most of the reference's tie-break decisions
    d = os.path.join(GOLD, case)
    names, seqs = read_fasta(os.path.join(d, "input.fasta"))
    if case == "tree500":
        from additive import random_tree_metric
        D = random_tree_metric(len(seqs), 22)[0]
    else:
        D = ctx.score_all(seqs)
    meta = json.load(open(os.path.join(d, "meta.json")))
    assert hashlib.sha256(D.tobytes()).hexdigest() == meta["D_sha256"]
    joins, st = ctx.nj(D, stats=True)
    _same(joins, golden_joins(case))
    assert newick(joins, names) == open(os.path.join(d, "tree.nwk")).read()
    assert st["ambiguous_steps"] == 0 and st["pq_trigger_open"] == 0
    assert st["reference_identical"] == 1


def test_device_nj_flags_trees_the_reference_may_build_differently(ctx):
    # dup300: 100 sequences three times.  The reference's bin heaps and its
    # cut to eight candidates decide 58 joins, and its tree departs from the
    # exact argmin at join 22 (tests/test_nj_model_cpu.py).  The device
    # returns the exact-argmin tree, counts the ambiguous steps and reports
    # the tree as not guaranteed to be the reference's.
    d = os.path.join(GOLD, "dup300")
    _, seqs = read_fasta(os.path.join(d, "input.fasta"))
    D = ctx.score_all(seqs)
    joins, st = ctx.nj(D, stats=True)
    oj, ost = O.nj(D)
    for a, b in zip(joins, oj):
        assert (a["i"], a["j"], a["len_i"], a["len_j"], a["q"]) == (b["i"], b["j"], b["len_i"], b["len_j"], b["q"])
    assert st["ambiguous_steps"] == ost["ambiguous_steps"] > 0
    assert st["reference_identical"] == 0
    ref = golden_joins("dup300")
    assert [(int(a["i"]), int(a["j"])) for a in joins[:22]] == [(int(b["i"]), int(b["j"])) for b in ref[:22]]
    assert (int(joins[22]["i"]), int(joins[22]["j"])) != (int(ref[22]["i"]), int(ref[22]["j"]))


@pytest.mark.parametrize("seed,n", [(1, 2), (2, 3), (3, 17), (4, 64), (5, 257), (6, 600)])
def test_device_nj_matches_oracle(ctx, seed, n):
    S = synth.family(n, 90, ps=0.1, pi=0.01, seed=seed)
    D = ctx.score_all(S)
    joins, st = ctx.nj(D, stats=True)
    oj, ost = O.nj(D)
    assert len(joins) == len(oj)
    for a, b in zip(joins, oj):
        assert (a["i"], a["j"], a["node"], a["n"]) == (b["i"], b["j"], b["node"], b["n"])
        assert (a["len_i"], a["len_j"], a["q"], a["ti"], a["tj"]) == (b["len_i"], b["len_j"], b["q"], b["ti"], b["tj"])
    assert st["ambiguous_steps"] == ost["ambiguous_steps"]
    assert st["tie_steps"] == ost["tie_steps"]
    assert st["rebuilds"] == ost["rebuilds"]


def test_device_nj_ties_and_duplicates(ctx):
    # identical sequences and a small integer matrix with many exact ties
    S = synth.family(40, 60, ps=0.02, pi=0.0, seed=9)
    seqs = [S[i] for i in range(len(S))] + [S[0], S[0], S[1]]
    D = ctx.score_all(seqs)
    joins, st = ctx.nj(D, stats=True)
    oj, ost = O.nj(D)
    for a, b in zip(joins, oj):
        assert (a["i"], a["j"], a["len_i"], a["len_j"]) == (b["i"], b["j"], b["len_i"], b["len_j"])
    assert st["tie_steps"] == ost["tie_steps"] and st["ambiguous_steps"] == ost["ambiguous_steps"]
    assert st["reference_identical"] == (1 if st["ambiguous_steps"] == 0 else 0)
    rng = np.random.default_rng(0)
    M = rng.integers(0, 5, size=(30, 30)).astype(np.float32)
    M = np.triu(M, 1) + np.triu(M, 1).T
    joins, st = ctx.nj(M, stats=True)
    oj, ost = O.nj(M)
    for a, b in zip(joins, oj):
        assert (a["i"], a["j"], a["len_i"], a["len_j"]) == (b["i"], b["j"], b["len_i"], b["len_j"])
    assert st["ambiguous_steps"] == ost["ambiguous_steps"]


_BOTH_PATHS = """
import sys, numpy as np; sys.path.insert(0, 'tests'); import oracle_py as O
from mestrado_gb300 import Context, synth
c = Context(10, 2)

def check(D, exact_q=True):
    j, st = c.nj(D, stats=True)
    oj, ost = O.nj(D)
    assert len(j) == len(oj)
    assert st['rebuilds'] == ost['rebuilds'] and st['tie_steps'] == ost['tie_steps']
    assert st['ambiguous_steps'] == ost['ambiguous_steps']
    for a, b in zip(j, oj):
        assert (a['i'], a['j'], a['node'], a['n'], a['len_i'], a['len_j']) == \
            (b['i'], b['j'], b['node'], b['n'], b['len_i'], b['len_j'])
        assert not exact_q or (a['q'], a['ti'], a['tj']) == (b['q'], b['ti'], b['tj'])

for seed, n in ((11, 450), (12, 640), (2, 3), (3, 17), (4, 205)):
    check(c.score_all(synth.family(n, 90, ps=0.1, pi=0.01, seed=seed)))
# identical sequences (exact ties) and a small integer matrix with many ties:
# the pick falls back to the candidate scan
S = synth.family(40, 60, ps=0.02, pi=0.0, seed=9)
check(c.score_all([S[i] for i in range(len(S))] + [S[0], S[0], S[1]]))
rng = np.random.default_rng(0)
M = rng.integers(0, 5, size=(30, 30)).astype(np.float32)
check(np.triu(M, 1) + np.triu(M, 1).T)
M = rng.integers(0, 3, size=(300, 300)).astype(np.float32)
check(np.triu(M, 1) + np.triu(M, 1).T)
# tens of thousands of exactly tied pairs per join (the pick from per-CTA
# firsts and a counting scan): 420 copies of one sequence, three sequences
# 140 times each, a constant matrix
check(c.score_all([S[5]] * 420))
check(c.score_all([S[k] for k in (1, 2, 3) for _ in range(140)]))
M = np.full((400, 400), 5.0, dtype=np.float32)
np.fill_diagonal(M, 0.0)
check(M)
print('ok')
"""


# the three launch forms, selected by the size thresholds
_FORMS = {
    "cta": {},                                                          # defaults: one CTA up to 160 taxa
    "smem": {"NWG_NJ_CTA_MAX_N": "0"},                                  # matrix in a cluster's shared memory
    "cluster": {"NWG_NJ_CTA_MAX_N": "0", "NWG_NJ_SMEM_MAX_N": "0",
                "NWG_NJ_CLUSTER_MAX_N": "100000"},                      # one cluster over L2
    "full_gpu": {"NWG_NJ_CLUSTER_MAX_N": "0"},                          # cooperative launch over every SM
}


@pytest.mark.parametrize("path", list(_FORMS))
def test_every_nj_form_matches_oracle(path):
    # every launch form gives the oracle's joins on families, tiny n,
    # duplicates and tie-heavy integer matrices; run in a child process so
    # that the thresholds apply from the library's first use
    import subprocess
    import sys
    env = dict(os.environ, **_FORMS[path])
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    r = subprocess.run([sys.executable, "-c", _BOTH_PATHS], cwd=root, env=env, capture_output=True, text=True,
                       timeout=900)
    assert r.returncode == 0 and r.stdout.strip().endswith("ok"), r.stdout + r.stderr


@pytest.mark.parametrize("path", ["smem", "cluster", "full_gpu"])
@pytest.mark.parametrize("case", ["cfg0", "nj300", "nj1200"])
def test_every_nj_form_matches_reference_tree(case, path):
    # the golden reference trees through the forms the default sizes do not
    # pick (the default run covers one CTA up to 160 taxa and a cluster's
    # shared memory up to 768)
    import subprocess
    import sys
    code = (
        "import sys, json, os; sys.path.insert(0, 'tests')\n"
        "from mestrado_gb300 import Context, newick\n"
        "from fasta import read_fasta\n"
        "from test_nj_cpu import golden_joins\n"
        f"d = os.path.join('tests', 'golden', '{case}')\n"
        "names, seqs = read_fasta(os.path.join(d, 'input.fasta'))\n"
        "c = Context(10, 2)\n"
        "j, st = c.nj(c.score_all(seqs), stats=True)\n"
        f"ref = golden_joins('{case}')\n"
        "assert len(j) == len(ref)\n"
        "for a, b in zip(j, ref):\n"
        "    assert (a['node'], a['i'], a['j'], a['len_i'], a['len_j']) == "
        "(b['node'], b['i'], b['j'], b['len_i'], b['len_j'])\n"
        "assert newick(j, names) == open(os.path.join(d, 'tree.nwk')).read()\n"
        "print('ok')\n")
    env = dict(os.environ, **_FORMS[path])
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    r = subprocess.run([sys.executable, "-c", code], cwd=root, env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0 and r.stdout.strip().endswith("ok"), r.stdout + r.stderr


def test_grid_barrier_timeout_is_reported_and_context_recovers(ctx):
    # failure detection without a GPU fault: the first grid barrier of the
    # full-GPU form is made unreachable (its arrival count starts one short),
    # every CTA gives up after the spin limit (about two seconds), the call
    # returns a CUDA status, and the same context then joins correctly
    from mestrado_gb300 import NWGError
    from mestrado_gb300._native import NWG_ERR_CUDA
    S = synth.family(2100, 36, ps=0.1, pi=0.01, seed=17)   # above the cluster threshold: the full-GPU form
    D = ctx.score_all(S)
    os.environ["NWG_NJ_INJECT_BARRIER_STALL"] = "1"
    try:
        with pytest.raises(NWGError) as e:
            ctx.nj(D)
        assert e.value.status == NWG_ERR_CUDA
    finally:
        del os.environ["NWG_NJ_INJECT_BARRIER_STALL"]
    joins = ctx.nj(D)
    oj, _ = O.nj(D)
    for a, b in zip(joins, oj):
        assert (a["i"], a["j"], a["len_i"], a["len_j"]) == (b["i"], b["j"], b["len_i"], b["len_j"])
