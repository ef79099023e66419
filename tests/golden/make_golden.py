"""Generate the golden fixtures of tests/golden/ (run in a checkout that has
the reference sources; the GPU machine never runs this).

For each case: the synthetic input (FASTA, from the seeded generator), the
distance matrix the reference's recurrence gives (oracle restatement,
sha256 + a sample), and what the reference's OWN neighbor-joining code
produces on it -- SpeciesBlock.cpp/TreeNode.cpp compiled unchanged through the
one-rank MPI shim (oracle/_ref/ref_nj): every join, both branch lengths as
exact doubles, the Newick .tree text and the cherry list buildAlign hands to
AlignmentMatch.

    python tests/golden/make_golden.py            # all cases
    python tests/golden/make_golden.py cfg0       # one case
"""
from __future__ import annotations

import hashlib
import json
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

from mestrado_gb300 import synth  # noqa: E402
import oracle_py  # noqa: E402
from additive import random_tree_metric  # noqa: E402

REF = os.environ.get("NWG_REFERENCE") or os.path.normpath(os.path.join(ROOT, os.pardir, "reference"))

CASES = {
    # benchmark configuration 0: 64 sequences, one family, root 300
    "cfg0": lambda: synth.config(0),
    # 300 sequences: crosses the first row-sum rebuild (after 201 joins)
    "nj300": lambda: synth.family(300, 120, ps=0.05, pi=0.005, seed=11),
    # 1200 short sequences in 6 families: rebuilds at 600, 300, 150 active
    "nj1200": lambda: synth.family(200, 60, ps=0.08, pi=0.005, families=6, seed=12),
    # benchmark configuration 3: 8000 sequences, 40 families, uniform root
    # lengths 100-300 (integer-only generator path: regenerated identically
    # on x86-64 and aarch64, so the input itself is not stored)
    "cfg3": lambda: synth.config(3),
    # 100 sequences, each twice: 91 joins decided by the tie-break alone
    "dup200": lambda: synth.family(100, 80, ps=0.05, pi=0.005, seed=31).subset(
        [k for k in range(100) for _ in range(2)]),
    # 100 sequences, each three times: the reference's bin heaps and its cut to
    # eight candidates decide 58 joins (the exact argmin departs at join 22)
    "dup300": lambda: synth.family(100, 80, ps=0.05, pi=0.005, seed=31).subset(
        [k for k in range(100) for _ in range(3)]),
    # a tree metric (below) on 500 taxa: integer path lengths, exact q ties;
    # the sequences only give the FASTA its names
    "tree500": lambda: synth.family(500, 30, ps=0.05, pi=0.0, seed=13),
}
NO_INPUT = {"cfg3"}
# cases whose matrix is not the sequences' scores
MATRIX = {
    "tree500": lambda S: random_tree_metric(len(S), 22)[0],
}


def build_ref():
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref", f"REF={REF}"], check=True)
    return os.path.join(ROOT, "oracle", "_ref", "ref_nj")


def make(name: str) -> None:
    S = CASES[name]()
    n = len(S)
    out = os.path.join(HERE, name)
    os.makedirs(out, exist_ok=True)
    fasta = os.path.join(out, "input.fasta")
    S.to_fasta(fasta)
    keep_input = name not in NO_INPUT
    D = MATRIX[name](S) if name in MATRIX else oracle_py.score_all(S, threads=os.cpu_count() or 4)
    ref = build_ref()
    with tempfile.TemporaryDirectory() as td:
        dpath = os.path.join(td, "D.f32")
        D.tofile(dpath)
        env = dict(os.environ, NWG_REF_D=dpath)
        subprocess.run([ref, fasta, os.path.join(td, "out")], check=True, cwd=td, env=env,
                       stdout=subprocess.DEVNULL)
        Dref = np.fromfile(os.path.join(td, "out.D"), dtype=np.float32).reshape(n, n)
        assert np.array_equal(Dref, D)
        with open(os.path.join(td, "out.joins")) as f:
            joins = f.read()
        with open(os.path.join(td, "input.tree")) as f:
            tree = f.read()
        with open(os.path.join(td, "out.cherries")) as f:
            cherries = f.read()
    with open(os.path.join(out, "joins.txt"), "w") as f:
        f.write(joins)
    with open(os.path.join(out, "tree.nwk"), "w") as f:
        f.write(tree)
    with open(os.path.join(out, "cherries.txt"), "w") as f:
        f.write(cherries)
    rng = np.random.default_rng(5)
    idx = rng.integers(0, n, size=(min(4000, n * n), 2))
    meta = {
        "n": n,
        "cells": S.cells(),
        "D_sha256": hashlib.sha256(np.ascontiguousarray(D).tobytes()).hexdigest(),
        "D_sample": [[int(i), int(j), float(D[i, j])] for i, j in idx[:2000]],
        "lengths_sha256": hashlib.sha256(S.lengths.astype(np.int64).tobytes()).hexdigest(),
        "residues_sha256": hashlib.sha256(S.residues).hexdigest(),
        "generator": "see the CASES table of make_golden.py",
    }
    if n <= 128:
        np.save(os.path.join(out, "D.npy"), D)
    if not keep_input:
        os.remove(fasta)
    with open(os.path.join(out, "meta.json"), "w") as f:
        json.dump(meta, f)
    print(name, n, "joins", joins.count("\n"), flush=True)


if __name__ == "__main__":
    for name in (sys.argv[1:] or list(CASES)):
        make(name)
