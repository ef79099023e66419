"""Host side of the NJ path: the Newick text from a join list (CPU only)."""
import os

import numpy as np
import pytest

from mestrado_gb300 import newick
from mestrado_gb300._native import JOIN_DTYPE
from fasta import read_fasta

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def golden_joins(case):
    rows = [l.split() for l in open(os.path.join(GOLD, case, "joins.txt"))]
    j = np.zeros(len(rows), dtype=np.dtype(JOIN_DTYPE))
    for k, r in enumerate(rows):
        j[k]["node"], j[k]["i"], j[k]["j"] = int(r[0]), int(r[1]), int(r[2])
        j[k]["len_i"], j[k]["len_j"] = float.fromhex(r[3]), float.fromhex(r[4])
    return j


@pytest.mark.parametrize("case", ["cfg0", "nj300", "nj1200", "dup200", "dup300", "tree500"])
def test_newick_text_matches_reference(case):
    names, _ = read_fasta(os.path.join(GOLD, case, "input.fasta"))
    text = newick(golden_joins(case), names)
    assert text == open(os.path.join(GOLD, case, "tree.nwk")).read()
