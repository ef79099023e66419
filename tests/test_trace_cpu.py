"""Host side of the traceback path: the cherry list (CPU only)."""
import os

import numpy as np

from mestrado_gb300 import cherries

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _joins(case):
    rows = [l.split() for l in open(os.path.join(GOLD, case, "joins.txt"))]
    left = np.array([int(r[1]) for r in rows], dtype=np.int32)
    right = np.array([int(r[2]) for r in rows], dtype=np.int32)
    return left, right


def test_cherries_small_tree():
    # ((0,1),(2,(3,4))): nodes 5=(3,4), 6=(0,1), 7=(2,5), 8=(6,7)
    left = np.array([3, 0, 2, 6], dtype=np.int32)
    right = np.array([4, 1, 5, 7], dtype=np.int32)
    node, l, r = cherries(left, right, 5)
    assert list(zip(node, l, r)) == [(6, 0, 1), (5, 3, 4)]


def test_reference_cherry_list_is_a_prefix():
    # buildAlign on one rank hands AlignmentMatch the first (n0-1)/3 getNodes
    # triples minus the last (SpeciesBlock.cpp:1393-1455); its vecSize==2
    # entries must be the first cherries of the full post-order list.
    for case in ("cfg0", "nj300", "nj1200", "dup200", "tree500"):
        left, right = _joins(case)
        n = len(left) + 1
        node, l, r = cherries(left, right, n)
        ref = [tuple(int(v) for v in line.split()) for line in open(os.path.join(GOLD, case, "cherries.txt"))]
        assert len(ref) <= len(node)
        assert ref == list(zip(node.tolist(), l.tolist(), r.tolist()))[: len(ref)]
        # every internal node whose children are leaves is listed once
        all_cherries = {(n + k) for k in range(n - 1) if left[k] < n and right[k] < n}
        assert set(node.tolist()) == all_cherries


def test_oracle_alignments_rescore_to_their_score():
    # every traceback reproduces its own DP score under the recurrence's model
    import numpy as np
    import oracle_py as O
    from rescore import rescore
    rng = np.random.default_rng(4)
    letters = np.frombuffer(b"ARNDCQEGHILKMFPSTWYV", dtype=np.uint8)
    sub = O.blosum()
    for _ in range(60):
        x = letters[rng.integers(0, 20, rng.integers(1, 150))].tobytes()
        y = letters[rng.integers(0, 20, rng.integers(1, 150))].tobytes()
        ax, ay, sc = O.traceback(x, y)
        assert ax.replace(b"-", b"") == x and ay.replace(b"-", b"") == y
        assert rescore(ax, ay, sub) == sc


def test_oracle_alignments_rescore_under_other_gap_models():
    # the same property for gap models with go >= ge (with go < ge a run of
    # gaps is cheaper reopened than extended, which this run-cost model does
    # not express; the reference only runs 10/2)
    import numpy as np
    import oracle_py as O
    from rescore import rescore
    letters = np.frombuffer(b"ARNDCQEGHILKMFPSTWYV", dtype=np.uint8)
    sub = O.blosum()
    for go, ge in ((5, 1), (11, 1), (20, 5), (6, 6)):
        rng = np.random.default_rng(go * 7 + ge)
        for _ in range(25):
            x = letters[rng.integers(0, 20, rng.integers(1, 120))].tobytes()
            y = letters[rng.integers(0, 20, rng.integers(1, 120))].tobytes()
            ax, ay, sc = O.traceback(x, y, go, ge)
            assert ax.replace(b"-", b"") == x and ay.replace(b"-", b"") == y
            assert sc == O.score_pair(x, y, go, ge)
            assert rescore(ax, ay, sub, go, ge) == sc
