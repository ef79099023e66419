"""Edge cases of the host-only entry points (no device work): the Newick text
of TreeNode::buildTreeOutput (TreeNode.cpp:61-81, SpeciesBlock.cpp:1328-1338)
and the cherry list of AlignmentMatch.cu:167-186."""
import ctypes

import numpy as np
import pytest

from mestrado_gb300 import _native, cherries, newick
from mestrado_gb300._native import JOIN_DTYPE


def _joins(rows):
    j = np.zeros(len(rows), dtype=np.dtype(JOIN_DTYPE))
    for k, (node, i, jj, li, lj) in enumerate(rows):
        j[k]["node"], j[k]["i"], j[k]["j"], j[k]["len_i"], j[k]["len_j"] = node, i, jj, li, lj
    return j


def _len(v):
    # ":" << setprecision(4) << showpoint << setw(8) << v is printf's "%#.4g"
    # right-aligned in 8 columns (the iostream conversions are defined by printf's)
    return ":" + ("%#.4g" % v).rjust(8)


def _raw_newick(joins, names, cap):
    arr = (ctypes.c_char_p * len(names))(*[x.encode() for x in names])
    buf = ctypes.create_string_buffer(max(cap, 1)) if cap else None
    jp = joins.ctypes.data_as(ctypes.c_void_p) if joins is not None else None
    got = _native.lib().nwg_newick(jp, len(names), arr, buf, cap)
    return got, (buf.raw if buf is not None else None)


def test_newick_two_and_three_leaves():
    j = _joins([(2, 0, 1, 0.5, 1.25)])
    assert newick(j, ["a", "b"]) == "(\na" + _len(0.5) + ",\nb" + _len(1.25) + ")\n;\n"
    # ((x,y),z) with a negative and a large branch length
    j = _joins([(3, 0, 1, -0.125, 3.0), (4, 3, 2, 12345.678, 1e-5)])
    want = "(\n(\nx" + _len(-0.125) + ",\ny" + _len(3.0) + ")\n" + _len(12345.678) + ",\nz" + _len(1e-5) + ")\n;\n"
    assert newick(j, ["x", "y", "z"]) == want
    assert _len(1.25) == ":   1.250" and _len(-0.125) == ": -0.1250"


def test_newick_single_leaf_has_no_length():
    got, _ = _raw_newick(None, ["only"], 0)
    assert got == len("only;\n")
    assert newick(np.zeros(0, dtype=np.dtype(JOIN_DTYPE)), ["only"]) == "only;\n"


def test_newick_truncates_and_returns_the_full_length():
    j = _joins([(2, 0, 1, 0.5, 1.25)])
    full = newick(j, ["a", "b"])
    for cap in (1, 2, 5, len(full), len(full) + 1):
        got, raw = _raw_newick(j, ["a", "b"], cap)
        assert got == len(full)
        m = min(len(full), cap - 1)
        assert raw[:m] == full[:m].encode() and raw[m] == 0


def test_newick_rejects_malformed_joins():
    bad = [
        [(3, 0, 1, 0.1, 0.1)],            # node id is not n + k
        [(2, 0, 2, 0.1, 0.1)],            # child id not below the new node
        [(2, -1, 1, 0.1, 0.1)],           # negative child
    ]
    for rows in bad:
        with pytest.raises(_native.NWGError) as e:
            newick(_joins(rows), ["a", "b"])
        assert e.value.status == _native.NWG_ERR_INVALID
    got, _ = _raw_newick(None, [], 0)
    assert got == -_native.NWG_ERR_INVALID


def test_cherries_degenerate_and_shaped_trees():
    e = np.zeros(0, dtype=np.int32)
    for n in (0, 1):
        node, l, r = cherries(e, e, n)
        assert len(node) == 0
    node, l, r = cherries(np.array([0]), np.array([1]), 2)
    assert list(zip(node, l, r)) == [(2, 0, 1)]
    # caterpillar (((((0,1),2),3),4),5): one cherry
    left = np.array([0, 6, 7, 8, 9], dtype=np.int32)
    right = np.array([1, 2, 3, 4, 5], dtype=np.int32)
    assert list(zip(*cherries(left, right, 6))) == [(6, 0, 1)]
    # balanced ((0,1),(2,3)),((4,5),(6,7)): four cherries in getNodes post-order
    left = np.array([0, 2, 4, 6, 8, 10, 12], dtype=np.int32)
    right = np.array([1, 3, 5, 7, 9, 11, 13], dtype=np.int32)
    assert list(zip(*cherries(left, right, 8))) == [(8, 0, 1), (9, 2, 3), (10, 4, 5), (11, 6, 7)]
    # children swapped: the post-order follows left before right
    assert list(zip(*cherries(right, left, 8))) == [(11, 7, 6), (10, 5, 4), (9, 3, 2), (8, 1, 0)]


def test_cherries_reject_ids_out_of_range():
    for left, right in (([0, 5], [1, 2]), ([0, -1], [1, 2]), ([0, 1], [1, 4])):
        with pytest.raises(_native.NWGError) as e:
            cherries(np.array(left), np.array(right), 3)
        assert e.value.status == _native.NWG_ERR_INVALID
