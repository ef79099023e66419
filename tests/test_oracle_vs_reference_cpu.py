"""The oracle's neighbor joining against the reference's own buildTree
(SpeciesBlock.cpp and TreeNode.cpp compiled unchanged through the one-rank
shim into oracle/_ref/ref_nj) on fresh seeded matrices: sequence families,
duplicated sequences, tree metrics, small-integer and real-valued matrices.
The matrix is handed to the reference as its distance matrix (NWG_REF_D), so
any matrix can be compared.  Where the oracle counts no ambiguous step the
join lists and branch lengths are identical bit for bit.  CPU only; skipped
where the reference checkout is absent."""
import os
import subprocess

import numpy as np
import pytest

import oracle_py as O
from additive import random_tree_metric
from mestrado_gb300 import synth

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
from refsrc import REF

pytestmark = pytest.mark.skipif(not os.path.isfile(os.path.join(REF, "SpeciesBlock.cpp")),
                                reason="reference sources not present")


@pytest.fixture(scope="module")
def ref_nj():
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref", f"REF={REF}"], check=True)
    return os.path.join(ROOT, "oracle", "_ref", "ref_nj")


def _symmetric(M):
    M = np.triu(M.astype(np.float32), 1)
    return M + M.T


def _matrix(kind, seed):
    rng = np.random.default_rng(seed)
    if kind == "family":
        return O.score_all(synth.family(90, 150, ps=0.1, pi=0.01, seed=seed), threads=os.cpu_count() or 2)
    if kind == "families":
        S = synth.family(80, 60, ps=0.08, pi=0.005, families=3, seed=seed)
        return O.score_all(S, threads=os.cpu_count() or 2)
    if kind == "duplicates":
        S = synth.family(120, 50, ps=0.05, pi=0.005, seed=seed)
        return O.score_all(S.subset([k for k in range(120) for _ in range(2)]), threads=os.cpu_count() or 2)
    if kind == "tree":
        return random_tree_metric(350, seed)[0]
    if kind == "integers":
        return _symmetric(rng.integers(0, 50, size=(200, 200)))
    if kind == "gaussian":
        return _symmetric(rng.normal(0, 100, size=(300, 300)))
    raise ValueError(kind)


def _reference_joins(ref, D, tmp_path):
    # the FASTA only names the taxa: the matrix comes from the file
    fasta = tmp_path / "in.fasta"
    fasta.write_text("".join(f">t{k}\nA\n" for k in range(len(D))))
    dpath = tmp_path / "D.f32"
    np.ascontiguousarray(D, dtype=np.float32).tofile(dpath)
    env = dict(os.environ, NWG_REF_D=str(dpath))
    subprocess.run([ref, str(fasta), str(tmp_path / "out")], check=True, cwd=tmp_path, env=env,
                   stdout=subprocess.DEVNULL, timeout=120)
    rows = [line.split() for line in open(tmp_path / "out.joins")]
    joins = [(int(k), int(l), int(r), float.fromhex(a), float.fromhex(b)) for k, l, r, a, b in rows]
    tree = (tmp_path / "in.tree").read_text()
    cherries = [tuple(int(v) for v in line.split()) for line in open(tmp_path / "out.cherries")]
    return joins, tree, cherries


@pytest.mark.parametrize("kind,seed", [("family", 101), ("families", 102), ("duplicates", 103), ("tree", 41),
                                       ("tree", 42), ("integers", 104), ("gaussian", 105), ("gaussian", 106)])
def test_oracle_nj_equals_reference_on_fresh_matrices(ref_nj, tmp_path, kind, seed):
    D = _matrix(kind, seed)
    joins, st = O.nj(D)
    assert st["ambiguous_steps"] == 0
    ref, tree, ref_cherries = _reference_joins(ref_nj, D, tmp_path)
    assert len(ref) == len(joins) == len(D) - 1
    for r, j in zip(ref, joins):
        assert r == (j["node"], j["i"], j["j"], j["len_i"], j["len_j"])
    # the .tree text (labels are the header lines, '>' included) and the
    # cherries buildAlign hands on, a prefix of the full post-order list
    from mestrado_gb300 import cherries, newick
    from mestrado_gb300._native import JOIN_DTYPE
    n = len(D)
    lib_joins = np.zeros(len(joins), dtype=np.dtype(JOIN_DTYPE))
    for f in joins.dtype.names:
        lib_joins[f] = joins[f]
    assert newick(lib_joins, [f">t{k}" for k in range(n)]) == tree
    node, left, right = cherries(joins["i"], joins["j"], n)
    assert ref_cherries == list(zip(node.tolist(), left.tolist(), right.tolist()))[: len(ref_cherries)]


def _reference_conversion_table():
    # AlignmentScore::conversion (AlignmentScore.cu:10-27), read from the source
    # text.  Its initializer lists 255 values: entry 255 is zero-filled.
    import re
    src = open(os.path.join(REF, "AlignmentScore.cu")).read()
    body = src[src.index("AlignmentScore::conversion[256]"):]
    body = body[body.index("{") + 1:body.index("}")]
    table = [int(v) for v in re.findall(r"-?\d+", body)]
    assert len(table) == 255
    return table + [0]


def test_encoding_equals_reference_table_for_every_byte():
    from mestrado_gb300 import _native, encode
    table = _reference_conversion_table()
    for b in range(1, 255):   # byte 0 ends a C string: not a residue
        if table[b] < 0:
            with pytest.raises(_native.NWGError) as e:
                encode([bytes([b])])
            assert e.value.status == _native.NWG_ERR_BAD_RESIDUE
        else:
            codes, _ = encode([bytes([b, b, 65])])
            assert list(codes) == [0, table[b], table[b]]   # reversed: 'A' (code 0) first
    # byte 0xFF: the reference's zero-filled entry reads it as 'A'; it is no
    # residue letter, and this library reports it like every byte outside the
    # alphabet
    assert table[255] == 0
    with pytest.raises(_native.NWGError) as e:
        encode([bytes([255])])
    assert e.value.status == _native.NWG_ERR_BAD_RESIDUE


def test_substitution_matrix_equals_reference():
    # blosum64.txt and substitutionMatrix (definitions.cuh:96-121) of the
    # reference, read from their text; the oracle's built-in matrix
    import re
    txt = [int(v) for v in re.findall(r"-?\d+", open(os.path.join(REF, "blosum64.txt")).read())]
    src = open(os.path.join(REF, "definitions.cuh")).read()
    body = src[src.index("substitutionMatrix[SUBSTITUTION_MATRIX_SIZE]"):]
    body = body[body.index("{") + 1:body.index("}")]
    cuh = [int(v) for v in re.findall(r"-?\d+", body)]
    assert len(txt) == len(cuh) == 576 and txt == cuh
    assert np.asarray(O.blosum(), dtype=np.int64).reshape(576).tolist() == cuh


def test_reference_wire_blocks_and_matrix_layout(ref_nj, tmp_path):
    # Without a precomputed matrix the harness lets SpeciesBlock build its own
    # wire blocks (SpeciesBlock.cpp:309-322) and fill m_distances through the
    # AlignmentScore calls of :356-363, with the oracle decoding each block and
    # scoring each pair.  Its matrix equals score_all on the FASTA: the block
    # format and the row/column layout are the reference's.
    from fasta import read_fasta
    S = synth.family(23, 40, ps=0.15, pi=0.03, families=2, seed=107)   # ragged lengths
    fasta = tmp_path / "in.fasta"
    S.to_fasta(str(fasta))
    subprocess.run([ref_nj, str(fasta), str(tmp_path / "out")], check=True, cwd=tmp_path,
                   stdout=subprocess.DEVNULL, timeout=120, env={k: v for k, v in os.environ.items()
                                                               if k != "NWG_REF_D"})
    n = len(S)
    Dref = np.fromfile(tmp_path / "out.D", dtype=np.float32).reshape(n, n)
    _, seqs = read_fasta(str(fasta))
    assert np.array_equal(Dref, O.score_all(seqs))
    assert len(set(len(s) for s in seqs)) > 10
