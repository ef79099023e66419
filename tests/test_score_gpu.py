"""Parity of the sm_103a scoring kernels with the oracle (bit-exact: integer
scores stored as float32).  Every call goes through the C ABI."""
import os

import numpy as np
import pytest

import oracle_py as O
from mestrado_gb300 import (MODE_BATCHED, MODE_BATCHED_INT32, MODE_PLAIN, AlignmentScore, NWGError,
                            encode, make_wire, synth)
from mestrado_gb300 import _native

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
MODES = [MODE_BATCHED, MODE_PLAIN, MODE_BATCHED_INT32]


def _rand_set(seed, n, lo, hi, alphabet=b"ARNDCQEGHILKMFPSTWYV"):
    rng = np.random.default_rng(seed)
    letters = np.frombuffer(alphabet, dtype=np.uint8)
    lens = rng.integers(lo, hi + 1, size=n)
    return [letters[rng.integers(0, len(letters), L)].tobytes() for L in lens]


@pytest.mark.parametrize("mode", MODES)
def test_cfg0_matrix_equals_golden(ctx, mode):
    D0 = np.load(os.path.join(GOLD, "cfg0", "D.npy"))
    S = synth.config(0)
    D, st = ctx.score_all(S, mode=mode, stats=True)
    assert np.array_equal(D, D0)
    assert st["pairs"] == 64 * 65 // 2
    assert st["cells"] == S.cells()


@pytest.mark.parametrize("mode", MODES)
@pytest.mark.parametrize("seed,n,lo,hi", [(1, 40, 1, 60), (2, 33, 100, 420), (3, 21, 300, 900),
                                          (4, 12, 700, 2100)])
def test_random_lengths_match_oracle(ctx, mode, seed, n, lo, hi):
    seqs = _rand_set(seed, n, lo, hi)
    D = ctx.score_all(seqs, mode=mode)
    assert np.array_equal(D, O.score_all(seqs, threads=os.cpu_count()))


def test_full_alphabet_and_identical_and_single_residue(ctx):
    seqs = _rand_set(7, 10, 1, 50, alphabet=b"ARNDCQEGHILKMFPSTWYVBZX*")
    seqs += [b"A", b"W", seqs[3], seqs[3], b"*"]
    Dref = O.score_all(seqs)
    for mode in MODES:
        assert np.array_equal(ctx.score_all(seqs, mode=mode), Dref)


def test_one_and_two_sequences(ctx):
    for seqs in ([b"MKV"], [b"MKV", b"MKVL"]):
        assert np.array_equal(ctx.score_all(seqs), O.score_all(seqs))


def test_overflow_guard_routes_to_int32(ctx):
    # W scores 11 against itself: a 3200-residue W run bounds H at 35200 > int16
    seqs = [b"W" * 3200, b"W" * 3100 + b"A" * 50, b"MKV" * 300, b"W" * 3000, b"ACDEFGHIKL" * 310,
            b"MKVL" * 770]
    D, st = ctx.score_all(seqs, mode=MODE_BATCHED, stats=True)
    assert st["reruns"] > 0            # int16 attempt rejected by the bound, re-run on int32
    assert np.array_equal(D, O.score_all(seqs, threads=os.cpu_count()))
    assert D[0, 0] == 3200 * 11
    # lengths above the int16 length guard take int32 lanes for the whole set
    long = [b"MKV" * 2400, b"W" * 10, b"ACDEFGHIKL" * 30]
    D, st = ctx.score_all(long, mode=MODE_BATCHED, stats=True)
    assert st["pairs_int32"] == 6 and st["pairs_int16"] == 0
    assert np.array_equal(D, O.score_all(long, threads=os.cpu_count()))


def test_long_sequences_every_mode(ctx):
    # far above the lengths of any workload: many bands per pair, int32 lanes
    seqs = _rand_set(11, 4, 1, 3, alphabet=b"ARNDCQEGHILKMFPSTWYV")
    seqs += _rand_set(12, 1, 16384, 16384) + _rand_set(13, 1, 9001, 9001) + _rand_set(14, 1, 4001, 4001)
    Dref = O.score_all(seqs, threads=os.cpu_count())
    for mode in MODES:
        assert np.array_equal(ctx.score_all(seqs, mode=mode), Dref), mode


def test_thousands_of_tiny_sequences_every_mode(ctx):
    # 4.5 million pairs of 1-4 residues: the bucketing and the pair bookkeeping, not the DP
    seqs = _rand_set(15, 3000, 1, 4, alphabet=b"ARNDCQEGHILKMFPSTWYVBZX*")
    Dref = O.score_all(seqs, threads=os.cpu_count())
    for mode in MODES:
        assert np.array_equal(ctx.score_all(seqs, mode=mode), Dref), mode


def test_cached_plan_and_graph_replay_with_new_residues(ctx):
    # same lengths, different residues: the cached plan and graph are reused
    a = _rand_set(31, 50, 20, 700)
    lens_a = [len(x) for x in a]
    rng = np.random.default_rng(3)
    letters = np.frombuffer(b"ARNDCQEGHILKMFPSTWYV", dtype=np.uint8)
    b = [letters[rng.integers(0, 20, L)].tobytes() for L in lens_a]
    for seqs in (a, b, a):
        for _ in range(2):
            assert np.array_equal(ctx.score_all(seqs), O.score_all(seqs, threads=os.cpu_count()))


def test_block_shape_with_column_offset(ctx):
    X = _rand_set(9, 17, 20, 400)
    Y = _rand_set(10, 13, 5, 300)
    for mode in MODES:
        D = np.full((17, 40), -1.0, dtype=np.float32)
        ctx.score_block(X, Y, D=D, r0=20, mode=mode)
        ref = np.array([[O.score_pair(x, y) for y in Y] for x in X], dtype=np.float32)
        assert np.array_equal(D[:, 20:33], ref)
        assert (D[:, :20] == -1).all() and (D[:, 33:] == -1).all()


def test_pair_list(ctx):
    seqs = _rand_set(11, 30, 1, 500)
    codes, off = encode(seqs)
    rng = np.random.default_rng(0)
    pi, pj = rng.integers(0, 30, 200), rng.integers(0, 30, 200)
    out = ctx.score_pairs(codes, off, pi, pj)
    ref = O.score_list(codes, off, pi, pj)
    assert np.array_equal(out, ref)


def test_reference_class_mirror(ctx):
    S = synth.family(40, 200, seed=21)
    wire = make_wire(S)
    al = AlignmentScore(10, 2, 16, int(S.lengths.max()))
    al.loadDB(wire, len(S))
    D = [[0.0] * len(S) for _ in range(len(S))]
    al.computeDistanceMtx(wire, len(S), D, 0)
    assert np.array_equal(np.array(D, dtype=np.float32), O.score_all(S))
    # a second block at a column offset (two-rank ring step shape)
    half = S.subset(range(20))
    other = S.subset(range(20, 40))
    al2 = AlignmentScore(10, 2, 16, 400)
    al2.loadDB(make_wire(half), 20)
    D2 = np.zeros((20, 40), dtype=np.float32)
    al2.computeDistanceMtx(make_wire(other, rank=1), 20, D2, 20)
    assert np.array_equal(D2[:, 20:], O.score_all(S)[:20, 20:])


def test_errors_are_status_codes(ctx):
    with pytest.raises(NWGError) as e:
        ctx.score_all(codes=np.array([0, 1, 30], dtype=np.int8), offsets=np.array([0, 3], dtype=np.int64))
    assert e.value.status == _native.NWG_ERR_BAD_RESIDUE
    with pytest.raises(NWGError) as e:
        ctx.score_all(codes=np.array([0, 1], dtype=np.int8), offsets=np.array([0, 2, 2], dtype=np.int64))
    assert e.value.status == _native.NWG_ERR_EMPTY_SEQ


def test_config1_full_size_properties_and_sample(ctx):
    S = synth.config(1)
    n = len(S)
    codes, off = encode(S)
    Db, st = ctx.score_all(codes=codes, offsets=off, mode=MODE_BATCHED, stats=True)
    assert st["pairs"] == n * (n + 1) // 2
    assert np.array_equal(Db, Db.T)
    Dp = ctx.score_all(codes=codes, offsets=off, mode=MODE_PLAIN)
    assert np.array_equal(Db, Dp)
    rng = np.random.default_rng(1)
    pi, pj = rng.integers(0, n, 3000), rng.integers(0, n, 3000)
    ref = O.score_list(codes, off, pi, pj, threads=os.cpu_count())
    assert np.array_equal(Db[pi, pj], ref.astype(np.float32))
    diag = O.score_list(codes, off, np.arange(0, n, 37), np.arange(0, n, 37), threads=os.cpu_count())
    assert np.array_equal(np.diag(Db)[::37], diag.astype(np.float32))


@pytest.mark.parametrize("R", [4, 8, 12, 16, 20, 24, 32])
@pytest.mark.parametrize("V,W", [(0, 32), (1, 32), (2, 32), (3, 32), (4, 32), (5, 32), (0, 16), (2, 16), (3, 16),
                                 (4, 16), (5, 16), (0, 8), (2, 8), (3, 8), (4, 8), (5, 8),
                                 (0, 1), (2, 1), (3, 1), (4, 1)])
def test_every_kernel_template_matches_oracle(R, V, W):
    # the autotuner may pick any (rows per lane, register layout, front width)
    # for any length class: every template must be exact, single- and
    # multi-band, with fronts of one warp finishing at different columns.
    # W = 1 is one pair per thread (each lane its own front, bands of R rows,
    # up to 225 bands here)
    _check_template(R, V, W)


@pytest.mark.parametrize("R", [18, 22, 26, 28, 30])
@pytest.mark.parametrize("V,W", [(2, 32), (3, 32), (4, 32), (2, 16), (3, 16), (4, 16), (2, 8), (3, 8), (4, 8)])
def test_finer_band_templates_match_oracle(R, V, W):
    # rows per lane that are not multiples of 4 (the lane's last 4-row profile
    # load is partly used) and 28: int16x2 wavefronts with layouts 2 to 4
    _check_template(R, V, W)


@pytest.mark.parametrize("R", [8, 16, 24, 32])
@pytest.mark.parametrize("W", [32, 16, 8])
def test_split_strip_templates_match_oracle(R, W):
    # layout 6: layout 3 with each lane's strip in two halves one column apart
    # (two columns of skew between lanes), single- and multi-band
    _check_template(R, 6, W)


@pytest.mark.parametrize("go,ge", [(3, 5), (15, 1), (0, 0), (40, 30)])
def test_split_strips_under_gap_models(go, ge):
    from mestrado_gb300 import Context
    seqs = _gap_case_sets()["short"]
    ref = O.score_all(seqs, go, ge, threads=os.cpu_count())
    with Context(go, ge) as c:
        c.set_tuning(16, 6, 16)
        assert np.array_equal(c.score_all(seqs), ref)


def _check_template(R, V, W):
    from mestrado_gb300 import Context
    seqs = _rand_set(40 + R, 26, 1, 900)
    ref = O.score_all(seqs, threads=os.cpu_count())
    with Context(10, 2) as c:
        c.set_tuning(R, V, W)
        for mode in (MODE_BATCHED, MODE_BATCHED_INT32):
            assert np.array_equal(c.score_all(seqs, mode=mode), ref)
        # a block (no triangle), X and Y from different sets
        xs = _rand_set(90 + R, 13, 1, 700)
        Db = c.score_block(xs, seqs)
        assert np.array_equal(Db, O.score_all(xs + seqs, threads=os.cpu_count())[:13, 13:])


def _gap_case_sets():
    rng = np.random.default_rng(8)
    letters = b"ARNDCQEGHILKMFPSTWYV"
    def rnd(L):
        return bytes(rng.choice(list(letters), L).tolist())
    return {
        # long sequences with a large extension penalty: int16 lanes would
        # overflow at the boundary row alone (-ge*(c+1)), so they must not be used
        "long_ge20": [rnd(L) for L in (2100, 1900, 1500, 700, 640, 580, 90)],
        "short": [rnd(L) for L in rng.integers(1, 500, 30)],
        # identical high-scoring runs: the H upper bound decides int16 vs int32
        "runs": [b"W" * 1200, b"W" * 1100, b"C" * 1300, rnd(1250), rnd(400), b"W" * 900],
    }


@pytest.mark.parametrize("go,ge,mat,case", [
    (3, 5, "blosum", "short"), (15, 1, "blosum", "short"), (0, 0, "blosum", "short"),
    (10, 20, "blosum", "long_ge20"), (10, 2, "x3", "runs"), (10, 2, "x3", "short"),
    (40, 30, "blosum", "short")])
@pytest.mark.parametrize("V", [0, 1, 2, 3, 4, 5])
def test_gap_penalties_and_matrices_match_oracle(go, ge, mat, case, V):
    # the int16 guard follows the context's penalties and matrix
    from mestrado_gb300 import Context
    sub = O.blosum().astype(np.int32)
    if mat == "x3":
        sub = np.clip(sub * 3, -128, 127)
    sub = sub.astype(np.int8)
    seqs = _gap_case_sets()[case]
    ref = O.score_all(seqs, go, ge, threads=os.cpu_count(), sub=sub)
    with Context(go, ge, sub=sub) as c:
        # one band of 32 lanes per class where it fits: rows per lane = the
        # class's rows / 32 rounded up to a multiple of 4, at most 32
        rows = [min(32, -(-(-(-r // 32)) // 4) * 4) for r in _native.TUNE_CLASS_ROWS]
        c.set_tuning(rows, V)
        for mode in (MODE_BATCHED, MODE_PLAIN):
            assert np.array_equal(c.score_all(seqs, mode=mode), ref)


def test_autotune_then_exact(tmp_path, monkeypatch):
    monkeypatch.setenv("NWG_TUNE_CACHE", str(tmp_path))
    from mestrado_gb300 import Context
    with Context(10, 2) as c:
        r = c.autotune(force=True)
        assert not r["from_cache"] and len(r["classes"]) == _native.TUNE_CLASSES
        assert all(k["gcups"] > 0 for k in r["classes"])
        seqs = _rand_set(77, 40, 10, 1200)
        assert np.array_equal(c.score_all(seqs), O.score_all(seqs, threads=os.cpu_count()))
    with Context(10, 2) as c:
        r2 = c.autotune()
        assert r2["from_cache"]
        assert [(k["rows_per_lane"], k["variant"], k["lanes"]) for k in r2["classes"]] == \
            [(k["rows_per_lane"], k["variant"], k["lanes"]) for k in r["classes"]]
