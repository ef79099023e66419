"""ctypes view of the CPU oracle (oracle/liboracle.so) -- test infrastructure.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import
this module; the product package never does.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE_DIR = os.path.join(ROOT, "oracle")
_LIB = None


class Join(ctypes.Structure):
    _fields_ = [
        ("i", ctypes.c_int32), ("j", ctypes.c_int32), ("node", ctypes.c_int32), ("n", ctypes.c_int32),
        ("d", ctypes.c_float), ("pad", ctypes.c_float), ("q", ctypes.c_double),
        ("ti", ctypes.c_double), ("tj", ctypes.c_double),
        ("len_i", ctypes.c_double), ("len_j", ctypes.c_double),
    ]


class NJStats(ctypes.Structure):
    _fields_ = [("ambiguous_steps", ctypes.c_int64), ("tie_steps", ctypes.c_int64),
                ("rebuilds", ctypes.c_int64), ("pq_trigger_open", ctypes.c_int64)]


def build() -> str:
    subprocess.run(["make", "-s", "-C", ORACLE_DIR, "liboracle.so"], check=True)
    return os.path.join(ORACLE_DIR, "liboracle.so")


def lib():
    global _LIB
    if _LIB is None:
        path = os.path.join(ORACLE_DIR, "liboracle.so")
        if not os.path.exists(path):
            build()
        L = ctypes.CDLL(path)
        P = ctypes.POINTER
        L.nwo_blosum.restype = P(ctypes.c_int8)
        L.nwo_encode_reverse.argtypes = [ctypes.c_char_p, ctypes.c_int, P(ctypes.c_int8)]
        L.nwo_encode_reverse.restype = ctypes.c_int
        L.nwo_parse_wire.argtypes = [ctypes.c_char_p, ctypes.c_int, P(ctypes.c_int8), P(ctypes.c_int64)]
        L.nwo_parse_wire.restype = ctypes.c_int
        L.nwo_score_pair.argtypes = [P(ctypes.c_int8), ctypes.c_int, P(ctypes.c_int8), ctypes.c_int,
                                     ctypes.c_int, ctypes.c_int, P(ctypes.c_int8)]
        L.nwo_score_pair.restype = ctypes.c_int
        L.nwo_score_all.argtypes = [P(ctypes.c_int8), P(ctypes.c_int64), ctypes.c_int, ctypes.c_int,
                                    ctypes.c_int, P(ctypes.c_int8), P(ctypes.c_float), ctypes.c_int64,
                                    ctypes.c_int]
        L.nwo_score_list.argtypes = [P(ctypes.c_int8), P(ctypes.c_int64), P(ctypes.c_int32),
                                     P(ctypes.c_int32), ctypes.c_int64, ctypes.c_int, ctypes.c_int,
                                     P(ctypes.c_int8), P(ctypes.c_int32), ctypes.c_int]
        L.nwo_traceback.argtypes = [P(ctypes.c_int8), ctypes.c_int, P(ctypes.c_int8), ctypes.c_int,
                                    ctypes.c_int, ctypes.c_int, P(ctypes.c_int8), ctypes.c_char_p,
                                    ctypes.c_char_p, P(ctypes.c_int)]
        L.nwo_traceback.restype = ctypes.c_int
        L.nwo_nj.argtypes = [P(ctypes.c_float), ctypes.c_int, P(Join), P(NJStats)]
        L.nwo_msa.argtypes = [P(ctypes.c_int8), P(ctypes.c_int64), ctypes.c_int, P(ctypes.c_int32), P(ctypes.c_int32),
                              ctypes.c_int, ctypes.c_int, P(ctypes.c_int8), ctypes.c_char_p, ctypes.c_int64]
        L.nwo_msa.restype = ctypes.c_int64
        _LIB = L
    return _LIB


def _p(a, ct):
    return a.ctypes.data_as(ctypes.POINTER(ct))


def blosum() -> np.ndarray:
    return np.ctypeslib.as_array(lib().nwo_blosum(), shape=(576,)).copy()


def encode(seqset):
    """Reversed 8-bit codes and offsets for a synth.SeqSet (or list of bytes)."""
    if isinstance(seqset, (list, tuple)):
        seqs = list(seqset)
    else:
        seqs = [seqset[i] for i in range(len(seqset))]
    lens = np.array([len(s) for s in seqs], dtype=np.int64)
    off = np.zeros(len(seqs) + 1, dtype=np.int64)
    np.cumsum(lens, out=off[1:])
    codes = np.zeros(max(int(off[-1]), 1), dtype=np.int8)
    bad = 0
    for k, s in enumerate(seqs):
        buf = (ctypes.c_int8 * max(len(s), 1)).from_buffer(codes, int(off[k]))
        bad += lib().nwo_encode_reverse(s, len(s), buf)
    if bad:
        raise ValueError(f"{bad} residues outside the 24-letter alphabet")
    return codes, off


def score_pair(x: bytes, y: bytes, go: int = 10, ge: int = 2) -> int:
    (cx, ox) = encode([x])
    (cy, oy) = encode([y])
    sub = blosum()
    return lib().nwo_score_pair(_p(cx, ctypes.c_int8), len(x), _p(cy, ctypes.c_int8), len(y), go, ge,
                                _p(sub, ctypes.c_int8))


def score_all(seqset, go: int = 10, ge: int = 2, threads: int = 0, sub=None) -> np.ndarray:
    codes, off = encode(seqset)
    n = len(off) - 1
    D = np.zeros((n, n), dtype=np.float32)
    sub = blosum() if sub is None else np.ascontiguousarray(sub, dtype=np.int8).reshape(576)
    lib().nwo_score_all(_p(codes, ctypes.c_int8), _p(off, ctypes.c_int64), n, go, ge,
                        _p(sub, ctypes.c_int8), _p(D, ctypes.c_float), n, threads)
    return D


def score_list(codes, off, pi, pj, go: int = 10, ge: int = 2, threads: int = 0, sub=None) -> np.ndarray:
    pi = np.ascontiguousarray(pi, dtype=np.int32)
    pj = np.ascontiguousarray(pj, dtype=np.int32)
    out = np.zeros(len(pi), dtype=np.int32)
    sub = blosum() if sub is None else np.ascontiguousarray(sub, dtype=np.int8).reshape(576)
    lib().nwo_score_list(_p(codes, ctypes.c_int8), _p(off, ctypes.c_int64), _p(pi, ctypes.c_int32),
                         _p(pj, ctypes.c_int32), len(pi), go, ge, _p(sub, ctypes.c_int8),
                         _p(out, ctypes.c_int32), threads)
    return out


def traceback(x: bytes, y: bytes, go: int = 10, ge: int = 2):
    """(aligned_x, aligned_y, score) for X = columns, Y = rows."""
    (cx, _), (cy, _) = encode([x]), encode([y])
    sub = blosum()
    bx = ctypes.create_string_buffer(len(x) + len(y) + 1)
    by = ctypes.create_string_buffer(len(x) + len(y) + 1)
    sc = ctypes.c_int(0)
    lib().nwo_traceback(_p(cx, ctypes.c_int8), len(x), _p(cy, ctypes.c_int8), len(y), go, ge,
                        _p(sub, ctypes.c_int8), bx, by, ctypes.byref(sc))
    return bx.value, by.value, sc.value


def msa(seqset, left, right, go: int = 10, ge: int = 2, sub=None):
    """Progressive alignment along the guide tree (internal node n+k joins
    left[k], right[k]): list of n gapped rows, forward order."""
    codes, off = encode(seqset)
    n = len(off) - 1
    left = np.ascontiguousarray(left, dtype=np.int32)
    right = np.ascontiguousarray(right, dtype=np.int32)
    sub = blosum() if sub is None else np.ascontiguousarray(sub, dtype=np.int8).reshape(576)
    L = lib().nwo_msa(_p(codes, ctypes.c_int8), _p(off, ctypes.c_int64), n, _p(left, ctypes.c_int32),
                      _p(right, ctypes.c_int32), go, ge, _p(sub, ctypes.c_int8), None, 0)
    if L < 0:
        raise ValueError("malformed tree")
    buf = ctypes.create_string_buffer(int(n * L) + 1)
    lib().nwo_msa(_p(codes, ctypes.c_int8), _p(off, ctypes.c_int64), n, _p(left, ctypes.c_int32),
                  _p(right, ctypes.c_int32), go, ge, _p(sub, ctypes.c_int8), buf, n * L)
    raw = buf.raw
    return [raw[k * L:(k + 1) * L] for k in range(n)]


def nj(D: np.ndarray):
    """Exact-argmin restatement of buildTree; returns (joins structured array, stats)."""
    D = np.array(D, dtype=np.float32, copy=True, order="C")
    n = D.shape[0]
    joins = (Join * max(n - 1, 1))()
    st = NJStats()
    lib().nwo_nj(_p(D, ctypes.c_float), n, joins, ctypes.byref(st))
    rows = [(j.i, j.j, j.node, j.n, j.d, j.q, j.ti, j.tj, j.len_i, j.len_j) for j in joins][: max(n - 1, 0)]
    dt = np.dtype([("i", "i4"), ("j", "i4"), ("node", "i4"), ("n", "i4"), ("d", "f4"), ("q", "f8"),
                   ("ti", "f8"), ("tj", "f8"), ("len_i", "f8"), ("len_j", "f8")])
    return np.array(rows, dtype=dt), {k: getattr(st, k) for k, _ in NJStats._fields_}


class NJModelStats(ctypes.Structure):
    _fields_ = [("rebuilds", ctypes.c_int64), ("pq_triggers", ctypes.c_int64),
                ("out_of_range_bins", ctypes.c_int64)]


def nj_model(D: np.ndarray):
    """buildTree with its bins, bin heaps, candidate list and prediction array,
    on the reference's own standard containers (oracle/nj_model.cpp): the
    reference's joins, ties and roundings included.  Returns (joins
    structured array, stats)."""
    D = np.array(D, dtype=np.float32, copy=True, order="C")
    n = D.shape[0]
    joins = (Join * max(n - 1, 1))()
    st = NJModelStats()
    L = lib()
    L.nwo_nj_model.argtypes = [ctypes.POINTER(ctypes.c_float), ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
    L.nwo_nj_model(_p(D, ctypes.c_float), n, ctypes.cast(joins, ctypes.c_void_p),
                   ctypes.cast(ctypes.byref(st), ctypes.c_void_p))
    rows = [(j.i, j.j, j.node, j.n, j.d, j.q, j.ti, j.tj, j.len_i, j.len_j) for j in joins][: max(n - 1, 0)]
    dt = np.dtype([("i", "i4"), ("j", "i4"), ("node", "i4"), ("n", "i4"), ("d", "f4"), ("q", "f8"),
                   ("ti", "f8"), ("tj", "f8"), ("len_i", "f8"), ("len_j", "f8")])
    return np.array(rows, dtype=dt), {k: getattr(st, k) for k, _ in NJModelStats._fields_}
