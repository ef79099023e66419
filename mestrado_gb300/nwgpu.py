"""Python host side of libnwgpu: contexts and the reference's AlignmentScore.

Every compute call goes through the C ABI (include/nwgpu.h).  Arrays are
numpy on the host; the ``*_dev`` forms take raw device pointers (for example
``torch.Tensor.data_ptr()``) and optionally a CUDA stream handle.
"""
from __future__ import annotations

import ctypes
import struct

import numpy as np

from ._native import (MODE_BATCHED, MODE_BATCHED_INT32, MODE_PLAIN, NWGError, Stats, c_f32p,
                      c_i8p, c_i32p, c_i64p, check, lib)

__all__ = ["Context", "AlignmentScore", "Server", "cherries", "encode", "make_wire", "newick", "parse_wire"]


def _p(a: np.ndarray, ct):
    return a.ctypes.data_as(ct)


def _as_seq_list(seqs):
    if hasattr(seqs, "residues") and hasattr(seqs, "offsets"):
        return seqs.residues, np.asarray(seqs.offsets, dtype=np.int64)
    parts = [s.encode() if isinstance(s, str) else bytes(s) for s in seqs]
    off = np.zeros(len(parts) + 1, dtype=np.int64)
    np.cumsum([len(p) for p in parts], out=off[1:])
    return b"".join(parts), off


def encode(seqs):
    """Reversed 8-bit codes + offsets for ASCII sequences (AlignmentScore.cu:142-178)."""
    res, off = _as_seq_list(seqs)
    codes = np.zeros(max(int(off[-1]), 1), dtype=np.int8)
    st = lib().nwg_encode(res, _p(off, c_i64p), len(off) - 1, _p(codes, c_i8p))
    check(st)
    return codes, off


def make_wire(seqs, rank: int = 0) -> bytes:
    """The sequence block rank 0 sends in SpeciesBlock.cpp:309-322:
    [int rank][{int seqNo, int len, char[len], '\\0'} x n]."""
    res, off = _as_seq_list(seqs)
    out = [struct.pack("<i", rank)]
    for k in range(len(off) - 1):
        s = res[off[k]:off[k + 1]]
        out.append(struct.pack("<ii", k, len(s)) + s + b"\0")
    return b"".join(out)


def parse_wire(buf: bytes, n: int):
    """Decode a wire block into reversed codes + offsets (AlignmentScore::parse)."""
    off = np.zeros(n + 1, dtype=np.int64)
    check(lib().nwg_parse_wire(buf, n, None, _p(off, c_i64p)))
    codes = np.zeros(max(int(off[-1]), 1), dtype=np.int8)
    check(lib().nwg_parse_wire(buf, n, _p(codes, c_i8p), _p(off, c_i64p)))
    return codes, off


class Context:
    """One libnwgpu context: gap penalties, substitution matrix, CUDA stream."""

    def __init__(self, gap_open: int = 10, gap_ext: int = 2, sub=None):
        self._lib = lib()
        h = ctypes.c_void_p()
        subp = None
        if sub is not None:
            self._sub = np.ascontiguousarray(sub, dtype=np.int8).reshape(576)
            subp = _p(self._sub, c_i8p)
        check(self._lib.nwg_ctx_create(gap_open, gap_ext, subp, ctypes.byref(h)))
        self.h = h
        self.gap_open, self.gap_ext = gap_open, gap_ext

    def close(self):
        if getattr(self, "h", None):
            self._lib.nwg_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _check(self, st):
        check(st, self.h)

    def set_stream(self, stream_handle: int | None):
        self._check(self._lib.nwg_set_stream(self.h, ctypes.c_void_p(stream_handle or 0)))

    # ---- measurement -----------------------------------------------------
    def dpx_peak(self, lanes16: bool = True, form: int | None = None) -> float:
        """Cells/s of the bare cell update on every SM (roofline): the fastest
        form, or one form (nwg_dpx_peak_form)."""
        v = ctypes.c_double()
        if form is None:
            self._check(self._lib.nwg_dpx_peak(self.h, 1 if lanes16 else 0, ctypes.byref(v)))
        else:
            self._check(self._lib.nwg_dpx_peak_form(self.h, 1 if lanes16 else 0, int(form), ctypes.byref(v)))
        return v.value

    def autotune(self, force: bool = False) -> dict:
        """Pick the wave-kernel template per length class (cached per device)."""
        from ._native import TuneResult
        r = TuneResult()
        self._check(self._lib.nwg_autotune(self.h, 1 if force else 0, ctypes.byref(r)))
        return r.as_dict()

    def set_tuning(self, rows_per_lane, variant, lanes=None):
        """Kernel choice per length class (TUNE_CLASSES entries each; a scalar
        is used for every class): rows per lane, register layout, lanes per
        wavefront (default 32)."""
        from ._native import TUNE_CLASSES
        k = TUNE_CLASSES
        rp = np.ascontiguousarray(np.broadcast_to(rows_per_lane, (k,)), dtype=np.int32)
        vv = np.ascontiguousarray(np.broadcast_to(variant, (k,)), dtype=np.int32)
        ww = np.ascontiguousarray(np.broadcast_to(32 if lanes is None else lanes, (k,)), dtype=np.int32)
        self._check(self._lib.nwg_set_tuning_lanes(self.h, _p(rp, c_i32p), _p(vv, c_i32p), _p(ww, c_i32p)))

    def set_launch_timing(self, on: bool):
        self._check(self._lib.nwg_set_launch_timing(self.h, 1 if on else 0))

    def launch_records(self):
        from ._native import LaunchRec
        n = self._lib.nwg_launch_records(self.h, None, 0)
        if n < 0:
            raise NWGError(-n, "launch records")
        arr = (LaunchRec * max(n, 1))()
        self._lib.nwg_launch_records(self.h, arr, n)
        return [arr[k].as_dict() for k in range(n)]

    # ---- scoring ---------------------------------------------------------
    def score_all(self, seqs=None, *, codes=None, offsets=None, mode: int = MODE_BATCHED,
                  out: np.ndarray | None = None, stats: bool = False):
        """Full n x n distance matrix (float32) of ASCII ``seqs`` or of
        pre-encoded ``codes``/``offsets``.  Host buffers in and out."""
        if codes is None:
            codes, offsets = encode(seqs)
        codes = np.ascontiguousarray(codes, dtype=np.int8)
        offsets = np.ascontiguousarray(offsets, dtype=np.int64)
        n = len(offsets) - 1
        D = out if out is not None else np.empty((n, n), dtype=np.float32)
        st = Stats()
        self._check(self._lib.nwg_score_all(self.h, _p(codes, c_i8p), _p(offsets, c_i64p), n,
                                            _p(D, c_f32p), D.strides[0] // 4, mode, ctypes.byref(st)))
        return (D, st.as_dict()) if stats else D

    def score_all_dev(self, d_codes: int, offsets: np.ndarray, d_D: int, ld: int,
                      mode: int = MODE_BATCHED, stats: bool = False):
        """Device-resident form: ``d_codes``/``d_D`` are device pointers."""
        offsets = np.ascontiguousarray(offsets, dtype=np.int64)
        st = Stats()
        self._check(self._lib.nwg_score_all_dev(self.h, ctypes.c_void_p(d_codes), _p(offsets, c_i64p),
                                                len(offsets) - 1, ctypes.c_void_p(d_D), ld, mode,
                                                ctypes.byref(st) if stats else None))
        return st.as_dict() if stats else None

    def score_block(self, xseqs=None, yseqs=None, *, D=None, r0: int = 0, mode: int = MODE_BATCHED,
                    xcodes=None, xoffsets=None, ycodes=None, yoffsets=None, stats: bool = False):
        """D[x][r0 + y] = score(X_x, Y_y): the computeDistanceMtx block shape."""
        if xcodes is None:
            xcodes, xoffsets = encode(xseqs)
        if ycodes is None:
            ycodes, yoffsets = encode(yseqs)
        nx, ny = len(xoffsets) - 1, len(yoffsets) - 1
        if D is None:
            D = np.zeros((nx, r0 + ny), dtype=np.float32)
        xoffsets = np.ascontiguousarray(xoffsets, dtype=np.int64)
        yoffsets = np.ascontiguousarray(yoffsets, dtype=np.int64)
        st = Stats()
        self._check(self._lib.nwg_score_block(self.h, _p(xcodes, c_i8p), _p(xoffsets, c_i64p), nx,
                                              _p(ycodes, c_i8p), _p(yoffsets, c_i64p), ny, _p(D, c_f32p),
                                              D.strides[0] // 4, r0, mode, ctypes.byref(st)))
        return (D, st.as_dict()) if stats else D

    def set_trace_lanes(self, lanes: int):
        """Front width of the traceback kernel (32, 16 or 8 lanes per pair;
        0: chosen per call)."""
        self._check(self._lib.nwg_set_trace_lanes(self.h, int(lanes)))

    def align_pairs(self, codes, offsets, px, py, stats: bool = False):
        """Gapped alignments (X = px[k] columns, Y = py[k] rows): list of
        (aligned_x, aligned_y, score) in forward order."""
        px = np.ascontiguousarray(px, dtype=np.int32)
        py = np.ascontiguousarray(py, dtype=np.int32)
        offsets = np.ascontiguousarray(offsets, dtype=np.int64)
        codes = np.ascontiguousarray(codes, dtype=np.int8)
        m = len(px)
        L = np.diff(offsets)
        stride = int((L[px] + L[py]).max()) + 1 if m else 1
        bx = ctypes.create_string_buffer(max(m * stride, 1))
        by = ctypes.create_string_buffer(max(m * stride, 1))
        ln = np.zeros(max(m, 1), dtype=np.int32)
        sc = np.zeros(max(m, 1), dtype=np.int32)
        st = Stats()
        self._check(self._lib.nwg_align_pairs(self.h, _p(codes, c_i8p), _p(offsets, c_i64p), len(offsets) - 1,
                                              _p(px, c_i32p), _p(py, c_i32p), m, bx, by, stride,
                                              _p(ln, c_i32p), _p(sc, c_i32p), ctypes.byref(st)))
        rawx, rawy = bx.raw, by.raw
        out = [(rawx[k * stride:k * stride + ln[k]], rawy[k * stride:k * stride + ln[k]], int(sc[k]))
               for k in range(m)]
        return (out, st.as_dict()) if stats else out

    def nj(self, D, stats: bool = False):
        """Neighbor joining on the device: structured array of the n-1 joins."""
        from ._native import JOIN_DTYPE, NJStats
        D = np.ascontiguousarray(D, dtype=np.float32)
        n = D.shape[0]
        joins = np.zeros(max(n - 1, 1), dtype=np.dtype(JOIN_DTYPE))
        st = NJStats()
        self._check(self._lib.nwg_nj(self.h, _p(D, c_f32p), D.strides[0] // 4, n,
                                     joins.ctypes.data_as(ctypes.c_void_p), ctypes.byref(st)))
        joins = joins[: max(n - 1, 0)]
        return (joins, st.as_dict()) if stats else joins

    def nj_dev(self, d_D: int, n: int, ld: int, stats: bool = False):
        from ._native import JOIN_DTYPE, NJStats
        joins = np.zeros(max(n - 1, 1), dtype=np.dtype(JOIN_DTYPE))
        st = NJStats()
        self._check(self._lib.nwg_nj_dev(self.h, ctypes.c_void_p(d_D), ld, n,
                                         joins.ctypes.data_as(ctypes.c_void_p), ctypes.byref(st)))
        joins = joins[: max(n - 1, 0)]
        return (joins, st.as_dict()) if stats else joins

    def msa(self, seqs=None, left=None, right=None, *, codes=None, offsets=None, stats: bool = False):
        """Progressive alignment along the guide tree (node n+k joins left[k],
        right[k], e.g. the i and j of the nj() records): list of n gapped
        rows in forward order."""
        if codes is None:
            codes, offsets = encode(seqs)
        offsets = np.ascontiguousarray(offsets, dtype=np.int64)
        n = len(offsets) - 1
        left = np.ascontiguousarray(left if left is not None else [], dtype=np.int32)
        right = np.ascontiguousarray(right if right is not None else [], dtype=np.int32)
        L = ctypes.c_int64()
        st = Stats()
        self._check(self._lib.nwg_msa(self.h, _p(codes, c_i8p), _p(offsets, c_i64p), n, _p(left, c_i32p),
                                      _p(right, c_i32p), ctypes.byref(L), ctypes.byref(st)))
        buf = ctypes.create_string_buffer(max(n * L.value, 1))
        self._check(self._lib.nwg_msa_rows(self.h, buf, L.value))
        raw = buf.raw
        rows = [raw[k * L.value:(k + 1) * L.value] for k in range(n)]
        return (rows, st.as_dict()) if stats else rows

    def encode_dev(self, d_ascii: int, offsets, d_codes: int):
        """Encode and reverse on the device (device pointers, host offsets);
        returns the count of bytes outside the alphabet (codes -1 there)."""
        from ._native import NWG_ERR_BAD_RESIDUE
        offsets = np.ascontiguousarray(offsets, dtype=np.int64)
        bad = np.zeros(1, dtype=np.int64)
        st = self._lib.nwg_encode_dev(self.h, ctypes.c_void_p(d_ascii), _p(offsets, c_i64p), len(offsets) - 1,
                                      ctypes.c_void_p(d_codes), _p(bad, c_i64p))
        if st != NWG_ERR_BAD_RESIDUE:
            self._check(st)
        return int(bad[0])

    def parse_wire_dev(self, wire: bytes, d_wire: int, n: int, d_codes: int):
        """Offsets of the wire block's sequences and their codes on the device
        (d_wire: device copy of `wire`); returns (offsets, bad count)."""
        from ._native import NWG_ERR_BAD_RESIDUE
        off = np.zeros(n + 1, dtype=np.int64)
        bad = np.zeros(1, dtype=np.int64)
        st = self._lib.nwg_parse_wire_dev(self.h, wire, ctypes.c_void_p(d_wire), n, ctypes.c_void_p(d_codes),
                                          _p(off, c_i64p), _p(bad, c_i64p))
        if st != NWG_ERR_BAD_RESIDUE:
            self._check(st)
        return off, int(bad[0])

    def score_pairs(self, codes, offsets, pi, pj):
        """Scores of explicit pairs (int32 lanes, one thread per pair)."""
        pi = np.ascontiguousarray(pi, dtype=np.int32)
        pj = np.ascontiguousarray(pj, dtype=np.int32)
        out = np.zeros(len(pi), dtype=np.int32)
        offsets = np.ascontiguousarray(offsets, dtype=np.int64)
        self._check(self._lib.nwg_score_pairs(self.h, _p(codes, c_i8p), _p(offsets, c_i64p),
                                              len(offsets) - 1, _p(pi, c_i32p), _p(pj, c_i32p), len(pi),
                                              _p(out, c_i32p), None))
        return out


class Server:
    """The serving loop: alignment jobs (distance matrix + guide tree each)
    submitted at any time, admitted by HBM footprint and run in shared
    batches on the device (nwg_server_* in include/nwgpu.h)."""

    def __init__(self, gap_open: int = 10, gap_ext: int = 2, hbm_budget: int = 8 << 30,
                 max_batch_jobs: int = 256):
        self._lib = lib()
        h = ctypes.c_void_p()
        check(self._lib.nwg_server_create(gap_open, gap_ext, int(hbm_budget), int(max_batch_jobs),
                                          ctypes.byref(h)))
        self.h = h

    def submit(self, seqs) -> int:
        """Queue one job (its sequences); returns the job id at once."""
        res, off = _as_seq_list(seqs)
        off = np.ascontiguousarray(off, dtype=np.int64)
        jid = ctypes.c_uint64()
        check(self._lib.nwg_server_submit(self.h, res, _p(off, c_i64p), len(off) - 1, ctypes.byref(jid)))
        return jid.value

    def wait(self, job_id: int, n: int, timeout_ms: int = -1):
        """(D, joins, info) of a finished job; the job is released."""
        from ._native import JOIN_DTYPE, NWG_ERR_TIMEOUT, JobInfo
        D = np.zeros((n, n), dtype=np.float32)
        joins = np.zeros(max(n - 1, 1), dtype=np.dtype(JOIN_DTYPE))
        info = JobInfo()
        st = self._lib.nwg_server_wait(self.h, job_id, int(timeout_ms), _p(D, c_f32p),
                                       joins.ctypes.data_as(ctypes.c_void_p), ctypes.byref(info))
        if st == NWG_ERR_TIMEOUT:
            raise TimeoutError(f"job {job_id} not finished within {timeout_ms} ms")
        check(st)
        return D, joins[: max(n - 1, 0)], info.as_dict()

    def close(self):
        if getattr(self, "h", None):
            self._lib.nwg_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


def cherries(left, right, n_leaves: int):
    """(node, left, right) of every guide-tree cherry in getNodes post-order."""
    left = np.ascontiguousarray(left, dtype=np.int32)
    right = np.ascontiguousarray(right, dtype=np.int32)
    n = lib().nwg_cherries(_p(left, c_i32p), _p(right, c_i32p), n_leaves, None, None, None)
    if n < 0:
        raise NWGError(-n, "nwg_cherries")
    node = np.zeros(max(n, 1), dtype=np.int32)
    l = np.zeros(max(n, 1), dtype=np.int32)
    r = np.zeros(max(n, 1), dtype=np.int32)
    lib().nwg_cherries(_p(left, c_i32p), _p(right, c_i32p), n_leaves, _p(node, c_i32p), _p(l, c_i32p),
                       _p(r, c_i32p))
    return node[:n], l[:n], r[:n]


def newick(joins, names) -> str:
    """The reference's .tree text (TreeNode::buildTreeOutput + ";\\n")."""
    from ._native import JOIN_DTYPE
    j = np.ascontiguousarray(joins, dtype=np.dtype(JOIN_DTYPE))
    n = len(names)
    arr = (ctypes.c_char_p * n)(*[x.encode() if isinstance(x, str) else bytes(x) for x in names])
    need = lib().nwg_newick(j.ctypes.data_as(ctypes.c_void_p), n, arr, None, 0)
    if need < 0:
        raise NWGError(int(-need), "nwg_newick")
    buf = ctypes.create_string_buffer(int(need) + 1)
    lib().nwg_newick(j.ctypes.data_as(ctypes.c_void_p), n, arr, buf, need + 1)
    return buf.value.decode()


class AlignmentScore:
    """The reference class AlignmentScore (AlignmentScore.cuh:10-38) on libnwgpu.

    ``AlignmentScore(10, 2, 16, maxSeqLen)`` then ``loadDB(lbuf, lSz)`` and
    ``computeDistanceMtx(rbuf, rSz, distances, r0)`` as SpeciesBlock.cpp:361-363
    calls them.  ``distances`` is an (lSz x N) float32 array (or a list of
    per-row lists, as the C++ vector<vector<float>>); row x, column r0+y gets
    score(X_x, Y_y).  The window size is accepted and ignored: the GPU path
    has no windows.  Errors raise NWGError instead of exiting.
    """

    def __init__(self, gapOpen: int, gapExt: int, wSize: int, maxSeqLen: int):
        self.ctx = Context(gapOpen, gapExt)
        self.windowSize = wSize
        self.maxSeqLength = maxSeqLen
        self.xSize = 0
        self._x = None
        self._xbuf = None

    def parse(self, input: bytes, size: int):
        """Returns (codes, starts, lengths) -- AlignmentScore::parse's outputs."""
        codes, off = parse_wire(input, size)
        return codes, off[:-1].copy(), np.diff(off)

    def loadDB(self, lbuf: bytes, lSz: int):
        self.xSize = lSz
        self._xbuf = bytes(lbuf)
        self._x = parse_wire(lbuf, lSz)

    def computeDistanceMtx(self, rbuf: bytes, rSz: int, distances, r0: int):
        if self._x is None:
            raise NWGError(6, "loadDB must come first")
        ycodes, yoff = parse_wire(rbuf, rSz)
        xcodes, xoff = self._x
        as_list = not isinstance(distances, np.ndarray)
        same = (bytes(rbuf) == self._xbuf and rSz == self.xSize)
        if same:
            # the square, symmetric block of one rank: all pairs once
            D = self.ctx.score_all(codes=xcodes, offsets=xoff)
            block = D
        else:
            block = self.ctx.score_block(xcodes=xcodes, xoffsets=xoff, ycodes=ycodes, yoffsets=yoff)
        if as_list:
            for x in range(self.xSize):
                distances[x][r0:r0 + rSz] = block[x, :rSz].tolist()
        else:
            distances[:self.xSize, r0:r0 + rSz] = block[:, :rSz]
