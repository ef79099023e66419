"""ctypes binding of libnwgpu.so (the C ABI of include/nwgpu.h).

The library is loaded from this package directory only; there is no fallback.
If it is missing the import fails loudly -- build it with
``python -c "import __graft_entry__ as g; g.build()"``.
"""
from __future__ import annotations

import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libnwgpu.so")

P = ctypes.POINTER
c_i8p = P(ctypes.c_int8)
c_i32p = P(ctypes.c_int32)
c_i64p = P(ctypes.c_int64)
c_f32p = P(ctypes.c_float)
c_f64p = P(ctypes.c_double)

NWG_OK = 0
NWG_ERR_NO_DEVICE = 1
NWG_ERR_OOM = 2
NWG_ERR_BAD_RESIDUE = 3
NWG_ERR_TIMEOUT = 4
NWG_ERR_OVERFLOW = 5
NWG_ERR_INVALID = 6
NWG_ERR_CUDA = 7
NWG_ERR_EMPTY_SEQ = 8
NWG_ERR_NJ_AMBIGUOUS = 9

MODE_BATCHED = 0
MODE_PLAIN = 1
MODE_BATCHED_INT32 = 2


class Stats(ctypes.Structure):
    _fields_ = [
        ("pairs", ctypes.c_int64),
        ("cells", ctypes.c_int64),
        ("pairs_int16", ctypes.c_int64),
        ("pairs_int32", ctypes.c_int64),
        ("reruns", ctypes.c_int64),
        ("launches", ctypes.c_int32),
        ("buckets", ctypes.c_int32),
        ("kernel_ms", ctypes.c_double),
        ("h2d_ms", ctypes.c_double),
        ("d2h_ms", ctypes.c_double),
        ("total_ms", ctypes.c_double),
    ]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class NWGError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"nwgpu status {status}: {msg}")
        self.status = status


_SIGS = {
    "nwg_status_str": ([ctypes.c_int], ctypes.c_char_p),
    "nwg_ctx_create": ([ctypes.c_int, ctypes.c_int, c_i8p, P(ctypes.c_void_p)], ctypes.c_int),
    "nwg_ctx_destroy": ([ctypes.c_void_p], ctypes.c_int),
    "nwg_set_stream": ([ctypes.c_void_p, ctypes.c_void_p], ctypes.c_int),
    "nwg_last_error": ([ctypes.c_void_p], ctypes.c_char_p),
    "nwg_parse_wire": ([ctypes.c_char_p, ctypes.c_int, c_i8p, c_i64p], ctypes.c_int),
    "nwg_encode": ([ctypes.c_char_p, c_i64p, ctypes.c_int, c_i8p], ctypes.c_int),
    "nwg_score_all": ([ctypes.c_void_p, c_i8p, c_i64p, ctypes.c_int, c_f32p, ctypes.c_int64,
                       ctypes.c_int, P(Stats)], ctypes.c_int),
    "nwg_score_all_dev": ([ctypes.c_void_p, ctypes.c_void_p, c_i64p, ctypes.c_int, ctypes.c_void_p,
                           ctypes.c_int64, ctypes.c_int, P(Stats)], ctypes.c_int),
    "nwg_score_block": ([ctypes.c_void_p, c_i8p, c_i64p, ctypes.c_int, c_i8p, c_i64p, ctypes.c_int,
                         c_f32p, ctypes.c_int64, ctypes.c_int64, ctypes.c_int, P(Stats)], ctypes.c_int),
    "nwg_score_pairs": ([ctypes.c_void_p, c_i8p, c_i64p, ctypes.c_int, c_i32p, c_i32p, ctypes.c_int64,
                         c_i32p, P(Stats)], ctypes.c_int),
}

_lib = None


def lib():
    """The loaded libnwgpu.so with argument types set; raises if absent."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} is missing: the CUDA extension must be built "
                              "(__graft_entry__.build()); there is no CPU fallback")
        L = ctypes.CDLL(LIB_PATH)
        for name, (args, res) in _SIGS.items():
            f = getattr(L, name)
            f.argtypes = args
            f.restype = res
        for name, (args, res) in EXTRA_SIGS.items():
            if hasattr(L, name):
                f = getattr(L, name)
                f.argtypes = args
                f.restype = res
        _lib = L
    return _lib


class LaunchRec(ctypes.Structure):
    _fields_ = [
        ("kind", ctypes.c_int32),
        ("rows_per_lane", ctypes.c_int32),
        ("lanes16", ctypes.c_int32),
        ("grid", ctypes.c_int32),
        ("pairs", ctypes.c_int64),
        ("cells", ctypes.c_int64),
        ("ms", ctypes.c_double),
        ("variant", ctypes.c_int32),
        ("lanes", ctypes.c_int32),
    ]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


TUNE_CLASSES = 16
# Y rows of the tuning classes (the last one takes every longer Y)
TUNE_CLASS_ROWS = [64, 96, 128, 160, 192, 224, 256, 320, 384, 448, 512, 640, 768, 1024, 1536, 2**31 - 1]


class TuneResult(ctypes.Structure):
    _fields_ = [
        ("classes", ctypes.c_int32),
        ("from_cache", ctypes.c_int32),
        ("max_rows", ctypes.c_int32 * TUNE_CLASSES),
        ("rows_per_lane", ctypes.c_int32 * TUNE_CLASSES),
        ("variant", ctypes.c_int32 * TUNE_CLASSES),
        ("lanes", ctypes.c_int32 * TUNE_CLASSES),
        ("pad", ctypes.c_int32),
        ("gcups", ctypes.c_double * TUNE_CLASSES),
        ("seconds", ctypes.c_double),
    ]

    def as_dict(self):
        n = self.classes
        return {"from_cache": bool(self.from_cache), "seconds": self.seconds,
                "classes": [{"max_rows": self.max_rows[k], "rows_per_lane": self.rows_per_lane[k],
                             "variant": self.variant[k], "lanes": self.lanes[k], "gcups": self.gcups[k]}
                            for k in range(n)]}


class Join(ctypes.Structure):
    _fields_ = [
        ("i", ctypes.c_int32), ("j", ctypes.c_int32), ("node", ctypes.c_int32), ("n", ctypes.c_int32),
        ("d", ctypes.c_float), ("pad", ctypes.c_float), ("q", ctypes.c_double),
        ("ti", ctypes.c_double), ("tj", ctypes.c_double),
        ("len_i", ctypes.c_double), ("len_j", ctypes.c_double),
    ]


class NJStats(ctypes.Structure):
    _fields_ = [("ambiguous_steps", ctypes.c_int64), ("tie_steps", ctypes.c_int64),
                ("rebuilds", ctypes.c_int64), ("pq_trigger_open", ctypes.c_int64),
                ("device_ms", ctypes.c_double), ("launches", ctypes.c_int32),
                ("reference_identical", ctypes.c_int32)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_ if k != "pad"}


JOIN_DTYPE = [("i", "i4"), ("j", "i4"), ("node", "i4"), ("n", "i4"), ("d", "f4"), ("pad", "f4"),
              ("q", "f8"), ("ti", "f8"), ("tj", "f8"), ("len_i", "f8"), ("len_j", "f8")]

class JobInfo(ctypes.Structure):
    _fields_ = [("n", ctypes.c_int32), ("status", ctypes.c_int32), ("batch_jobs", ctypes.c_int32),
                ("nj_reference_identical", ctypes.c_int32), ("queue_ms", ctypes.c_double), ("latency_ms", ctypes.c_double),
                ("cells", ctypes.c_int64), ("nj_ambiguous_steps", ctypes.c_int64),
                ("nj_tie_steps", ctypes.c_int64), ("nj_rebuilds", ctypes.c_int64)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_ if k != "pad"}


EXTRA_SIGS: dict = {
    "nwg_nj": ([ctypes.c_void_p, c_f32p, ctypes.c_int64, ctypes.c_int, ctypes.c_void_p, P(NJStats)],
               ctypes.c_int),
    "nwg_nj_dev": ([ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_int, ctypes.c_void_p,
                    P(NJStats)], ctypes.c_int),
    "nwg_newick": ([ctypes.c_void_p, ctypes.c_int, P(ctypes.c_char_p), ctypes.c_char_p, ctypes.c_int64],
                   ctypes.c_int64),
    "nwg_autotune": ([ctypes.c_void_p, ctypes.c_int, P(TuneResult)], ctypes.c_int),
    "nwg_set_tuning": ([ctypes.c_void_p, c_i32p, c_i32p], ctypes.c_int),
    "nwg_set_tuning_lanes": ([ctypes.c_void_p, c_i32p, c_i32p, c_i32p], ctypes.c_int),
    "nwg_align_pairs": ([ctypes.c_void_p, c_i8p, c_i64p, ctypes.c_int, c_i32p, c_i32p, ctypes.c_int,
                         ctypes.c_char_p, ctypes.c_char_p, ctypes.c_int64, c_i32p, c_i32p, P(Stats)],
                        ctypes.c_int),
    "nwg_set_trace_lanes": ([ctypes.c_void_p, ctypes.c_int], ctypes.c_int),
    "nwg_cherries": ([c_i32p, c_i32p, ctypes.c_int, c_i32p, c_i32p, c_i32p], ctypes.c_int),
    "nwg_dpx_peak": ([ctypes.c_void_p, ctypes.c_int, P(ctypes.c_double)], ctypes.c_int),
    "nwg_dpx_peak_form": ([ctypes.c_void_p, ctypes.c_int, ctypes.c_int, P(ctypes.c_double)], ctypes.c_int),
    "nwg_msa": ([ctypes.c_void_p, c_i8p, c_i64p, ctypes.c_int, c_i32p, c_i32p, c_i64p, P(Stats)], ctypes.c_int),
    "nwg_msa_rows": ([ctypes.c_void_p, ctypes.c_char_p, ctypes.c_int64], ctypes.c_int),
    "nwg_encode_dev": ([ctypes.c_void_p, ctypes.c_void_p, c_i64p, ctypes.c_int, ctypes.c_void_p, c_i64p],
                       ctypes.c_int),
    "nwg_parse_wire_dev": ([ctypes.c_void_p, ctypes.c_char_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, c_i64p,
                            c_i64p], ctypes.c_int),
    "nwg_set_launch_timing": ([ctypes.c_void_p, ctypes.c_int], ctypes.c_int),
    "nwg_launch_records": ([ctypes.c_void_p, P(LaunchRec), ctypes.c_int], ctypes.c_int),
    "nwg_server_create": ([ctypes.c_int, ctypes.c_int, ctypes.c_int64, ctypes.c_int, P(ctypes.c_void_p)],
                          ctypes.c_int),
    "nwg_server_submit": ([ctypes.c_void_p, ctypes.c_char_p, c_i64p, ctypes.c_int, P(ctypes.c_uint64)],
                          ctypes.c_int),
    "nwg_server_wait": ([ctypes.c_void_p, ctypes.c_uint64, ctypes.c_int, c_f32p, ctypes.c_void_p, P(JobInfo)],
                        ctypes.c_int),
    "nwg_server_destroy": ([ctypes.c_void_p], ctypes.c_int),
}


def exported_symbols():
    """Names of the C ABI declared in include/*.h, as parsed from the headers."""
    import re
    inc = os.path.join(os.path.dirname(HERE), "include")
    names = []
    for fn in sorted(os.listdir(inc)):
        if not fn.endswith(".h") or fn == "nwgpu_synth.h":
            continue
        txt = open(os.path.join(inc, fn)).read()
        txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
        names += re.findall(r"\b(nwg_[a-z0-9_]+)\s*\(", txt)
    return sorted(set(names))


def check(status: int, ctx=None) -> None:
    if status != NWG_OK:
        msg = lib().nwg_status_str(status).decode()
        if ctx is not None:
            extra = lib().nwg_last_error(ctx)
            if extra:
                msg += " (" + extra.decode() + ")"
        raise NWGError(status, msg)
