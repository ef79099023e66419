"""Seeded synthetic protein families (ctypes wrapper of libnwsynth.so).

The benchmark configurations name synthetic families of given shapes; the
model (Yule tree, per-edge substitutions and geometric indels) lives in
csrc/synth.cpp.  Sequences come back as ASCII ``bytes`` plus int32 lengths.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None

ROOT_FIXED, ROOT_UNIFORM, ROOT_LOGNORMAL = 0, 1, 2


class Spec(ctypes.Structure):
    _fields_ = [
        ("families", ctypes.c_int32),
        ("per_family", ctypes.c_int32),
        ("root_mode", ctypes.c_int32),
        ("clip_lo", ctypes.c_int32),
        ("clip_hi", ctypes.c_int32),
        ("pad", ctypes.c_int32),
        ("root_a", ctypes.c_double),
        ("root_b", ctypes.c_double),
        ("ps", ctypes.c_double),
        ("pi", ctypes.c_double),
    ]


class _Out(ctypes.Structure):
    _fields_ = [
        ("n", ctypes.c_int32),
        ("pad", ctypes.c_int32),
        ("total", ctypes.c_int64),
        ("residues", ctypes.POINTER(ctypes.c_char)),
        ("lengths", ctypes.POINTER(ctypes.c_int32)),
    ]


def _lib():
    global _LIB
    if _LIB is None:
        path = os.path.join(_HERE, "libnwsynth.so")
        if not os.path.exists(path):
            raise RuntimeError(f"{path} is missing: run __graft_entry__.build() first")
        lib = ctypes.CDLL(path)
        lib.nws_generate.argtypes = [ctypes.POINTER(Spec), ctypes.c_uint64, ctypes.POINTER(_Out)]
        lib.nws_generate.restype = ctypes.c_int
        lib.nws_release.argtypes = [ctypes.POINTER(_Out)]
        lib.nws_config_spec.argtypes = [ctypes.c_int, ctypes.POINTER(Spec)]
        lib.nws_config_spec.restype = ctypes.c_int
        lib.nws_config_seed.argtypes = [ctypes.c_int]
        lib.nws_config_seed.restype = ctypes.c_uint64
        _LIB = lib
    return _LIB


class SeqSet:
    """Concatenated ASCII residues plus lengths; ``seqs[i]`` gives bytes."""

    def __init__(self, residues: bytes, lengths: np.ndarray):
        self.residues = residues
        self.lengths = np.asarray(lengths, dtype=np.int64)
        self.offsets = np.zeros(len(self.lengths) + 1, dtype=np.int64)
        np.cumsum(self.lengths, out=self.offsets[1:])

    def __len__(self) -> int:
        return len(self.lengths)

    def __getitem__(self, i: int) -> bytes:
        return self.residues[self.offsets[i]:self.offsets[i + 1]]

    def subset(self, idx) -> "SeqSet":
        parts = [self[i] for i in idx]
        return SeqSet(b"".join(parts), np.array([len(p) for p in parts], dtype=np.int64))

    def cells(self) -> int:
        """Sum over i<j of L_i*L_j (the GCUPS work unit, diagonal excluded)."""
        L = self.lengths.astype(np.float64)
        s = L.sum()
        return int(round((s * s - (L * L).sum()) / 2))

    def to_fasta(self, path: str, prefix: str = "s") -> None:
        with open(path, "w") as f:
            for i in range(len(self)):
                f.write(f">{prefix}{i}\n")
                seq = self[i].decode()
                for k in range(0, len(seq), 60):
                    f.write(seq[k:k + 60] + "\n")


def generate(spec: Spec, seed: int) -> SeqSet:
    lib = _lib()
    out = _Out()
    rc = lib.nws_generate(ctypes.byref(spec), ctypes.c_uint64(seed), ctypes.byref(out))
    if rc != 0:
        raise ValueError(f"nws_generate failed ({rc})")
    try:
        res = ctypes.string_at(out.residues, out.total)
        lens = np.ctypeslib.as_array(out.lengths, shape=(out.n,)).astype(np.int64).copy()
    finally:
        lib.nws_release(ctypes.byref(out))
    return SeqSet(res, lens)


def config_spec(cfg: int) -> Spec:
    sp = Spec()
    if _lib().nws_config_spec(cfg, ctypes.byref(sp)) != 0:
        raise ValueError(f"unknown configuration {cfg}")
    return sp


def config_seed(cfg: int) -> int:
    return int(_lib().nws_config_seed(cfg))


def config(cfg: int) -> SeqSet:
    """Sequences of benchmark configuration ``cfg`` (0..3) with its seed."""
    return generate(config_spec(cfg), config_seed(cfg))


def family(per_family: int, root_len: int, ps: float = 0.05, pi: float = 0.005,
           families: int = 1, seed: int = 1, clip_lo: int = 1, clip_hi: int = 4000) -> SeqSet:
    sp = Spec(families=families, per_family=per_family, root_mode=ROOT_FIXED,
              clip_lo=clip_lo, clip_hi=clip_hi, root_a=float(root_len), ps=ps, pi=pi)
    return generate(sp, seed)


def lognormal_families(families: int, per_family: int, median: float, sigma: float,
                       clip_lo: int, clip_hi: int, ps: float, pi: float, seed: int) -> SeqSet:
    sp = Spec(families=families, per_family=per_family, root_mode=ROOT_LOGNORMAL,
              clip_lo=clip_lo, clip_hi=clip_hi, root_a=median, root_b=sigma, ps=ps, pi=pi)
    return generate(sp, seed)


def serving_jobs(count: int, rate: float = 200.0, seed: int | None = None,
                 n_lo: int = 8, n_hi: int = 512, median: float = 250.0, sigma: float = 0.5,
                 clip_lo: int = 30, clip_hi: int = 2000):
    """The serving workload: ``count`` independent families arriving as a
    Poisson process of ``rate`` jobs/s.  Each job has a log-uniform number of
    sequences in [n_lo, n_hi] and a lognormal root length (median, sigma)
    clipped to [clip_lo, clip_hi]; its sequences mutate as in the 64-sequence
    single-family configuration (ps 0.05, pi 0.005).  Returns a list of
    (arrival_s, SeqSet); per-job sub-seeds follow from ``seed`` (default: the
    serving configuration's seed)."""
    if seed is None:
        seed = config_seed(4)
    rng = np.random.default_rng(seed)
    t = np.cumsum(rng.exponential(1.0 / rate, size=count))
    ns = np.rint(np.exp(rng.uniform(np.log(n_lo), np.log(n_hi), size=count))).astype(int)
    sub = rng.integers(1, 2**62, size=count)
    jobs = []
    for k in range(count):
        S = lognormal_families(1, int(ns[k]), median, sigma, clip_lo, clip_hi, 0.05, 0.005, int(sub[k]))
        jobs.append((float(t[k]), S))
    return jobs
