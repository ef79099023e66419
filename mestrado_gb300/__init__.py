"""mestrado_gb300 -- GB300-native all-pairs Needleman-Wunsch, cherry traceback
and neighbor joining for the ptersnow/mestrado progressive aligner.

The compute path is libnwgpu.so (hand-written sm_103a CUDA behind the C ABI of
include/nwgpu.h); this package is its Python host side:

* :class:`Context` -- one device context (gap penalties, matrix, stream);
* :class:`AlignmentScore` -- the reference class of AlignmentScore.cuh:10-38
  (``loadDB`` / ``computeDistanceMtx``) on top of the C ABI;
* :class:`Server` -- the serving loop (continuous batching of alignment jobs);
* :func:`make_wire` -- the sequence block of SpeciesBlock.cpp:309-322.
"""
from __future__ import annotations

from ._native import (MODE_BATCHED, MODE_BATCHED_INT32, MODE_PLAIN, NWGError, Stats, check, lib)
from .nwgpu import AlignmentScore, Context, Server, cherries, encode, make_wire, newick, parse_wire

__all__ = [
    "AlignmentScore", "Context", "Server", "cherries", "encode", "newick", "make_wire", "parse_wire", "NWGError", "Stats",
    "MODE_BATCHED", "MODE_PLAIN", "MODE_BATCHED_INT32", "check", "lib",
]
