"""nwg_score_pairs_noalloc: the pair-scoring entry point for hosts that cannot
let a library allocate (stream capture in the global mode, hosts that own all
device memory).  It must give exactly the scores of the existing pair-list
entry point, call after call, with its work memory in a static device array.
Collected last so that a run stopping at the first failure has run every other
test first; it also passes alone in a fresh process."""
import ctypes
import os

import numpy as np
import pytest

from mestrado_gb300 import Context, encode
from mestrado_gb300 import _native

pytestmark = pytest.mark.gpu

NWG_OK, NWG_ERR_INVALID = 0, 6


def _entry():
    lib = _native.lib()
    f = lib.nwg_score_pairs_noalloc
    vp = ctypes.c_void_p
    f.argtypes = [vp, vp, vp, vp, vp, ctypes.c_int64, vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, vp, vp]
    f.restype = ctypes.c_int
    return f


def _set(seed, n, lo, hi):
    rng = np.random.default_rng(seed)
    letters = np.frombuffer(b"ARNDCQEGHILKMFPSTWYVBZX*", dtype=np.uint8)
    lens = rng.integers(lo, hi + 1, size=n)
    return [letters[rng.integers(0, 24, L)].tobytes() for L in lens]


def test_noalloc_matches_pair_list_on_two_calls():
    import torch
    f = _entry()
    ctx = Context(10, 2)
    stream = torch.cuda.Stream()
    for call, (seed, n, lo, hi, npairs) in enumerate([(101, 60, 1, 700, 3000), (102, 45, 1, 1200, 2000)]):
        seqs = _set(seed, n, lo, hi)
        codes, off = encode(seqs)
        lens = np.diff(off).astype(np.int32)
        rng = np.random.default_rng(seed + 7)
        pi = rng.integers(0, n, npairs).astype(np.int32)
        pj = rng.integers(0, n, npairs).astype(np.int32)
        expect = ctx.score_pairs(codes, off, pi, pj)          # the existing entry point
        d_codes = torch.from_numpy(codes).cuda()
        d_start = torch.from_numpy(off[:-1].copy()).cuda()
        d_len = torch.from_numpy(lens).cuda()
        d_pi = torch.from_numpy(pi).cuda()
        d_pj = torch.from_numpy(pj).cuda()
        d_out = torch.full((npairs,), -7, dtype=torch.int32, device="cuda")
        torch.cuda.synchronize()
        rc = f(d_codes.data_ptr(), d_start.data_ptr(), d_len.data_ptr(), d_pi.data_ptr(), d_pj.data_ptr(),
               npairs, d_out.data_ptr(), int(lens.max()), 10, 2, None, stream.cuda_stream)
        assert rc == NWG_OK, f"call {call}: status {rc}"
        stream.synchronize()
        got = d_out.cpu().numpy()
        assert np.array_equal(got, expect), f"call {call}: scores differ"
    ctx.close()


def test_noalloc_rejects_sizes_beyond_its_maximum():
    f = _entry()
    # 32 MiB of (H, F) rows for at least 128 concurrent pairs: max_len <= 32768
    assert f(1, 1, 1, 1, 1, 1, 1, 32769, 10, 2, None, None) == NWG_ERR_INVALID
    assert f(1, 1, 1, 1, 1, 1, 1, 0, 10, 2, None, None) == NWG_ERR_INVALID
    assert f(None, None, None, None, None, 0, None, 100, 10, 2, None, None) == NWG_OK
