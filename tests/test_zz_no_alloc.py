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


def _dev_arrays(codes, start, lens, pi, pj):
    import torch
    return (torch.from_numpy(codes).cuda(), torch.from_numpy(start).cuda(), torch.from_numpy(lens).cuda(),
            torch.from_numpy(pi).cuda(), torch.from_numpy(pj).cuda(),
            torch.full((len(pi),), -7, dtype=torch.int32, device="cuda"))


def _call(f, arrs, max_len, stream=None):
    d_codes, d_start, d_len, d_pi, d_pj, d_out = arrs
    return f(d_codes.data_ptr(), d_start.data_ptr(), d_len.data_ptr(), d_pi.data_ptr(), d_pj.data_ptr(),
             len(d_pi), d_out.data_ptr(), max_len, 10, 2, None, stream)


def test_noalloc_each_thread_scores_many_pairs():
    # max_len 32768 leaves room for 128 concurrent pairs: one block of 128
    # threads, so every thread walks the grid-stride loop about 25 times and
    # reuses its scratch column, once for a 30,000-residue X
    import torch
    f = _entry()
    seqs = _set(103, 40, 1, 400) + _set(104, 1, 30000, 30000)
    codes, off = encode(seqs)
    lens = np.diff(off).astype(np.int32)
    rng = np.random.default_rng(5)
    pi = rng.integers(0, 40, 3200).astype(np.int32)
    pj = rng.integers(0, 40, 3200).astype(np.int32)
    pi[:3], pj[:3] = 40, (0, 1, 2)          # the long sequence as X
    pi[3:6], pj[3:6] = (3, 4, 5), 40        # and as Y
    with Context(10, 2) as ctx:
        expect = ctx.score_pairs(codes, off, pi, pj)
    arrs = _dev_arrays(codes, off[:-1].copy(), lens, pi, pj)
    for call in range(2):
        arrs[-1].fill_(-7)
        torch.cuda.synchronize()
        assert _call(f, arrs, 32768) == NWG_OK
        torch.cuda.synchronize()
        assert np.array_equal(arrs[-1].cpu().numpy(), expect), f"call {call}: scores differ"


def test_noalloc_skips_pairs_outside_the_declared_size():
    # X longer than max_len, and an empty sequence on either side: INT_MIN,
    # no scratch access; every other pair is scored as usual
    import torch
    f = _entry()
    seqs = _set(105, 30, 1, 600)
    codes, off = encode(seqs)
    lens = np.diff(off).astype(np.int32)
    start = off[:-1].copy()
    # sequence 30: empty (length 0, starting at the end of the codes)
    lens = np.append(lens, np.int32(0))
    start = np.append(start, np.int64(off[-1]))
    rng = np.random.default_rng(9)
    pi = rng.integers(0, 31, 2500).astype(np.int32)
    pj = rng.integers(0, 31, 2500).astype(np.int32)
    pi[0], pj[0] = 30, 1
    pi[1], pj[1] = 2, 30
    max_len = 300
    bad = (lens[pi] > max_len) | (lens[pi] == 0) | (lens[pj] == 0)
    assert bad.sum() > 100 and (~bad).sum() > 100
    with Context(10, 2) as ctx:
        good = ctx.score_pairs(codes, off, pi[~bad], pj[~bad])
    arrs = _dev_arrays(codes, start, lens, pi, pj)
    torch.cuda.synchronize()
    assert _call(f, arrs, max_len) == NWG_OK
    torch.cuda.synchronize()
    got = arrs[-1].cpu().numpy()
    assert np.all(got[bad] == np.iinfo(np.int32).min)
    assert np.array_equal(got[~bad], good)


def test_noalloc_call_leaves_free_device_memory_unchanged():
    # After the first call on the device (set-up, and the module's own load),
    # a call takes no device memory: the free amount the driver reports is the
    # same before and after it.
    import torch
    f = _entry()
    seqs = _set(106, 50, 1, 500)
    codes, off = encode(seqs)
    lens = np.diff(off).astype(np.int32)
    rng = np.random.default_rng(3)
    pi = rng.integers(0, 50, 4000).astype(np.int32)
    pj = rng.integers(0, 50, 4000).astype(np.int32)
    arrs = _dev_arrays(codes, off[:-1].copy(), lens, pi, pj)
    assert _call(f, arrs, int(lens.max())) == NWG_OK
    torch.cuda.synchronize()
    first = arrs[-1].cpu().numpy()
    free0, _ = torch.cuda.mem_get_info()
    arrs[-1].fill_(-7)
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert _call(f, arrs, int(lens.max())) == NWG_OK
    torch.cuda.synchronize()
    free2, _ = torch.cuda.mem_get_info()
    assert free1 == free0 and free2 == free1
    assert np.array_equal(arrs[-1].cpu().numpy(), first)
