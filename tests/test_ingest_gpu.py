"""Residue encoding and reversal on the device (AlignmentScore::parse,
AlignmentScore.cu:142-178) against the host form and the oracle, with bytes
outside the alphabet; the serving loop encodes on the device too."""
import numpy as np
import pytest
import torch

import oracle_py as O
from mestrado_gb300 import NWGError, Server, encode, make_wire, parse_wire, synth
from mestrado_gb300._native import NWG_ERR_BAD_RESIDUE

pytestmark = pytest.mark.gpu


def _host_codes(seqs):
    # the reference's table: every byte outside the alphabet becomes -1
    order = b"ARNDCQEGHILKMFPSTWYVBZX*"
    tab = {c: k for k, c in enumerate(order)}
    return [np.array([tab.get(b, -1) for b in reversed(s)], dtype=np.int8) for s in seqs]


def test_encode_dev_matches_host(ctx):
    S = synth.family(300, 200, seed=5)
    seqs = [S[i] for i in range(len(S))] + [b"ARNDCQEGHILKMFPSTWYVBZX*", b"W"]
    codes, off = encode(seqs)
    assert np.array_equal(codes[: off[-1]], O.encode(seqs)[0][: off[-1]])
    res = b"".join(seqs)
    d_ascii = torch.frombuffer(bytearray(res), dtype=torch.uint8).cuda()
    d_codes = torch.empty(len(res), dtype=torch.int8, device="cuda")
    assert ctx.encode_dev(d_ascii.data_ptr(), off, d_codes.data_ptr()) == 0
    assert np.array_equal(d_codes.cpu().numpy(), codes[: off[-1]])


def test_encode_dev_counts_bytes_outside_the_alphabet(ctx):
    seqs = [b"ACDEFj", b"OUZ", b"MKV", b"acgt"]
    res = b"".join(seqs)
    off = np.cumsum([0] + [len(s) for s in seqs]).astype(np.int64)
    d_ascii = torch.frombuffer(bytearray(res), dtype=torch.uint8).cuda()
    d_codes = torch.empty(len(res), dtype=torch.int8, device="cuda")
    assert ctx.encode_dev(d_ascii.data_ptr(), off, d_codes.data_ptr()) == 1 + 2 + 4
    assert np.array_equal(d_codes.cpu().numpy(), np.concatenate(_host_codes(seqs)))


def test_parse_wire_dev_matches_host(ctx):
    S = synth.family(150, 120, seed=6)
    seqs = [S[i] for i in range(len(S))]
    wire = make_wire(seqs, rank=3)
    codes, off = parse_wire(wire, len(seqs))
    d_wire = torch.frombuffer(bytearray(wire), dtype=torch.uint8).cuda()
    d_codes = torch.empty(int(off[-1]), dtype=torch.int8, device="cuda")
    off2, bad = ctx.parse_wire_dev(wire, d_wire.data_ptr(), len(seqs), d_codes.data_ptr())
    assert bad == 0 and np.array_equal(off2, off)
    assert np.array_equal(d_codes.cpu().numpy(), codes[: off[-1]])


def test_serving_reports_bad_residues_per_job(ctx):
    good = synth.family(40, 100, seed=7)
    badjob = [good[0], good[1][:50] + b"j" + good[1][51:], good[2]]
    with Server(max_batch_jobs=8) as srv:
        a = srv.submit(good)
        b = srv.submit(badjob)
        D, J, info = srv.wait(a, len(good))
        with pytest.raises(NWGError) as e:
            srv.wait(b, len(badjob))
        assert e.value.status == NWG_ERR_BAD_RESIDUE
    assert np.array_equal(D, ctx.score_all(good))
