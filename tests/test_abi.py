"""The C ABI library loads and exports every symbol include/*.h declares;
host-only helpers (no device work) behave like the reference's parse."""
import ctypes
import os

import numpy as np
import pytest

import oracle_py as O
from mestrado_gb300 import _native, make_wire, parse_wire, encode
from mestrado_gb300 import synth


def test_library_exports_every_declared_symbol():
    lib = _native.lib()
    names = _native.exported_symbols()
    assert "nwg_score_all" in names and "nwg_ctx_create" in names
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_status_strings():
    lib = _native.lib()
    for s in range(0, 10):
        assert lib.nwg_status_str(s)


def test_wire_parse_matches_oracle():
    S = synth.family(9, 41, seed=4)          # odd lengths included
    wire = make_wire(S)
    codes, off = parse_wire(wire, len(S))
    oc = np.zeros_like(codes)
    ooff = np.zeros_like(off)
    O.lib().nwo_parse_wire(wire, len(S), oc.ctypes.data_as(ctypes.POINTER(ctypes.c_int8)),
                           ooff.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)))
    assert np.array_equal(off, ooff) and np.array_equal(codes, oc)
    ec, eo = encode(S)
    assert np.array_equal(ec, codes) and np.array_equal(eo, off)


def test_bad_residue_rejected():
    with pytest.raises(_native.NWGError) as e:
        encode([b"ACDJ"])
    assert e.value.status == _native.NWG_ERR_BAD_RESIDUE
    with pytest.raises(_native.NWGError) as e:
        encode([b"ACD", b""])
    assert e.value.status == _native.NWG_ERR_EMPTY_SEQ


def test_context_without_device_reports_no_device():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a device is present")
    with pytest.raises(_native.NWGError) as e:
        from mestrado_gb300 import Context
        Context(10, 2)
    assert e.value.status == _native.NWG_ERR_NO_DEVICE
