"""The C++ drop-in on the device: a host program of this project's own
(tests/dropin_driver.cpp) includes include/nwgpu_compat.hpp, links
libnwgpu.so and calls the reference's class interface the way the aligner's
host code does -- AlignmentScore::loadDB / computeDistanceMtx with a full
square block, with two column blocks at r0 = 0 and r0 = h, and with a row
block of the second half (SpeciesBlock.cpp:356-363, :395), then
AlignmentMatch::computeAlignment on an iNode list of cherries
(SpeciesBlock.cpp:1402-1403, :1498).  Every matrix and every aligned pair is
compared with the oracle."""
import os
import subprocess

import numpy as np
import pytest

import oracle_py as O
from mestrado_gb300 import synth

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def driver(tmp_path_factory):
    from mestrado_gb300 import _native
    _native.lib()
    exe = str(tmp_path_factory.mktemp("dropin") / "dropin_driver")
    cmd = ["g++", "-O2", "-std=c++17", "-I", os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "dropin_driver.cpp"),
           "-L", os.path.join(ROOT, "mestrado_gb300"), "-lnwgpu",
           "-Wl,-rpath," + os.path.join(ROOT, "mestrado_gb300"), "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    return exe


@pytest.mark.parametrize("n,root,seed", [(37, 160, 5), (120, 420, 6)])
def test_compat_classes_on_the_device(driver, tmp_path, n, root, seed):
    S = synth.family(n, root, ps=0.08, pi=0.01, seed=seed)
    (tmp_path / "seqs.txt").write_bytes(b"\n".join(S) + b"\n")
    rng = np.random.default_rng(seed)
    perm = rng.permutation(n)
    pairs = [(int(perm[2 * k]), int(perm[2 * k + 1])) for k in range(n // 2)]
    (tmp_path / "cherries.txt").write_text("".join(f"{a} {b}\n" for a, b in pairs))
    prefix = str(tmp_path / "out")
    r = subprocess.run([driver, str(tmp_path / "seqs.txt"), str(tmp_path / "cherries.txt"), prefix],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-3000:]
    ref = O.score_all(S).astype(np.float32)
    h = n // 2
    square = np.fromfile(prefix + ".square", dtype=np.float32).reshape(n, n)
    split = np.fromfile(prefix + ".split", dtype=np.float32).reshape(n, n)
    rows = np.fromfile(prefix + ".rows", dtype=np.float32).reshape(n - h, n)
    assert np.array_equal(square, ref)
    assert np.array_equal(split, ref)
    assert np.array_equal(rows, ref[h:])
    lines = open(prefix + ".aln", "rb").read().split(b"\n")
    for k, (a, b) in enumerate(pairs):
        flag, ax, ay = lines[3 * k: 3 * k + 3]
        ox, oy, _ = O.traceback(S[a], S[b])
        assert flag == b"1"
        assert (ax, ay) == (ox, oy), f"cherry {a},{b}"
