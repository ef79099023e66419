"""Drop-in check: the reference's own host program (wnj.cpp + SpeciesBlock.cpp
+ TreeNode.cpp + CmdLineOptions.cpp + FastaFile.cpp, compiled unchanged from
the reference checkout) builds and links against libnwgpu.so through
include/nwgpu_compat.hpp and the one-rank MPI stand-in.  Without a device it
then behaves as the reference does without one (AlignmentScore.cu:119-122):
prints the no-device line and exits 0.  Skipped where the reference checkout
is absent."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
from refsrc import REF

pytestmark = pytest.mark.skipif(not os.path.isfile(os.path.join(REF, "SpeciesBlock.cpp")),
                                reason="reference sources not present")


def test_reference_host_program_links_against_libnwgpu(tmp_path):
    from mestrado_gb300 import _native
    _native.lib()    # the library is built
    exe = tmp_path / "clustal"
    cmd = ["g++", "-O2", "-w", "-include", os.path.join(ROOT, "include", "nwgpu_compat.hpp"),
           "-I", os.path.join(ROOT, "oracle", "ref_shim"), "-I", os.path.join(ROOT, "include"),
           "-I", "/usr/local/cuda/include", "-I", REF,
           os.path.join(REF, "wnj.cpp"), os.path.join(REF, "SpeciesBlock.cpp"), os.path.join(REF, "TreeNode.cpp"),
           os.path.join(REF, "CmdLineOptions.cpp"), os.path.join(REF, "FastaFile.cpp"),
           "-L", os.path.join(ROOT, "mestrado_gb300"), "-lnwgpu",
           "-Wl,-rpath," + os.path.join(ROOT, "mestrado_gb300"), "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    fasta = tmp_path / "in.fasta"
    fasta.write_text(">a\nMKVLAAGIV\n>b\nMKVLSAGIV\n>c\nMRVLAAGLV\n")
    import torch
    if torch.cuda.is_available():
        pytest.skip("a device is present: the full run is covered by the GPU tests")
    r = subprocess.run([str(exe), str(fasta)], capture_output=True, text=True, cwd=tmp_path, timeout=60)
    assert r.returncode == 0
    assert "There are no available device(s) that support CUDA" in r.stderr
