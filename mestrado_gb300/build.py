"""In-tree build of the native libraries (no cmake, no pip install).

libnwgpu.so   CUDA kernels + C ABI, nvcc for sm_103a only
libnwsynth.so seeded synthetic families (host C++)

Objects go to mestrado_gb300/_build/, shared libraries next to this file.
Translation units compile in parallel; a unit is rebuilt when its source or a
header in csrc/ or include/ is newer than its object.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
INCLUDE = os.path.join(ROOT, "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
           "-I", INCLUDE, "-I", CSRC]
CXXFLAGS = ["-O2", "-std=c++17", "-fPIC", "-I", INCLUDE]


def _nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found")
    return cand


def _headers():
    return glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh")) + \
        glob.glob(os.path.join(INCLUDE, "*.h")) + glob.glob(os.path.join(INCLUDE, "*.hpp"))


def _stale(obj: str, src: str) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(p) > t for p in [src] + _headers())


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout)
    return r.stdout


def build(verbose: bool = False, extra_nvflags=None) -> None:
    os.makedirs(BUILD, exist_ok=True)
    nvcc = _nvcc()
    cu = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    cpp = [p for p in sorted(glob.glob(os.path.join(CSRC, "*.cpp"))) if not p.endswith("synth.cpp")]
    jobs = []
    objs = []
    for src in cu:
        obj = os.path.join(BUILD, os.path.basename(src) + ".o")
        objs.append(obj)
        if _stale(obj, src):
            jobs.append([nvcc, *ARCH, *NVFLAGS, *(extra_nvflags or []), "-c", src, "-o", obj])
    for src in cpp:
        obj = os.path.join(BUILD, os.path.basename(src) + ".o")
        objs.append(obj)
        if _stale(obj, src):
            jobs.append(["g++", *CXXFLAGS, "-I", CSRC, "-I", "/usr/local/cuda/include", "-c", src, "-o", obj])
    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        for out in ex.map(_run, jobs):
            if verbose and out.strip():
                print(out)
    lib = os.path.join(HERE, "libnwgpu.so")
    if jobs or not os.path.exists(lib):
        _run([nvcc, *ARCH, "-shared", "-o", lib, *objs, "-lcudart"])
    synth_src = os.path.join(CSRC, "synth.cpp")
    slib = os.path.join(HERE, "libnwsynth.so")
    if _stale(slib, synth_src):
        _run(["g++", *CXXFLAGS, "-shared", "-o", slib, synth_src])


if __name__ == "__main__":
    build(verbose="-v" in sys.argv)
    print("built", os.path.join(HERE, "libnwgpu.so"))
