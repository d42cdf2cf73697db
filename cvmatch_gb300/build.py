"""Builds the in-tree shared library cvmatch_gb300/_build/libcvmatch_gpu.so.

One nvcc translation unit (the sm_103a kernels) and two host C++ units,
compiled in parallel, then linked against the CUDA runtime.  Host code
is built with -ffp-contract=off (the twiddle generator must round every
operation), device code with -fmad=false (no contraction of the pinned
sequence).  No cmake; runs on x86_64 and aarch64 alike.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libcvmatch_gpu.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _cuda_home() -> str:
    home = os.environ.get("CUDA_HOME") or os.environ.get("CUDA_PATH")
    if home and os.path.isdir(home):
        return home
    nvcc = shutil.which("nvcc")
    if nvcc:
        return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))
    return "/usr/local/cuda"


def _sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC)
                  if f.endswith((".cu", ".cpp", ".h", ".cuh")))


def _stale() -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = _sources() + [os.path.join(ROOT, "include", "cvmatch_gpu.h"), __file__]
    return any(os.path.getmtime(p) > t for p in deps)


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and not _stale():
        return LIB
    os.makedirs(OUT, exist_ok=True)
    cuda = _cuda_home()
    nvcc = os.path.join(cuda, "bin", "nvcc")
    inc = ["-I" + os.path.join(ROOT, "include"), "-I" + CSRC]
    cuda_inc = "-I" + os.path.join(cuda, "include")
    jobs = []
    objs = []
    for f in sorted(os.listdir(CSRC)):
        src = os.path.join(CSRC, f)
        obj = os.path.join(OUT, f + ".o")
        if f.endswith(".cu"):
            cmd = [nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-fmad=false",
                   "-Xcompiler", "-fPIC,-ffp-contract=off", *inc, "-c", src, "-o", obj]
        elif f.endswith(".cpp"):
            cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-fno-fast-math",
                   "-Wall", *inc, cuda_inc, "-c", src, "-o", obj]
        else:
            continue
        objs.append(obj)
        jobs.append((cmd, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
    failed = False
    for cmd, p in jobs:
        out, _ = p.communicate()
        if p.returncode != 0 or verbose:
            sys.stderr.write(" ".join(cmd) + "\n" + out.decode(errors="replace"))
        failed |= p.returncode != 0
    if failed:
        raise RuntimeError("cvmatch_gb300: compiling the CUDA library failed")
    libdir = os.path.join(cuda, "lib64")
    if not os.path.isdir(libdir):
        libdir = os.path.join(cuda, "lib")
    tmp = LIB + ".tmp"
    link = ["g++", "-shared", "-o", tmp, *objs, "-L" + libdir, "-lcudart", "-Wl,-rpath," + libdir, "-lpthread"]
    r = subprocess.run(link, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
    if r.returncode != 0:
        sys.stderr.write(" ".join(link) + "\n" + r.stdout.decode(errors="replace"))
        raise RuntimeError("cvmatch_gb300: linking the CUDA library failed")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
