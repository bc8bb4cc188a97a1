"""Build recipe for the in-tree native libraries (no cmake, no setup.py).

* ``_build/librwnmr_gb300.so`` -- CUDA walker engine + C ABI (include/rwnmr_gb300.h), compiled by
  nvcc for sm_103a only, plus the C++ host frontend (configs, image I/O, walker placement,
  sequences) in ``csrc/host``.
* ``_build/rwnmr_gb300`` -- the command-line driver mirroring the reference's ``RWNMR`` binary.

Translation units compile in parallel; a rebuild only recompiles what changed.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
OUT = os.path.join(PKG, "_build")
LIB = os.path.join(OUT, "librwnmr_gb300.so")
CLI = os.path.join(OUT, "rwnmr_gb300")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off"]
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall", "-Wno-unused-function"]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build rwnmr_gb300")


def _cuda_home() -> str:
    return os.path.dirname(os.path.dirname(os.path.realpath(_nvcc())))


def _sources():
    cu = sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))
    hostdir = os.path.join(CSRC, "host")
    cpp = []
    if os.path.isdir(hostdir):
        cpp = sorted(os.path.join(hostdir, f) for f in os.listdir(hostdir) if f.endswith(".cpp") and f != "cli.cpp")
    return cu, cpp


def _headers():
    hs = [os.path.join(ROOT, "include", f) for f in os.listdir(os.path.join(ROOT, "include"))]
    for d, _, fs in os.walk(CSRC):
        hs += [os.path.join(d, f) for f in fs if f.endswith((".cuh", ".h", ".hpp"))]
    return hs


def _stale(target: str, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False) -> str:
    """Compiles the engine library and CLI; returns the library path."""
    os.makedirs(OUT, exist_ok=True)
    cu, cpp = _sources()
    headers = _headers()
    nvcc = _nvcc()
    inc = ["-I", os.path.join(ROOT, "include"), "-I", CSRC]
    jobs = []
    objs = []
    for src in cu:
        obj = os.path.join(OUT, os.path.basename(src) + ".o")
        objs.append(obj)
        if _stale(obj, [src] + headers):
            jobs.append([nvcc] + ARCH + NVCC_FLAGS + inc + ["-c", src, "-o", obj])
    for src in cpp:
        obj = os.path.join(OUT, os.path.basename(src) + ".o")
        objs.append(obj)
        if _stale(obj, [src] + headers):
            jobs.append(["g++"] + CXX_FLAGS + inc + ["-c", src, "-o", obj])
    procs = [(j, subprocess.Popen(j, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)) for j in jobs]
    failed = []
    for j, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            failed.append((j, out.decode(errors="replace")))
        elif verbose and out:
            sys.stdout.write(out.decode(errors="replace"))
    if failed:
        msg = "\n".join(" ".join(j) + "\n" + o for j, o in failed)
        raise RuntimeError("rwnmr_gb300 build failed:\n" + msg)
    if jobs or _stale(LIB, objs):
        subprocess.run([nvcc] + ARCH + ["-shared", "-o", LIB] + objs, check=True)
    cli_src = os.path.join(CSRC, "host", "cli.cpp")
    if os.path.exists(cli_src) and _stale(CLI, [cli_src, LIB] + headers):
        subprocess.run(["g++"] + CXX_FLAGS + inc + [cli_src, "-o", CLI, "-L", OUT, "-lrwnmr_gb300",
                        "-Wl,-rpath,$ORIGIN", "-L", os.path.join(_cuda_home(), "lib64"), "-lcudart"], check=True)
    return LIB


if __name__ == "__main__":
    print(build(verbose=True))
