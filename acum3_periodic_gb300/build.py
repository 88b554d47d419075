"""Builds libacum.so (the C ABI of include/acum.h) and the acum_gb300 host executable
in-tree, under acum3_periodic_gb300/_build/, for sm_103a only.

CUDA sources go through nvcc with ``-gencode arch=compute_103a,code=sm_103a``; host C++
through g++; the translation units compile in parallel.  A stamp of the sources and
flags skips the rebuild when nothing changed.
"""
from __future__ import annotations

import hashlib
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libacum.so")
EXE = os.path.join(OUT, "acum_gb300")

CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA_HOME, "bin", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
                     "--expt-relaxed-constexpr", "-I" + os.path.join(ROOT, "include")]
CXX_FLAGS = ["-O2", "-fPIC", "-std=c++17", "-Wall", "-Wno-unused-function", "-I" + os.path.join(CUDA_HOME, "include"),
             "-I" + os.path.join(ROOT, "include"), "-pthread"]

CU_SOURCES = ["tonal.cu", "bpm.cu", "adjoint.cu", "probe.cu", "noalloc.cu", "permeable.cu"]
CPP_SOURCES = ["abi.cpp", "io.cpp", "batch.cpp"]


def _sources():
    cu = [s for s in CU_SOURCES if os.path.exists(os.path.join(CSRC, s))]
    cpp = [s for s in CPP_SOURCES if os.path.exists(os.path.join(CSRC, s))]
    return cu, cpp


def _stamp(cu, cpp) -> str:
    h = hashlib.sha256()
    for d in (CSRC, os.path.join(ROOT, "include")):
        for f in sorted(os.listdir(d)):
            p = os.path.join(d, f)
            if os.path.isfile(p):
                h.update(f.encode())
                with open(p, "rb") as fh:
                    h.update(fh.read())
    h.update(" ".join(NVCC_FLAGS + CXX_FLAGS + cu + cpp).encode())
    h.update(os.uname().machine.encode())
    return h.hexdigest()


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout)
    return r.stdout


def build(force: bool = False, verbose: bool = False) -> str:
    cu, cpp = _sources()
    os.makedirs(OUT, exist_ok=True)
    stamp = _stamp(cu, cpp)
    sf = os.path.join(OUT, "stamp")
    if not force and os.path.exists(LIB) and os.path.exists(EXE) and os.path.exists(sf):
        with open(sf) as f:
            if f.read() == stamp:
                return LIB
    jobs = []
    objs = []
    for s in cu:
        o = os.path.join(OUT, s + ".o")
        objs.append(o)
        jobs.append([NVCC] + NVCC_FLAGS + ["-c", os.path.join(CSRC, s), "-o", o])
    for s in cpp:
        o = os.path.join(OUT, s + ".o")
        objs.append(o)
        jobs.append(["g++"] + CXX_FLAGS + ["-c", os.path.join(CSRC, s), "-o", o])
    with ThreadPoolExecutor(max_workers=min(8, len(jobs))) as ex:
        logs = list(ex.map(_run, jobs))
    if verbose:
        for l in logs:
            sys.stdout.write(l)
    tmp = LIB + ".%d.tmp" % os.getpid()
    _run([NVCC] + ARCH + ["-shared", "-o", tmp] + objs + ["-Xcompiler", "-pthread"])
    os.replace(tmp, LIB)
    tmpe = EXE + ".%d.tmp" % os.getpid()
    _run(["g++", "-O2", "-std=c++17", "-I" + os.path.join(ROOT, "include"), os.path.join(CSRC, "main.cpp"),
          "-o", tmpe, "-L" + OUT, "-lacum", "-Wl,-rpath,$ORIGIN"])
    os.replace(tmpe, EXE)
    with open(sf, "w") as f:
        f.write(stamp)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
    print(LIB)
