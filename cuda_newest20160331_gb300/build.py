"""Build libbna.so in-tree with nvcc for sm_103a (no cmake, no torch extension).

Every .cu / .cpp file of csrc/ is compiled in parallel into _build/ and linked
into cuda_newest20160331_gb300/libbna.so.  Objects are rebuilt when their
source or any header is newer.  Host C++ is compiled with -ffp-contract=off so
the synthetic generator gives the same bits on x86_64 and aarch64.
"""
from __future__ import annotations

import glob
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(PKG, "csrc")
ROOT = os.path.dirname(PKG)
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libbna.so")
BIN = os.path.join(PKG, "bin")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _cuda_home() -> str:
    for c in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if c and os.path.exists(os.path.join(c, "bin", "nvcc")):
            return c
    nvcc = shutil.which("nvcc")
    if nvcc:
        return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))
    raise RuntimeError("nvcc not found: set CUDA_HOME")


def _headers() -> list[str]:
    return glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(CSRC, "*.h")) + \
        glob.glob(os.path.join(INCLUDE, "*.h"))


def _stale(obj: str, src: str, deps: list[str]) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in [src, *deps])


def _run(cmd: list[str], verbose: bool) -> None:
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"build failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    if verbose and (r.stdout.strip() or r.stderr.strip()):
        print(r.stdout, r.stderr, flush=True)


def build(verbose: bool = False, ptxas_verbose: bool = False) -> str:
    cuda = _cuda_home()
    nvcc = os.path.join(cuda, "bin", "nvcc")
    os.makedirs(BUILD, exist_ok=True)
    deps = _headers()
    jobs = []
    objs = []
    for src in sorted(glob.glob(os.path.join(CSRC, "*.cu"))):
        obj = os.path.join(BUILD, os.path.basename(src) + ".o")
        objs.append(obj)
        if _stale(obj, src, deps) or ptxas_verbose:
            cmd = [nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-c", src, "-o", obj,
                   "-I", INCLUDE, "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
                   "--expt-relaxed-constexpr"]
            if ptxas_verbose:
                cmd += ["-Xptxas", "-v"]
            jobs.append(cmd)
    for src in sorted(glob.glob(os.path.join(CSRC, "*.cpp"))):
        obj = os.path.join(BUILD, os.path.basename(src) + ".o")
        objs.append(obj)
        if _stale(obj, src, deps):
            jobs.append(["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-c", src,
                         "-o", obj, "-I", INCLUDE, "-I", os.path.join(cuda, "include")])
    if jobs:
        with ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            list(ex.map(lambda c: _run(c, verbose), jobs))
    if jobs or not os.path.exists(LIB):
        libdir = os.path.join(cuda, "lib64")
        tmp = LIB + ".tmp"
        _run([nvcc, *ARCH, "-shared", "-o", tmp, *objs, "-cudart", "shared",
              "-Xlinker", f"-rpath,{libdir}", "-lpthread"], verbose)
        os.replace(tmp, LIB)
    # command-line drop-ins (cli/*.cpp -> bin/bna_<name>), linked to libbna.so
    os.makedirs(BIN, exist_ok=True)
    tools = []
    # cormat.cpp also as bna_cormat_u, the unweighted tree's CUCorMat
    variants = [(src, os.path.splitext(os.path.basename(src))[0], [])
                for src in sorted(glob.glob(os.path.join(PKG, "cli", "*.cpp")))]
    variants += [(os.path.join(PKG, "cli", "cormat.cpp"), "cormat_u", ["-DBNA_UNWEIGHTED_TREE"])]
    for src, name, defs in variants:
        exe = os.path.join(BIN, "bna_" + name)
        if _stale(exe, src, deps + [LIB]):
            tools.append(["g++", "-O2", "-std=c++17", *defs, src, "-o", exe, "-I", INCLUDE,
                          "-I", os.path.join(cuda, "include"), "-L", PKG, "-lbna",
                          "-L", os.path.join(cuda, "lib64"), "-lcudart",
                          "-Wl,-rpath,$ORIGIN/..", "-Wl,-rpath," + os.path.join(cuda, "lib64")])
    if tools:
        with ThreadPoolExecutor(max_workers=len(tools)) as ex:
            list(ex.map(lambda c: _run(c, verbose), tools))
    return LIB


if __name__ == "__main__":
    build(verbose="-v" in sys.argv, ptxas_verbose="--ptxas" in sys.argv)
    print(LIB)
