"""ORACLE build recipe — test infrastructure only.

1. oracle/liboracle.so from oracle.c (the CPU restatement; builds anywhere).
2. When the reference tree is present (it is only on the development host;
   BNA_REFERENCE_ROOT names its root), oracle/_ref/ gets the reference's own
   CPU sources compiled as they lie there, with the shim headers of refshim/:
     libref_w.so  W/CorMat/CUCorMat/CUCorMat/CorMat.cpp   + ref_glue_w.cpp
     libref_u.so  U/CorMat/CorMat_CPU/CorMat/CorMat_CPU.cpp + ref_glue_u.cpp
     libref_m.so  U/Newman_Modularity_CPU/Modularity_CPU/Modularity_CPU.cpp
                  + ref_glue_m.cpp
   Both with -ffp-contract=off so they round exactly like the reference's
   scalar code.  main() of each file is renamed and never called.
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
# the reference tree (read-only); BNA_REFERENCE_ROOT points elsewhere, and
# where the tree is absent only liboracle.so is built
REF_ROOT = os.environ.get("BNA_REFERENCE_ROOT", "/root/reference/cuda_newest20160331")
W_SRC = os.path.join(REF_ROOT, "BNAPlatform-weighted-win64-cuda7.0-20160331", "src",
                     "CorMat", "CUCorMat", "CUCorMat", "CorMat.cpp")
U_SRC = os.path.join(REF_ROOT, "BNAPlatform-win64-cuda7.0-20160115", "src",
                     "CorMat", "CorMat_CPU", "CorMat", "CorMat_CPU.cpp")
M_SRC = os.path.join(REF_ROOT, "BNAPlatform-win64-cuda7.0-20160115", "src",
                     "Newman_Modularity_CPU", "Modularity_CPU", "Modularity_CPU.cpp")
LIB = os.path.join(HERE, "liboracle.so")
REF_DIR = os.path.join(HERE, "_ref")
REF_W = os.path.join(REF_DIR, "libref_w.so")
REF_U = os.path.join(REF_DIR, "libref_u.so")
REF_M = os.path.join(REF_DIR, "libref_m.so")


def _run(cmd, verbose):
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed: {' '.join(cmd)}\n{r.stderr}")


def _stale(out, srcs):
    return not os.path.exists(out) or any(os.path.getmtime(s) > os.path.getmtime(out) for s in srcs)


def build(verbose: bool = False) -> None:
    src = os.path.join(HERE, "oracle.c")
    if _stale(LIB, [src]):
        _run(["gcc", "-O2", "-std=c11", "-fPIC", "-shared", "-ffp-contract=off", "-pthread",
              src, "-o", LIB, "-lm"], verbose)
    if os.path.exists(W_SRC) and os.path.exists(U_SRC):
        os.makedirs(REF_DIR, exist_ok=True)
        shim = os.path.join(HERE, "refshim")
        common = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-w",
                  "-pthread", "-I", shim, "-Dmain=bna_ref_unused_main"]
        gw = os.path.join(HERE, "ref_glue_w.cpp")
        gu = os.path.join(HERE, "ref_glue_u.cpp")
        if _stale(REF_W, [W_SRC, gw]):
            _run(common + [W_SRC, gw, "-o", REF_W], verbose)
        if _stale(REF_U, [U_SRC, gu]):
            _run(common + [U_SRC, gu, "-o", REF_U], verbose)
        gm = os.path.join(HERE, "ref_glue_m.cpp")
        if os.path.exists(M_SRC) and _stale(REF_M, [M_SRC, gm, __file__]):
            # -Bsymbolic: the tool's global `verr` must not bind to libc's verr()
            _run(common + ["-Wl,-Bsymbolic", M_SRC, gm, "-o", REF_M], verbose)


if __name__ == "__main__":
    build(verbose="-v" in sys.argv)
