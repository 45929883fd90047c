"""Build the CUDA library of the FLIP substep in-tree (vare_gb300/_lib/libbora_flip.so).

Each translation unit is compiled by nvcc for sm_103a in parallel, then linked into one
shared library with a plain C ABI (include/bora_flip.h). No torch types cross the
boundary, so the library loads into any host process (ctypes, a C++ plugin, ...).

Floating-point contraction is disabled (-fmad=false) in the translation units whose
kernels restate the reference's float arithmetic, so that they round exactly like it;
their solver kernels call fmaf explicitly where they want fused multiply-adds. The
multigrid preconditioner restates nothing of the reference and is compiled with
contraction on (CONTRACT below); its double-float helpers multiply with __fmul_rn, which
is never contracted.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_lib")
LIB = os.path.join(OUT, "libbora_flip.so")

SOURCES = ["scan.cu", "grid_build.cu", "p2g.cu", "projection.cu", "multigrid.cu", "mg_mid.cu", "mg_passes.cu", "g2p.cu", "surface.cu",
           "vdb_export.cu", "tune.cu", "flip_api.cu", "serve.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
              "--expt-relaxed-constexpr", "-Xcudafe", "--diag_suppress=177"]
CONTRACT = {"multigrid.cu", "mg_mid.cu", "mg_passes.cu"}  # translation units compiled with -fmad=true


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _compile(src: str, verbose: bool) -> str:
    obj = os.path.join(OUT, os.path.splitext(src)[0] + ".o")
    path = os.path.join(CSRC, src)
    deps = [path] + [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith((".cuh", ".h"))]
    deps.append(os.path.join(HERE, "..", "include", "bora_flip.h"))
    if os.path.exists(obj) and all(os.path.getmtime(obj) >= os.path.getmtime(d) for d in deps):
        return obj
    fmad = "-fmad=true" if src in CONTRACT else "-fmad=false"
    cmd = [nvcc(), *ARCH, *NVCC_FLAGS, fmad, "-I", CSRC, "-c", path, "-o", obj]
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    if verbose:
        sys.stderr.write(r.stderr)
    return obj


def build(verbose: bool = False) -> str:
    os.makedirs(OUT, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose), SOURCES))
    if not os.path.exists(LIB) or any(os.path.getmtime(o) > os.path.getmtime(LIB) for o in objs):
        cmd = [nvcc(), *ARCH, "-shared", "-cudart", "static", "-o", LIB, *objs]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
