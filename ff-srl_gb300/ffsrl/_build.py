"""Builds libffsrl_cuda.so in-tree for sm_103a (one nvcc per translation unit, in parallel).

The library is left at ``ffsrl/libffsrl_cuda.so``; object files go to ``csrc/_build/``.
A unit is recompiled when its source or a header is newer than its object.
"""

from __future__ import annotations

import os
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = ROOT / "csrc"
INCLUDE = ROOT.parent / "include"
BUILD = CSRC / "_build"
LIB = PKG / "libffsrl_cuda.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
          f"-I{INCLUDE}", f"-I{CSRC}"]
# per-unit extra flags: the reference-shaped step, the renderer and the reference-
# arithmetic batched step round every product as written (no fused multiply-add), like
# the CPU restatement; the fast batched step uses the hardware's approximate division and
# square root (within 2 ulp)
UNITS = {
    "capi.cu": [],
    "plain.cu": ["-fmad=false"],
    "batched.cu": ["-prec-div=false", "-prec-sqrt=false"],
    "batched_ref.cu": ["-fmad=false"],
    "batched_study.cu": ["-fmad=false"],
    "render.cu": ["-fmad=false"],
    "instrument.cu": ["-fmad=false"],
    "cutting.cu": ["-fmad=false"],
    "serve.cu": [],
    "handle.cu": [],
    "bvh_build.cpp": [],
}


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.sep not in cand or os.path.exists(cand)):
            return cand
    return "nvcc"


def _headers_mtime() -> float:
    hs = list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + list(INCLUDE.glob("*.h"))
    return max((h.stat().st_mtime for h in hs), default=0.0)


def build(verbose: bool = False, force: bool = False) -> Path:
    BUILD.mkdir(parents=True, exist_ok=True)
    nvcc = _nvcc()
    hm = _headers_mtime()
    jobs = []
    objs = []
    for unit, extra in UNITS.items():
        src = CSRC / unit
        obj = BUILD / (unit + ".o")
        objs.append(obj)
        if force or not obj.exists() or obj.stat().st_mtime < max(src.stat().st_mtime, hm):
            cmd = [nvcc, *ARCH, *COMMON, *extra, "-c", str(src), "-o", str(obj)]
            if unit.endswith(".cpp"):
                cmd = [nvcc, *COMMON, "-x", "c++", "-c", str(src), "-o", str(obj)]
            jobs.append(cmd)

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        if verbose and (r.stdout or r.stderr):
            print(r.stdout, r.stderr)

    with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        list(ex.map(run, jobs))
    if jobs or not LIB.exists():
        cmd = [nvcc, *ARCH, "-shared", "-o", str(LIB), *map(str, objs), "-lcudart"]
        run(cmd)
    return LIB


if __name__ == "__main__":
    import sys
    print(build(verbose=True, force="--force" in sys.argv))
