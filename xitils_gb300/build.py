"""Build recipe for libxgb.so (sm_103a only).

Each CUDA translation unit is compiled by nvcc in parallel with
``-gencode arch=compute_103a,code=sm_103a`` and linked into the in-tree shared
library ``xitils_gb300/libxgb.so`` (CUDA runtime linked statically; no PyTorch
dependency). Per-unit flags:
  * integrator.cu, shade_*.cu, svndf.cu: ``-fmad=false``
    -- shading and fitting arithmetic stays unfused, as in the reference's float code;
  * api.cu: host code compiled with ``-ffp-contract=off`` for the same reason.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libxgb.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr", "-Xptxas", "-v"]
UNITS = {
    "api.cu": ["-Xcompiler", "-ffp-contract=off"],
    "bvh_build.cu": [],
    "trace.cu": [],
    "integrator.cu": ["-fmad=false"],
    "noalloc.cu": [],
    "guide.cu": [], "guide_tc.cu": [], "image.cu": [], "batch.cu": [],
    "svndf.cu": ["-fmad=false"],
    "shade_layered.cu": ["-fmad=false"], "shade_nested.cu": ["-fmad=false"], "shade_batch_nested.cu": ["-fmad=false"],
}


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise FileNotFoundError("nvcc not found")


def _deps() -> list[str]:
    out = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    out.append(os.path.join(os.path.dirname(PKG), "include", "xgb.h"))
    return out


def _compile(unit: str, extra: list[str]) -> tuple[str, str]:
    obj = os.path.join(BUILD, unit + ".o")
    cmd = [nvcc(), "-c"] + ARCH + COMMON + extra + [os.path.join(CSRC, unit), "-o", obj]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc failed for {unit}:\n{' '.join(cmd)}\n{res.stderr[-6000:]}")
    return obj, res.stderr


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    newest = max(os.path.getmtime(p) for p in _deps())
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= newest:
        return LIB
    with cf.ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        results = list(ex.map(lambda kv: _compile(*kv), UNITS.items()))
    if verbose:
        for _, log in results:
            sys.stderr.write(log)
    objs = [r[0] for r in results]
    tmp = LIB + ".tmp"
    cmd = [nvcc(), "-shared"] + ARCH + objs + ["-o", tmp]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"link failed:\n{' '.join(cmd)}\n{res.stderr[-4000:]}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
