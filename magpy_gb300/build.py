"""Builds the CUDA library libmagpy_gpu.so in-tree (sm_103a only).

Each translation unit of csrc/ is compiled in parallel with nvcc and linked
into magpy_gb300/_lib/libmagpy_gpu.so.  The FP64-faithful kernel is compiled
without fused multiply-add contraction (-fmad=false) so that every product
and sum rounds as in the reference's C++.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(os.path.dirname(PKG), "include")
OBJ = os.path.join(PKG, "_build")
LIBDIR = os.path.join(PKG, "_lib")
LIB = os.path.join(LIBDIR, "libmagpy_gpu.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
          "-I", CSRC, "-I", INCLUDE, "--expt-relaxed-constexpr"]
# per-unit extra flags
UNITS = {
    "sllg_fp64.cu": ["-fmad=false"],
    "dom.cu": ["-fmad=false"],
    "sllg_mixed.cu": [],
    "capi.cu": [],
}
EXTRA_UNITS_GLOB = ".cu"


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build magpy_gb300")


def _units() -> dict[str, list[str]]:
    units = dict(UNITS)
    for f in sorted(os.listdir(CSRC)):
        if f.endswith(EXTRA_UNITS_GLOB) and f not in units:
            units[f] = []
    return units


def _headers_mtime() -> float:
    paths = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".hpp"))]
    paths += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE)]
    return max(os.path.getmtime(p) for p in paths)


def build(verbose: bool = False, force: bool = False) -> str:
    """Compile (if stale) and return the path of libmagpy_gpu.so."""
    os.makedirs(OBJ, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    nvcc = _nvcc()
    hdr = _headers_mtime()
    # rebuild everything when the flags or the toolkit change
    stamp = os.path.join(OBJ, "flags.txt")
    sig = repr((nvcc, ARCH, COMMON, sorted(_units().items())))
    if not os.path.exists(stamp) or open(stamp).read() != sig:
        force = True
    jobs = []
    objs = []
    for unit, flags in _units().items():
        src = os.path.join(CSRC, unit)
        obj = os.path.join(OBJ, unit.replace(".cu", ".o"))
        objs.append(obj)
        stale = force or not os.path.exists(obj) or os.path.getmtime(obj) < max(
            os.path.getmtime(src), hdr)
        if stale:
            jobs.append([nvcc, *ARCH, *COMMON, *flags, "-c", src, "-o", obj])
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        results = list(ex.map(lambda cmd: subprocess.run(cmd, capture_output=True, text=True),
                              jobs))
    for cmd, r in zip(jobs, results):
        if verbose or r.returncode != 0:
            sys.stderr.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {cmd[-3]}")
    with open(stamp, "w") as f:
        f.write(sig)
    if jobs or not os.path.exists(LIB):
        cmd = [nvcc, *ARCH, "-shared", "-o", LIB, *objs, "-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            sys.stderr.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
            raise RuntimeError("link of libmagpy_gpu.so failed")
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
