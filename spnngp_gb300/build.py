"""Builds libspnngp_gb300.so in-tree from csrc/*.cu for sm_103a.

Every translation unit is compiled in parallel (the B/F kernel instantiations
are split across files for that reason), then linked into one shared library
with the CUDA runtime linked statically.  Objects go to ``_build/`` next to the
sources; the library lands next to this file.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libspnngp_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
              "--expt-relaxed-constexpr", "-diag-suppress", "177"]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build spnngp_gb300")


def _compile(nvcc: str, src: str, obj: str, extra: list[str]) -> tuple[str, int, str]:
    cmd = [nvcc, *NVCC_FLAGS, *ARCH, *extra, "-c", src, "-o", obj]
    p = subprocess.run(cmd, capture_output=True, text=True)
    return src, p.returncode, (p.stdout + p.stderr)


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, extra: list[str] | None = None, force: bool = False) -> str:
    """Compile (incrementally) and link the library; returns its path."""
    extra = list(extra or [])
    nvcc = _nvcc()
    os.makedirs(BUILD, exist_ok=True)
    sources = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    headers = sorted(glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh")) +
                     glob.glob(os.path.join(HERE, "..", "include", "*.h")))
    jobs = []
    objs = []
    for src in sources:
        obj = os.path.join(BUILD, os.path.basename(src)[:-3] + ".o")
        objs.append(obj)
        if force or _stale(obj, [src, *headers]):
            jobs.append((src, obj))
    if jobs:
        workers = max(1, min(len(jobs), os.cpu_count() or 4))
        with cf.ThreadPoolExecutor(workers) as ex:
            futs = [ex.submit(_compile, nvcc, s, o, extra) for s, o in jobs]
            for f in cf.as_completed(futs):
                src, rc, log = f.result()
                if verbose or rc != 0:
                    sys.stderr.write(log)
                if rc != 0:
                    raise RuntimeError(f"nvcc failed on {os.path.basename(src)}")
    if force or jobs or _stale(LIB, objs):
        cmd = [nvcc, *ARCH, "-shared", "-cudart", "static", "-o", LIB, *objs]
        p = subprocess.run(cmd, capture_output=True, text=True)
        if p.returncode != 0:
            sys.stderr.write(p.stdout + p.stderr)
            raise RuntimeError("linking libspnngp_gb300.so failed")
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="--force" in sys.argv))
