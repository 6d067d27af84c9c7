"""Builds libspnngp_gb300.so in-tree from csrc/*.cu for sm_103a.

Every translation unit is compiled in parallel, then linked into one shared
library with the CUDA runtime linked statically.  nngp_bf_inst.cu,
nngp_bfwd_inst.cu, nngp_bfr_inst.cu and nngp_bfw_inst.cu are compiled once per B/F kernel variant
(neighbor bound x correlation code) so the heavy kernel instantiations spread
over all cores.  Objects go to ``_build/`` next to the
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


# source -> [(object suffix, defines)]: sources compiled once per variant
# (FP64: the shared-memory kernel of nngp_bf_inst.cu for m <= 24, the warp-per-location
# kernel of nngp_bfwd_inst.cu for 24 < m <= 32; FP32R: the register kernel of nngp_bfr_inst.cu
# for m <= 16, the warp-per-location kernel of nngp_bfw_inst.cu for 16 < m <= 32, and the
# double-float re-solves of their flagged locations: thread per location for bounds 16 and 24,
# nngp_bfdf_inst.cu, warp per location for 32, nngp_bfwdf_inst.cu)
VARIANTS = {
    "nngp_bf_inst.cu": [(f"_m{m}_c{c}", [f"-DBF_M={m}", f"-DBF_COV={c}"])
                        for m in (16, 24) for c in (0, 1, 2, 3, 4)],
    "nngp_bfwd_inst.cu": [(f"_m{m}_c{c}", [f"-DBFWD_M={m}", f"-DBFWD_COV={c}"])
                          for m in (32,) for c in (0, 1, 2, 3, 4)],
    "nngp_bfr_inst.cu": [(f"_m{m}_c{c}", [f"-DBFR_M={m}", f"-DBFR_COV={c}"])
                         for m in (10, 15, 16) for c in (0, 1, 2, 3, 4)],
    "nngp_bfw_inst.cu": [(f"_m{m}_c{c}", [f"-DBFW_M={m}", f"-DBFW_COV={c}"])
                         for m in (20, 24, 32) for c in (0, 1, 2, 3, 4)],
    "nngp_bfdf_inst.cu": [(f"_m{m}_c{c}", [f"-DBFDF_M={m}", f"-DBFDF_COV={c}"])
                          for m in (16, 24) for c in (0, 1, 2, 3, 4)],
    "nngp_bfwdf_inst.cu": [(f"_m{m}_c{c}", [f"-DBFWDF_M={m}", f"-DBFWDF_COV={c}"])
                           for m in (32,) for c in (0, 1, 2, 3, 4)],
}


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
        base = os.path.basename(src)[:-3]
        for suffix, defs in VARIANTS.get(os.path.basename(src), [("", [])]):
            obj = os.path.join(BUILD, base + suffix + ".o")
            objs.append(obj)
            if force or _stale(obj, [src, *headers]):
                jobs.append((src, obj, defs))
    # stale objects of sources or variants that no longer exist must not be linked
    for old in glob.glob(os.path.join(BUILD, "*.o")):
        if old not in objs:
            os.remove(old)
    if jobs:
        workers = max(1, min(len(jobs), os.cpu_count() or 4))
        # heaviest first: the FP32R and general-model variants take longest
        jobs.sort(key=lambda j: ("bfw" not in j[1], "_c4" not in j[1], "_m32" not in j[1], "bfr" not in j[1]))
        with cf.ThreadPoolExecutor(workers) as ex:
            futs = [ex.submit(_compile, nvcc, s, o, extra + d) for s, o, d in jobs]
            for f in cf.as_completed(futs):
                src, rc, log = f.result()
                if verbose or rc != 0:
                    sys.stderr.write(log)
                if rc != 0:
                    raise RuntimeError(f"nvcc failed on {os.path.basename(src)}")
    if force or jobs or _stale(LIB, objs):
        # --no-undefined: a symbol missing from every object fails the link, not the first dlopen
        cmd = [nvcc, *ARCH, "-shared", "-cudart", "static", "-Xlinker", "--no-undefined", "-o", LIB, *objs]
        p = subprocess.run(cmd, capture_output=True, text=True)
        if p.returncode != 0:
            sys.stderr.write(p.stdout + p.stderr)
            raise RuntimeError("linking libspnngp_gb300.so failed")
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="--force" in sys.argv))
