"""Build libndtensors_gb300.so for sm_103a (GB300) with nvcc.

Each translation unit is compiled in parallel, then linked into a shared
library placed next to the Python bindings (``ndtensors_gb300/``).  Usage:

    python itensors.jl_gb300/build.py [--force] [--debug]
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
CSRC = HERE / "csrc"
OUT = HERE / "ndtensors_gb300" / "libndtensors_gb300.so"
BUILD = HERE / "_build"
SOURCES = ["nd_api.cu", "nd_permute.cu", "nd_plan.cu", "nd_contract.cu", "nd_gemm_f64.cu",
           "nd_ozaki.cu", "nd_linalg.cu", "nd_noalloc.cu", "nd_vector.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if c and (os.path.sep not in c or os.path.exists(c)):
            return c
    return "nvcc"


def _needs_build(force: bool) -> bool:
    if force or not OUT.exists():
        return True
    t = OUT.stat().st_mtime
    deps = [CSRC / s for s in SOURCES] + list(CSRC.glob("*.h")) + [HERE.parent / "include" / "ndtensors_gb300.h"]
    return any(p.stat().st_mtime > t for p in deps if p.exists())


def build(force: bool = False, debug: bool = False, verbose: bool = False) -> Path:
    if not _needs_build(force):
        return OUT
    BUILD.mkdir(exist_ok=True)
    nvcc = _nvcc()
    flags = ARCH + ["-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-O3"]
    if debug:
        flags += ["-DND_DEBUG=1"]

    def one(src):
        obj = BUILD / (Path(src).stem + ".o")
        cmd = [nvcc, *flags, "-c", str(CSRC / src), "-o", str(obj)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stderr}")
        if verbose and r.stderr:
            print(r.stderr, file=sys.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=min(len(SOURCES), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(one, SOURCES))
    tmp = OUT.with_suffix(".so.tmp")
    cmd = [nvcc, *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr}")
    os.replace(tmp, OUT)
    return OUT


if __name__ == "__main__":
    p = build(force="--force" in sys.argv, debug="--debug" in sys.argv, verbose="-v" in sys.argv)
    print(p)
