"""Builds libcfcull.so (the CUDA kernels + C ABI) in-tree with nvcc for sm_103a.

    python -m hellovulkan_gb300.build [--force]

Every translation unit is compiled in parallel with
``-gencode arch=compute_103a,code=sm_103a -lineinfo -O3 -fmad=false`` and the
host compiler flag ``-ffp-contract=off`` (the kernels' float arithmetic is
pinned; see include/cf_pinned_math.h), then linked into
``hellovulkan_gb300/libcfcull.so`` with the CUDA runtime linked statically.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
REPO = PKG.parent
CSRC = PKG / "csrc"
OBJ_DIR = PKG / "_build"
LIB = PKG / "libcfcull.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = [
    *ARCH, "-lineinfo", "-O3", "-std=c++20", "-fmad=false", "-prec-div=true", "-prec-sqrt=true", "-ftz=false",
    "-Xcompiler", "-fPIC,-fvisibility=hidden,-ffp-contract=off,-O2",
    "-I", str(REPO / "include"), "-I", str(CSRC),
]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found (set NVCC or put /usr/local/cuda/bin on PATH)")


def _sources():
    return sorted(list(CSRC.glob("*.cu")) + list(CSRC.glob("*.cpp")))


def _headers():
    return list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.h")) + list((REPO / "include").glob("*.h"))


def _newest(paths) -> float:
    return max((p.stat().st_mtime for p in paths), default=0.0)


def _compile(src: Path, obj: Path) -> None:
    cmd = [nvcc(), *NVCC_FLAGS, "-c", str(src), "-o", str(obj)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s%s" % (src.name, r.stdout, r.stderr))


def build(force: bool = False, verbose: bool = False) -> Path:
    srcs = _sources()
    hdr_time = _newest(_headers())
    OBJ_DIR.mkdir(parents=True, exist_ok=True)
    jobs = []
    for s in srcs:
        o = OBJ_DIR / (s.name + ".o")
        if force or not o.exists() or o.stat().st_mtime < max(s.stat().st_mtime, hdr_time, Path(__file__).stat().st_mtime):
            jobs.append((s, o))
    if jobs:
        with ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            list(ex.map(lambda j: _compile(*j), jobs))
    objs = [OBJ_DIR / (s.name + ".o") for s in srcs]
    if force or jobs or not LIB.exists() or LIB.stat().st_mtime < _newest(objs):
        tmp = LIB.with_suffix(".so.tmp%d" % os.getpid())
        cmd = [nvcc(), *ARCH, "-shared", "-cudart", "static", "-o", str(tmp), *map(str, objs)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n%s%s" % (r.stdout, r.stderr))
        os.replace(tmp, LIB)
    if verbose:
        print(LIB)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
