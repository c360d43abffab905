"""In-tree build of the engine library (libfastpart.so) for sm_103a.

Every translation unit is compiled in parallel with one ``-gencode`` and linked
into ``fastpartitioner_gb300/libfastpart.so``.  Host C++ is compiled without
floating-point contraction: the streaming partitioners evaluate the LDG score in
double precision and must round exactly like the reference's build.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = PKG / "libfastpart.so"
INCLUDE = PKG.parent / "include"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build fastpartitioner_gb300")


def _sources():
    return sorted(CSRC.glob("*.cu")) + sorted(CSRC.glob("*.cpp"))


def _defines() -> list:
    """FP_TIMING_STATS=1 in the environment builds the per-warp / per-CTA timing
    statistics of the refinement kernels (diagnostics; atomics in hot loops)."""
    return ["-DFP_TIMING_STATS"] if os.environ.get("FP_TIMING_STATS") == "1" else []


def _compile(src: Path, nvcc: str) -> Path:
    obj = BUILD / (src.name + ".o")
    common = ["-O3", "-std=c++17", "-I", str(INCLUDE), *_defines(), "-Xcompiler", "-fPIC,-ffp-contract=off"]
    if src.suffix == ".cu":
        cmd = [nvcc, *ARCH, "-lineinfo", *common, "-c", str(src), "-o", str(obj)]
    else:
        cmd = [nvcc, *common, "-x", "c++", "-c", str(src), "-o", str(obj)]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{res.stdout}\n{res.stderr}")
    return obj


def _stale() -> bool:
    if not LIB.exists():
        return True
    stamp = BUILD / "defines.txt"
    if (stamp.read_text() if stamp.exists() else "") != " ".join(_defines()):
        return True
    t = LIB.stat().st_mtime
    deps = _sources() + list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + list(INCLUDE.glob("*.h"))
    return any(p.stat().st_mtime > t for p in deps)


def build(force: bool = False, verbose: bool = False) -> Path:
    """Compiles the library if any source is newer than it; returns its path."""
    if not force and not _stale():
        return LIB
    nvcc = _nvcc()
    BUILD.mkdir(exist_ok=True)
    srcs = _sources()
    with cf.ThreadPoolExecutor(max_workers=min(len(srcs), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(lambda s: _compile(s, nvcc), srcs))
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [nvcc, *ARCH, "-shared", "-o", str(tmp), *map(str, objs)]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"link failed: {' '.join(cmd)}\n{res.stdout}\n{res.stderr}")
    os.replace(tmp, LIB)
    (BUILD / "defines.txt").write_text(" ".join(_defines()))
    if verbose:
        print(f"built {LIB}", file=sys.stderr)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
