"""Build of the engine's shared library, libneci_gpu.so, with nvcc for sm_103a.

The library is built in-tree (``neci_stable_gb300/_build/``) from the CUDA
sources under ``csrc/``: each translation unit is compiled in parallel, then
linked with ``-shared``.  FP64 kernels are compiled with ``--fmad=false`` so
that every a*b+c is two IEEE roundings, the operation order the CPU oracle
uses; the bit-exact parity tests depend on it.
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = BUILD / "libneci_gpu.so"
SOURCES = ["kernels.cu", "spawn_fp64.cu", "spawn_fp32.cu", "util_kernels.cu", "capi.cu", "noalloc.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "--fmad=false", "-std=c++17", "-Xcompiler", "-fPIC",
              "-Xcompiler", "-Wall", "--expt-relaxed-constexpr"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.sep not in cand or os.path.exists(cand)):
            return cand
    return "nvcc"


def _stale(target: Path, deps) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(Path(d).stat().st_mtime > t for d in deps)


def build(verbose: bool = False, force: bool = False) -> Path:
    """Compile csrc/*.cu into _build/libneci_gpu.so (incremental)."""
    BUILD.mkdir(exist_ok=True)
    headers = list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.h")) + [PKG.parent / "include" / "neci_gpu.h"]
    nvcc = _nvcc()
    jobs = []
    for src in SOURCES:
        obj = BUILD / (Path(src).stem + ".o")
        if force or _stale(obj, [CSRC / src] + headers):
            jobs.append([nvcc, *ARCH, *NVCC_FLAGS, "-c", str(CSRC / src), "-o", str(obj)])

    def run(cmd):
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed ({' '.join(cmd)}):\n{r.stdout}\n{r.stderr}")
        return r

    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        list(ex.map(run, jobs))
    objs = [BUILD / (Path(s).stem + ".o") for s in SOURCES]
    if force or jobs or _stale(LIB, objs):
        run([nvcc, *ARCH, "-shared", "-o", str(LIB), *map(str, objs)])
    return LIB


if __name__ == "__main__":
    print(build(verbose=True, force="--force" in sys.argv))
