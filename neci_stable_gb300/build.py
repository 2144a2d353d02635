"""Build of the engine's shared library, libneci_gpu.so, with nvcc for sm_103a.

The library is built in-tree (``neci_stable_gb300/_build/``) from the CUDA
sources under ``csrc/``: each translation unit is compiled in parallel, then
linked with ``-shared``.  Translation units with FP64 (or compensated FP32)
sums are compiled with ``--fmad=false`` so that every a*b+c is two IEEE
roundings, the operation order the CPU oracle uses; the bit-exact parity tests
depend on it.  The FP32 spawn kernels (``spawn_fp32.cu``) keep FMA
contraction: their amplitudes and table products are chains of multiplies,
and the only a*b+c forms there are float estimates that integer loops correct
exactly, so contraction changes no result.
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
SOURCES = ["kernels.cu", "spawn_fp64.cu", "spawn_fp32.cu", "util_kernels.cu", "sort_kernels.cu", "capi.cu", "noalloc.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
              "-Xcompiler", "-Wall", "--expt-relaxed-constexpr"]
# translation units compiled with FMA contraction (see the module docstring)
FMAD_SOURCES = {"spawn_fp32.cu"}


def _fmad(src: str) -> list:
    return ["--fmad=true"] if src in FMAD_SOURCES else ["--fmad=false"]


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
    # the objects depend on the headers and on the flags set here
    headers = (list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.h")) + [PKG.parent / "include" / "neci_gpu.h"] +
               [Path(__file__).resolve()])
    nvcc = _nvcc()
    jobs = []
    for src in SOURCES:
        obj = BUILD / (Path(src).stem + ".o")
        if force or _stale(obj, [CSRC / src] + headers):
            jobs.append([nvcc, *ARCH, *NVCC_FLAGS, *_fmad(src), "-c", str(CSRC / src), "-o", str(obj)])

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
        # -z defs: a symbol that no object defines fails the link, not the load
        run([nvcc, *ARCH, "-shared", "-Xlinker", "-z,defs", "-o", str(LIB), *map(str, objs)])
    return LIB


if __name__ == "__main__":
    print(build(verbose=True, force="--force" in sys.argv))
