"""Build recipe of ``libgbnufft.so`` (the CUDA kernels plus the C ABI).

Each translation unit under ``csrc/`` is compiled for sm_103a by ``nvcc``
in parallel, then linked into ``_build/libgbnufft.so`` against cuFFT and the
shared CUDA runtime.  Objects are rebuilt only when a source or header is
newer than the library.
"""

from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
INCLUDE = PKG.parent / "include"
BUILD = PKG / "_build"
LIB = BUILD / "libgbnufft.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr"]


def nvcc_path() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the GB300 NUFFT library needs the CUDA toolkit")


def _sources():
    return sorted(CSRC.glob("*.cu"))


def _deps():
    return sorted(CSRC.glob("*.cu")) + sorted(CSRC.glob("*.cuh")) + sorted(INCLUDE.glob("*.h"))


def is_stale() -> bool:
    if not LIB.exists():
        return True
    t = LIB.stat().st_mtime
    return any(p.stat().st_mtime > t for p in _deps())


def build(force: bool = False, verbose: bool = False, jobs: int | None = None) -> Path:
    """Compile the library if needed and return its path."""
    if not force and not is_stale():
        return LIB
    nvcc = nvcc_path()
    BUILD.mkdir(parents=True, exist_ok=True)
    srcs = _sources()
    objs = [BUILD / (s.stem + ".o") for s in srcs]

    def compile_one(pair):
        src, obj = pair
        cmd = [nvcc, *ARCH, *NVCC_FLAGS, f"-I{INCLUDE}", f"-I{CSRC}", "-c", str(src), "-o", str(obj)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src.name}:\n{r.stderr}")
        if verbose and r.stderr:
            print(r.stderr)
        return obj

    jobs = jobs or max(1, min(len(srcs), os.cpu_count() or 1))
    with ThreadPoolExecutor(jobs) as ex:
        list(ex.map(compile_one, zip(srcs, objs)))
    tmp = LIB.with_suffix(".so.tmp")
    cuda_lib = Path(nvcc).resolve().parent.parent / "lib64"
    cmd = [nvcc, *ARCH, "-shared", "-cudart", "shared", "-o", str(tmp), *map(str, objs),
           "-lcufft", "-Xlinker", "-rpath", "-Xlinker", str(cuda_lib)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True, verbose=True))
