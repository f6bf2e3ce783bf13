"""Build recipe of the C oracle ``oracle/_build/libesnufft.so`` (gcc + OpenMP).

``esnufft.c`` is compiled twice, as double (``es_*_d``, the checker) and as
float (``es_*_f``, the timed CPU baseline), and linked into one library.
Portable flags only (the same recipe builds on x86_64 and aarch64).
"""

from __future__ import annotations

import os
import shutil
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
SRC = HERE / "esnufft.c"
OUT = HERE / "_build"
LIB = OUT / "libesnufft.so"


def build(force: bool = False) -> Path:
    if not force and LIB.exists() and LIB.stat().st_mtime >= SRC.stat().st_mtime:
        return LIB
    cc = os.environ.get("CC") or shutil.which("gcc") or "cc"
    OUT.mkdir(exist_ok=True)
    objs = []
    for real, suffix in (("double", "_d"), ("float", "_f")):
        obj = OUT / f"esnufft{suffix}.o"
        cmd = [cc, "-O3", "-fopenmp", "-fPIC", "-std=c11", f"-DREAL={real}", f"-DSUFFIX={suffix}",
               "-D_DEFAULT_SOURCE", "-c", str(SRC), "-o", str(obj)]
        if real == "float":
            cmd.insert(-4, "-DREAL_IS_FLOAT")
        subprocess.run(cmd, check=True)
        objs.append(str(obj))
    tmp = LIB.with_suffix(".so.tmp")
    subprocess.run([cc, "-shared", "-fopenmp", "-o", str(tmp), *objs, "-lm"], check=True)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
