"""Build libphono_gpu.so in-tree with nvcc for sm_103a.

The library is a plain C-ABI shared object (include/phono.h); the CUDA
runtime is linked statically so the object loads without a toolkit on the
loader path.  Objects are compiled in parallel and relinked only when a
source is newer than the library.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = BUILD / "libphono_gpu.so"
SOURCES = ["fdtd_step.cu", "energy.cu", "lattice.cu", "api.cu"]
HEADERS = ["fdtd_common.cuh", "div_table.cuh", "tile_rows.cuh"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# No implicit FMA anywhere: device code uses explicit _rn intrinsics for the
# arithmetic whose rounding must match the reference, and the host code that
# derives coefficients (api.cu) must round each operation like NumPy does; GCC
# contracts a*b+c by default on aarch64, so -ffp-contract=off is required there.
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "--fmad=false", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
         "-Xcompiler", "-ffp-contract=off"]


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libphono_gpu.so")


def _stale(target: Path, deps) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(Path(d).stat().st_mtime > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> Path:
    BUILD.mkdir(exist_ok=True)
    cc = nvcc()
    hdrs = [CSRC / h for h in HEADERS] + [ROOT / "include" / "phono.h"]
    procs = []
    objs = []
    for src in SOURCES:
        obj = BUILD / (Path(src).stem + ".o")
        objs.append(obj)
        if force or _stale(obj, [CSRC / src] + hdrs):
            cmd = [cc, *ARCH, *FLAGS, "-I", str(ROOT / "include"), "-c", str(CSRC / src), "-o", str(obj) + ".tmp"]
            if verbose:
                print(" ".join(cmd), file=sys.stderr)
            procs.append((obj, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
    errors = []
    for obj, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            errors.append(out.decode(errors="replace"))
        else:
            os.replace(str(obj) + ".tmp", obj)
    if errors:
        raise RuntimeError("nvcc failed:\n" + "\n".join(errors))
    if force or procs or _stale(LIB, objs):
        cmd = [cc, *ARCH, "-shared", "-o", str(LIB) + ".tmp", *map(str, objs)]
        subprocess.run(cmd, check=True, capture_output=not verbose)
        os.replace(str(LIB) + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
