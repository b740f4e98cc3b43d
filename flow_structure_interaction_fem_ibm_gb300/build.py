"""In-tree build of the native libraries.

* ``_build/libfsi_mg.so``   -- the CUDA solver (sm_103a) and its C ABI
  (include/fsi_mg.h), compiled with nvcc.
* ``_build/libfsi_geom.so`` -- host geometry (icosphere, iblank, ghost list,
  image-point coefficients), compiled with g++.

Both are plain shared libraries loaded with ctypes; nothing here depends on
PyTorch.  Translation units compile in parallel.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
OUT = PKG / "_build"
INCLUDE = ROOT / "include"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

CUDA_SOURCES = ["fsi_mg.cu", "step_api.cu", "mg_kernels.cu", "step_kernels.cu"]
CUDA_HEADERS = ["mg_kernels.cuh", "device_util.cuh", "partition_solve.cuh", "mg_context.h"]


def nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return cand


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        sys.stderr.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
        raise RuntimeError(f"build step failed: {cmd[0]} {cmd[-1]}")
    return r


def _stale(target: Path, deps) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(Path(d).stat().st_mtime > t for d in deps if Path(d).exists())


def build_geometry(force: bool = False) -> Path:
    OUT.mkdir(exist_ok=True)
    src = CSRC / "geometry.cpp"
    lib = OUT / "libfsi_geom.so"
    if force or _stale(lib, [src]):
        tmp = lib.with_suffix(f".so.tmp{os.getpid()}")
        _run(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-pthread",
              "-o", str(tmp), str(src)])
        os.replace(tmp, lib)
    return lib


def build_solver(force: bool = False, extra_flags=None) -> Path:
    OUT.mkdir(exist_ok=True)
    lib = OUT / "libfsi_mg.so"
    srcs = [CSRC / s for s in CUDA_SOURCES]
    deps = srcs + [CSRC / h for h in CUDA_HEADERS] + [INCLUDE / "fsi_mg.h"]
    if not (force or _stale(lib, deps)):
        return lib
    flags = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-I", str(INCLUDE),
             "-I", str(CSRC), "--expt-relaxed-constexpr"] + ARCH + list(extra_flags or [])
    objs = []

    def compile_one(src: Path):
        obj = OUT / (src.stem + ".o")
        _run([nvcc(), "-c", *flags, "-o", str(obj), str(src)])
        return obj

    with ThreadPoolExecutor(max_workers=len(srcs)) as ex:
        objs = list(ex.map(compile_one, srcs))
    tmp = lib.with_suffix(f".so.tmp{os.getpid()}")
    _run([nvcc(), "-shared", *ARCH, "-o", str(tmp), *[str(o) for o in objs], "-lcudart"])
    os.replace(tmp, lib)
    return lib


def build_all(force: bool = False):
    with ThreadPoolExecutor(max_workers=2) as ex:
        g = ex.submit(build_geometry, force)
        s = ex.submit(build_solver, force)
        return g.result(), s.result()


if __name__ == "__main__":
    print(build_all(force="--force" in sys.argv))
