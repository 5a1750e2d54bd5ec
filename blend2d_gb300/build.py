"""Builds libblgpu.so (the sm_103a raster backend and its C ABI) in-tree.

    python -m blend2d_gb300.build [--jobs N] [--force]

Translation units compile in parallel; the library links CUDA's runtime statically so it only
needs the driver at load time. Device code is built with -fmad=false and host code with
-ffp-contract=off: the reference evaluates every a*b+c unfused, and bit-exact results depend on
doing the same.
"""
from __future__ import annotations

import argparse
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(BUILD, "libblgpu.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CUDA_SOURCES = ["kernels.cu", "noalloc.cu", "stroke.cu"]
HOST_SOURCES = ["frontend.cpp", "runtime.cpp", "context.cpp", "stroke.cpp"]


def nvcc() -> str:
    path = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(path):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libblgpu.so")
    return path


def _includes() -> list[str]:
    return ["-I", CSRC, "-I", os.path.join(ROOT, "include")]


def _compile(src: str) -> str:
    obj = os.path.join(BUILD, os.path.basename(src) + ".o")
    path = os.path.join(CSRC, src)
    if src.endswith(".cu"):
        cmd = [nvcc(), *ARCH, "-lineinfo", "-O3", "-std=c++17", "-fmad=false", "-Xptxas", "-v",
               "-Xcompiler", "-fPIC,-ffp-contract=off,-fvisibility=hidden", *_includes(), "-c", path, "-o", obj]
    else:
        cmd = [nvcc(), "-O2", "-std=c++17", "-x", "c++",
               "-Xcompiler", "-fPIC,-ffp-contract=off,-fno-fast-math,-fvisibility=hidden,-Wall",
               *_includes(), "-c", path, "-o", obj]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{res.stdout}\n{res.stderr}")
    with open(obj + ".log", "w") as f:
        f.write(res.stdout + res.stderr)
    return obj


def _stale() -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    deps += [os.path.join(ROOT, "include", f) for f in os.listdir(os.path.join(ROOT, "include"))]
    deps.append(os.path.abspath(__file__))
    return any(os.path.getmtime(d) > t for d in deps)


def _object_stale(src: str) -> bool:
    """A translation unit is recompiled when its object is older than it, than any header of the
    package or of include/, or than this script."""
    obj = os.path.join(BUILD, os.path.basename(src) + ".o")
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    deps = [os.path.join(CSRC, src), os.path.abspath(__file__)]
    deps += [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    deps += [os.path.join(ROOT, "include", f) for f in os.listdir(os.path.join(ROOT, "include"))]
    return any(os.path.getmtime(d) > t for d in deps)


def build(jobs: int | None = None, force: bool = False) -> str:
    """Compiles the translation units that changed and links libblgpu.so; returns its path."""
    if not force and not _stale():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    sources = CUDA_SOURCES + HOST_SOURCES
    todo = [src for src in sources if force or _object_stale(src)]
    with ThreadPoolExecutor(max_workers=jobs or max(1, len(todo))) as ex:
        list(ex.map(_compile, todo))
    objs = [os.path.join(BUILD, os.path.basename(src) + ".o") for src in sources]
    tmp = LIB + ".tmp"
    cmd = [nvcc(), *ARCH, "-shared", "-cudart", "static", "-o", tmp, *objs,
           "-Xlinker", "--no-undefined", "-lpthread", "-ldl", "-lrt"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"link failed: {' '.join(cmd)}\n{res.stdout}\n{res.stderr}")
    os.replace(tmp, LIB)
    return LIB


def main(argv=None) -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--jobs", type=int, default=None)
    ap.add_argument("--force", action="store_true")
    args = ap.parse_args(argv)
    print(build(args.jobs, args.force))
    return 0


if __name__ == "__main__":
    sys.exit(main())
