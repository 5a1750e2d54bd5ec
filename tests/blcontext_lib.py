"""Builds and runs the BLContext binding check (tests/native/blcontext_check.cpp), which links the
binding (blend2d_gb300/blcontext), the reference library built from its staged sources
(oracle/ref.mk) and libblgpu.so. Test infrastructure only."""
from __future__ import annotations

import json
import os
import platform
import subprocess

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
STAGED = os.path.join(ROOT, "baseline", "_ref", "blend2d-src")
FONT = os.path.join(ROOT, "baseline", "_ref", "fonts", "ABeeZee-Regular.ttf")
X86 = platform.machine() in ("x86_64", "AMD64")
VARIANT = "default" if X86 else "native"
# the LUT builder of that reference build (blend2d/pixelops/funcs.cpp:22-34): SSE2 on x86-64 no-JIT
# builds, the portable one elsewhere (BLGPU_LUT_SSE2 = 0, BLGPU_LUT_SCALAR = 2)
LUT = 0 if X86 else 2


def available() -> bool:
    return os.path.isfile(os.path.join(STAGED, "blend2d", "blend2d.h"))


def harness() -> str:
    from blend2d_gb300 import build as pkg_build
    pkg_build.build()
    subprocess.run(["make", "-s", "-j", str(max(2, os.cpu_count() or 2)), "-f", os.path.join(ROOT, "oracle", "ref.mk"),
                    f"VARIANT={VARIANT}", "blcontext"], check=True, cwd=ROOT)
    return os.path.join(ROOT, "oracle", "_ref", f"b2d_blcontext_{VARIANT}")


def run(*args: str, timeout: float = 600):
    res = subprocess.run([harness(), *args], capture_output=True, text=True, timeout=timeout)
    lines = res.stdout.strip().splitlines()
    return res.returncode, (json.loads(lines[-1]) if lines else None), res.stderr
