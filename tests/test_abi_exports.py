"""CPU checks of the drop-in boundary: libblgpu.so builds, loads without a GPU, and exports
exactly the entry points include/blgpu.h declares (no compute calls are made here)."""
import ctypes
import os
import re
import subprocess

import pytest

import blend2d_gb300 as bg
from blend2d_gb300 import build as pkg_build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = []
    for fname in sorted(os.listdir(os.path.join(ROOT, "include"))):
        if not fname.endswith(".h"):
            continue
        text = open(os.path.join(ROOT, "include", fname)).read()
        names += re.findall(r"^\s*BLGpuResult\s+(blgpu_\w+)\s*\(", text, flags=re.M)
    return names


@pytest.fixture(scope="module")
def lib_path():
    return pkg_build.build()


def test_header_declares_entry_points():
    names = declared_functions()
    assert len(names) >= 30
    assert len(set(names)) == len(names)


def test_library_exports_every_declared_symbol(lib_path):
    lib = ctypes.CDLL(lib_path)
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_no_undeclared_exports(lib_path):
    out = subprocess.run(["nm", "-D", "--defined-only", lib_path], capture_output=True, text=True, check=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if " T " in line}
    assert exported == set(declared_functions())


def test_python_bindings_cover_the_abi(lib_path):
    assert set(bg._SIGNATURES) == set(declared_functions())
    lib = bg.load_library()
    for name in bg._SIGNATURES:
        assert getattr(lib, name).restype is ctypes.c_uint32


def test_struct_layouts_match_header(tmp_path):
    """The ctypes mirrors have the sizes a C compiler gives the header's structs."""
    structs = {"BLGpuRuntimeCreateInfo": bg.RuntimeCreateInfo, "BLGpuImage": bg.Image,
               "BLGpuGradientStop": bg.GradientStop, "BLGpuGradient": bg.Gradient, "BLGpuPattern": bg.Pattern,
               "BLGpuStats": bg.Stats, "BLGpuLaunchConfig": bg.LaunchConfig, "BLGpuMemoryInfo": bg.MemoryInfo,
               "BLGpuStrokeOptions": bg.StrokeOptions}
    src = tmp_path / "sizes.c"
    src.write_text('#include <stdio.h>\n#include "blgpu.h"\nint main(void) {\n' +
                   "".join(f'  printf("%zu\\n", sizeof({name}));\n' for name in structs) + "  return 0;\n}\n")
    exe = tmp_path / "sizes"
    subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    sizes = [int(x) for x in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()]
    for (name, cls), size in zip(structs.items(), sizes):
        assert ctypes.sizeof(cls) == size, name


def test_missing_library_fails_loudly(tmp_path):
    saved = bg._lib
    bg._lib = None
    try:
        with pytest.raises(RuntimeError, match="missing"):
            bg.load_library(str(tmp_path / "nope.so"))
    finally:
        bg._lib = saved
