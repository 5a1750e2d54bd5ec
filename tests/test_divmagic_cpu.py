"""The magic-number remainder (csrc/divmagic.h) used by the affine pattern fetcher in place of
`n % d`: built for the host and checked against `%` on edge and random dividends and divisors."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def test_magic_remainder_matches_modulo(tmp_path):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("g++ is not available")
    exe = str(tmp_path / "divmagic_check")
    res = subprocess.run([cxx, "-O2", "-std=c++17", "-I", os.path.join(ROOT, "blend2d_gb300", "csrc"),
                          os.path.join(HERE, "native", "divmagic_check.cpp"), "-o", exe], capture_output=True, text=True)
    assert res.returncode == 0, res.stderr
    run = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert run.returncode == 0, run.stdout + run.stderr
    assert " 0 mismatches" in run.stdout
