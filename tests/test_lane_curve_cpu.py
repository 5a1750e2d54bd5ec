"""The lane-stepped curve flattener of the device edge builder (eb::LaneCurve in edge_build.cuh,
used by edge_curves_kernel) against its loop form (eb::curve_to, the restatement of the
reference's curve_to / flatten_unsafe): both compiled for the host from the same header, same
segments in the same order for random cubic, quadratic and conic curves across the clip box."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


@pytest.fixture(scope="module")
def checker(tmp_path_factory):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("g++ is not available")
    cuda_inc = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "include")
    exe = str(tmp_path_factory.mktemp("lane") / "lane_curve_check")
    cmd = [cxx, "-O2", "-std=c++17", "-ffp-contract=off", "-I", os.path.join(ROOT, "blend2d_gb300", "csrc"),
           "-I", cuda_inc, os.path.join(HERE, "native", "lane_curve_check.cpp"), "-o", exe]
    res = subprocess.run(cmd, capture_output=True, text=True)
    assert res.returncode == 0, res.stderr
    return exe


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_lane_curve_matches_loop_flattener(checker, seed):
    res = subprocess.run([checker, str(seed), "60000"], capture_output=True, text=True, timeout=300)
    assert res.returncode == 0, res.stdout + res.stderr
    assert "mismatches 0" in res.stdout
