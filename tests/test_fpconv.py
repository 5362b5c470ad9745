"""The kernels' integer-pipe FP32 <-> FP64 conversions (k_fpconv.cuh, built
for the host) against the CPU's own conversions, bit for bit
(tests/cpp/fpconv_check.cpp)."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_conversions_match_the_cpu(tmp_path):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no g++")
    exe = str(tmp_path / "fpconv_check")
    subprocess.run([cxx, "-std=c++17", "-O2", "-fno-fast-math",
                    os.path.join(ROOT, "tests", "cpp", "fpconv_check.cpp"), "-o", exe], check=True)
    r = subprocess.run([exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert int(r.stdout.split()[0]) > 1000000
