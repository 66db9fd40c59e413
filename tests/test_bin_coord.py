"""The binning's integer form of the node-to-grid reduction (cunfft_gb300/csrc/bin_coord.h),
checked on the CPU against the reference's FP64 rule u = llrint(n x) - signbit(x) - m,
c = n x - u (src/cunfft_kernel.cu:175-182): 2.4M coordinates on n = 2^1 .. 2^24,
including exact grid points, exact ties and their neighbours; window starts exact,
FP32 fractions to one FP32 ulp plus 2^-49."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_integer_coordinate_form_matches_fp64_rule(tmp_path):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("g++ not available")
    exe = tmp_path / "bin_coord_check"
    src = os.path.join(ROOT, "tests", "bin_coord_check.cpp")
    subprocess.run([cxx, "-O2", "-std=c++17", "-I", os.path.join(ROOT, "cunfft_gb300", "csrc"), src, "-o", str(exe)],
                   check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "u_mismatch 0" in r.stdout and "frac_beyond_tol 0" in r.stdout
