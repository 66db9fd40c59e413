"""Static resource rules of the tensor-core kernels for every supported (W, T0), checked
on the host (tests/layout_check.cu, compiled by nvcc without a GPU): shared memory within
the 227 KB a CTA may use, 16-byte aligned regions, tensor-memory columns within 512, and
M-tile / row mappings that cover the padded tile."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _nvcc():
    cand = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    return cand if os.path.exists(cand) else shutil.which("nvcc")


def test_tensor_core_kernel_layouts(tmp_path):
    nvcc = _nvcc()
    if nvcc is None:
        pytest.skip("nvcc not available")
    exe = tmp_path / "layout_check"
    subprocess.run([nvcc, "-std=c++17", "-O1", "-gencode", "arch=compute_103a,code=sm_103a",
                    "-I", os.path.join(ROOT, "cunfft_gb300", "csrc"), "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "layout_check.cu"), "-o", str(exe)], check=True, timeout=600)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "0 failures" in r.stdout
