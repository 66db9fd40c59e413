"""The C-ABI library loads and exports every symbol its headers declare (no GPU needed)."""
import ctypes
import os
import re
import subprocess

import pytest

from cunfft_gb300 import _native as nat

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INCLUDE = os.path.join(ROOT, "include")


def _declared(header):
    src = open(os.path.join(INCLUDE, header)).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    src = re.sub(r"#define(?:[^\n]*\\\n)*[^\n]*", "", src)
    names = re.findall(r"\b([A-Za-z_][A-Za-z0-9_]*)\s*\([^;{]*\)\s*;", src)
    return sorted(set(n for n in names if n not in ("if", "while", "for", "sizeof", "return")))


@pytest.fixture(scope="module")
def library():
    if not os.path.exists(nat.LIB_PATH):
        from cunfft_gb300.build import build
        build()
    return nat.lib()


@pytest.mark.parametrize("header", ["cunfft.h", "cunfft_x.h", "cunfft_util.h"])
def test_every_declared_symbol_is_exported(library, header):
    declared = _declared(header)
    assert declared, header
    missing = [n for n in declared if not hasattr(library, n)]
    assert not missing, f"{header}: not exported: {missing}"


def test_symbol_lists_cover_headers():
    declared = set(_declared("cunfft.h")) | set(_declared("cunfft_x.h")) | set(_declared("cunfft_util.h"))
    listed = set(nat.ABI_SYMBOLS) | set(nat.X_SYMBOLS) | set(nat.UTIL_SYMBOLS)
    assert declared == listed, (declared - listed, listed - declared)


def test_reference_entry_points_present(library):
    # every function of the reference's src/cunfft.h except nfft_def_fg_exp_l,
    # which the reference declares (src/cunfft.h:234) but never defines
    ref = ["warmUp_createPlan", "copyDataToDevice", "copyDataToDeviceAd", "copyDataToHost", "copyDataToHostAd",
           "copy_f_hat_ToHost", "copy_f_ToHost", "copy_g_ToHost", "copy_x_toHost", "cunfft_transform",
           "cunfft_adjoint", "cunfft_initPlan", "cunfft_freePlan", "cunfft_initDevicePara", "cunfft_init",
           "cunfft_initGuru", "cunfft_initHelp", "cunfft_reinit", "cunfft_reinitAd", "cunfft_finalize",
           "cunfft_finalizeDevice", "resetCUNFFTTimes", "cundft_transform", "cundft_adjoint",
           "nfft_init_fg_exp_l", "setProperties", "resetDevice"]
    for name in ref:
        assert hasattr(library, name), name


def test_plan_struct_layout_matches_header():
    """Compile a probe against include/cunfft_typedefs.h and compare offsets with the ctypes mirror."""
    probe = r"""
#include <stdio.h>
#include <stddef.h>
#include "cunfft_typedefs.h"
#define P(f) printf(#f " %zu\n", offsetof(cunfft_plan, f));
int main(void){ P(N_total) P(M_total) P(d) P(N) P(x) P(f_hat) P(f) P(sigma) P(n) P(n_total) P(m) P(b) P(g)
P(g_hat) P(fg_exp_l_cpu) P(g_gpu) P(fhat_gpu) P(x_gpu) P(f_gpu) P(fft_forward) P(fft_backward) P(CUNFFTTimes)
P(flags) printf("size %zu\n", sizeof(cunfft_plan)); printf("kdata %zu\n", sizeof(kdata)); return 0; }
"""
    import tempfile
    cuda_inc = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "include")
    if not os.path.isdir(cuda_inc):
        pytest.skip("CUDA headers not found")
    with tempfile.TemporaryDirectory() as td:
        src = os.path.join(td, "probe.c")
        exe = os.path.join(td, "probe")
        open(src, "w").write(probe)
        subprocess.run(["gcc", "-I", INCLUDE, "-I", cuda_inc, src, "-o", exe], check=True)
        out = subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split("\n")
    got = dict(line.split() for line in out if line.strip())
    for name, _ in nat.CunfftPlan._fields_:
        assert int(got[name]) == getattr(nat.CunfftPlan, name).offset, name
    assert int(got["size"]) == ctypes.sizeof(nat.CunfftPlan)
    assert int(got["kdata"]) == ctypes.sizeof(nat.KData)


def test_status_strings(library):
    assert library.cunfft_x_status_string(0) == b"success"
    assert library.cunfft_x_status_string(5) == b"nodes not set"
    assert b"sm_103a" in library.cunfft_x_version()


def test_host_only_helpers(library):
    """Entry points that run without a device."""
    import numpy as np
    out = np.zeros(14)
    library.nfft_init_fg_exp_l(out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), 2.5, 0)
    assert np.allclose(out, np.exp(-np.arange(14) ** 2 / 2.5), rtol=1e-13)
    assert library.next_power_of_2(100) == 128
    k = nat.KData()
    N = (ctypes.c_ssize_t * 2)(64, 32)
    n = (ctypes.c_ssize_t * 2)(128, 64)
    b = (ctypes.c_double * 2)(2.5, 2.5)
    s = (ctypes.c_double * 2)(2.0, 2.0)
    library.setProperties(N, n, b, s, 2, ctypes.byref(k))
    assert k.n[1] == 64 and abs(k.fac[0] - np.pi ** 2 * 2.5 / 128 ** 2) < 1e-15
    assert library.cunfft_x_set_default_cutoff(0) == nat.INVALID_ARGUMENT
    assert library.cunfft_x_set_default_cutoff(16) == nat.INVALID_ARGUMENT
    assert library.cunfft_x_set_default_cutoff(6) == nat.SUCCESS
