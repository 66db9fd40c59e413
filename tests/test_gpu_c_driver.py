"""A C program linked against libcunfft.so through the drop-in headers reproduces the
reference's logged known answers.

tests/c_driver/simple_test.c drives the plan API the way the reference's test driver
does (Tests/Scripts/simpleTest.cpp:62-177 forward, :179-260 adjoint): a fresh plan per
repetition, drand48 example data, cundft, reinit, cunfft, copies, E_inf.  This test
compiles it with gcc against include/ (no Python or ctypes in between), links -lcunfft,
runs ten repetitions in one process as the logged runs did, and compares the tenth
repetition's E_inf with the value the reference logged (within 1e-3 relative, the bar of
the ctypes known-answer tests).
"""
import json
import os
import re
import shutil
import subprocess

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
KATS = json.load(open(os.path.join(ROOT, "tests", "golden", "kats.json")))["kats"]


@pytest.fixture(scope="module")
def driver(tmp_path_factory):
    from cunfft_gb300 import _native

    _native.lib()  # builds libcunfft.so when needed
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    pkg = os.path.join(ROOT, "cunfft_gb300")
    exe = str(tmp_path_factory.mktemp("c_driver") / "simple_test")
    cc = shutil.which("gcc") or "cc"
    cmd = [cc, "-O2", "-Wall", "-I", os.path.join(ROOT, "include"), "-I", os.path.join(cuda, "include"),
           os.path.join(ROOT, "tests", "c_driver", "simple_test.c"), "-L", pkg, "-lcunfft",
           f"-Wl,-rpath,{pkg}", f"-Wl,-rpath,{os.path.join(cuda, 'lib64')}", "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def _kat(direction, N):
    for k in KATS:
        if k["direction"] == direction and k["m"] == 6 and k["N"] == N and k["skip_generations"] == 9:
            return k
    pytest.skip(f"no logged known answer for {direction} N={N}")


@pytest.mark.parametrize("direction,N", [("forward", [64, 64]), ("adjoint", [64, 64]), ("forward", [4096]),
                                         ("forward", [16, 16, 16])])
def test_c_driver_reproduces_logged_e_inf(driver, direction, N):
    k = _kat(direction, N)
    args = [driver, "fwd" if direction == "forward" else "adj", "10", str(len(N))] + [str(v) for v in N]
    r = subprocess.run(args, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    rows = [re.match(r"rep (\d+) e_inf (\S+) status (\d+)", ln) for ln in r.stdout.splitlines()]
    rows = [m for m in rows if m]
    assert len(rows) == 10 and all(m.group(3) == "0" for m in rows), r.stdout
    e10 = float(rows[-1].group(2))
    assert abs(e10 - k["e_inf"]) <= 1e-3 * k["e_inf"], (e10, k["e_inf"], k["file"], k["line"])
