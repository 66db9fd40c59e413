"""Error paths of the runtime, driven by host-side fault injection.

The reference exits the process on a failed CUDA call (cudaVerify under DEBUG,
src/cunfft_util.h:373-385) and ignores the error otherwise; here every failure becomes
a recorded status.  These tests make a device allocation or a cuFFT plan creation fail
on the host (CUNFFT_X_FAULT_ALLOC=k / CUNFFT_X_FAULT_CUFFT=k: the k-th such call of the
process reports out-of-memory / a cuFFT error without touching the device) and check
that the call returns the status, that nothing crashes, and that the next plan in the
same process still computes correct results.  No GPU fault is involved.  Each case runs
in a child process, since the fault counters are per process.
"""
import json
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CHILD = r"""
import json, sys
import numpy as np
import torch
sys.path.insert(0, ROOT)
import oracle as O
from cunfft_gb300 import _native as nat
from cunfft_gb300.nfft import NFFT

dev = torch.device("cuda:0")
rng = np.random.default_rng(9)
N, M = [16, 16, 16], 3000
x = rng.uniform(-0.5, 0.5, (M, 3))
fh = rng.uniform(-1, 1, N) + 1j * rng.uniform(-1, 1, N)
f = rng.uniform(-1, 1, M) + 1j * rng.uniform(-1, 1, M)
xt = torch.from_numpy(x).to(dev)

def run():
    p = NFFT(N, precision="f32", device=dev)
    try:
        p.set_nodes(xt)
        a = p.forward(torch.from_numpy(fh).to(dev)).cpu().numpy()
        b = p.adjoint(torch.from_numpy(f).to(dev)).cpu().numpy()
    finally:
        p.close()
    return a, b

out = {}
try:
    run()
    out["first"] = 0
except nat.CunfftError as e:
    out["first"] = e.status
a, b = run()  # the fault fires once: the next plan works
out["err"] = max(O.rel_l2(O.nfft_forward(x, fh, N), a), O.rel_l2(O.nfft_adjoint(x, f, N), b))
print(json.dumps(out))
"""


def _child(env_extra):
    env = dict(os.environ, **env_extra)
    code = CHILD.replace("ROOT", repr(ROOT))
    r = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    return json.loads(r.stdout.strip().splitlines()[-1])


# allocation k of one plan's life: 1-8 plan creation (roll-off table, grid, offsets,
# counters, item counts, status, sample maximum), 9-17 node bins, 18-19 the tensor-core
# interpolation's split planes and their scales (first forward)
@pytest.mark.parametrize("k", [1, 2, 8, 9, 13, 17, 18, 19])
def test_failed_allocation_is_a_status(k):
    from cunfft_gb300 import _native as nat

    out = _child({"CUNFFT_X_FAULT_ALLOC": str(k)})
    if k >= 18:
        # the automatically chosen tensor-core interpolation falls back to the shared-tile
        # form when its buffers cannot be had: the transform still succeeds
        assert out["first"] in (nat.SUCCESS, nat.ALLOC_FAILED), out
    else:
        assert out["first"] == nat.ALLOC_FAILED, out
    assert out["err"] < 1e-5, out


def test_failed_cufft_plan_is_a_status():
    from cunfft_gb300 import _native as nat

    out = _child({"CUNFFT_X_FAULT_CUFFT": "1"})
    assert out["first"] == nat.CUFFT_ERROR, out
    assert out["err"] < 1e-5, out


def test_reference_api_records_a_failed_allocation():
    """The drop-in ABI's void functions record the failure instead of exiting:
    cunfft_init with its second device allocation failing leaves ALLOC_FAILED in
    cunfft_x_last_error(plan), and cunfft_finalize still releases the plan."""
    code = r"""
import sys
sys.path.insert(0, ROOT)
from cunfft_gb300 import _native as nat
from cunfft_gb300.abi import ReferencePlan
q = ReferencePlan([32, 32], 1000)
print("status", q.status())
q.cunfft_finalize()
p = ReferencePlan([32, 32], 1000)  # the fault fired once
p.check()
p.cunfft_finalize()
print("second ok")
""".replace("ROOT", repr(ROOT))
    env = dict(os.environ, CUNFFT_X_FAULT_ALLOC="2")
    r = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    from cunfft_gb300 import _native as nat
    assert f"status {nat.ALLOC_FAILED}" in r.stdout and "second ok" in r.stdout, r.stdout + r.stderr
