"""Failure reporting without a GPU fault: a kernel's bounded completion wait that gives
up sets the plan's device status flag, synchronize() reports it once
(CUNFFT_X_DEVICE_CHECK_FAILED) and clears it, and the plan keeps working."""
import numpy as np
import pytest

import oracle as O

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

DEVICE_CHECK_FAILED = 7


def test_wait_that_gives_up_is_reported_once():
    from cunfft_gb300 import _native
    from cunfft_gb300.nfft import NFFT
    _native.lib()
    dev = torch.device("cuda:0")
    rng = np.random.default_rng(5)
    N, M = [16, 16, 32], 3000
    x = rng.uniform(-0.5, 0.5, (M, 3))
    fh = rng.uniform(-1, 1, N) + 1j * rng.uniform(-1, 1, N)
    p = NFFT(N, precision="f32", device=dev).set_nodes(torch.from_numpy(x).to(dev))
    p.synchronize()
    p.check_wait_timeout()
    with pytest.raises(_native.CunfftError) as ei:
        p.synchronize()
    assert ei.value.status == DEVICE_CHECK_FAILED
    assert "gave up" in str(ei.value)
    p.synchronize()  # the flag was cleared on read
    got = p.forward(torch.from_numpy(fh).to(dev)).cpu().numpy()
    p.synchronize()
    assert O.rel_l2(O.nfft_forward(x, fh, N), got) < 1e-5
    p.close()
