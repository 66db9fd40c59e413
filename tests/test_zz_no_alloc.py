"""cunfft_x_spread_noalloc: spreading for callers that cannot allocate device memory.

Some callers cannot call cudaMalloc: frameworks whose device memory all belongs to
their own pool allocator, real-time loops that must not pay for or fail on an
allocation, and host applications that forbid allocation inside plug-in callbacks.
The entry point keeps its scratch in a fixed array inside the library instead of
plan-owned allocations.  These tests call it through the C ABI twice in a row (the
second call reuses the scratch the first one left behind) and compare each result
with the plan-based spreading entry point cunfft_x_spread, within the tolerances of
the other parity tests; they also check the device status word it clears and fills,
an empty call after a non-empty one, and the size limit.  The file is collected
last on purpose.
"""
import ctypes

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

TOL = {"f64": 1e-12, "f32": 1e-5}


def _noalloc(lib):
    fn = lib.cunfft_x_spread_noalloc
    fn.restype = ctypes.c_int
    fn.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_int64), ctypes.c_int,
                   ctypes.c_int, ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                   ctypes.c_void_p]
    return fn


def _vp(t):
    return ctypes.c_void_p(t.data_ptr())


@pytest.mark.parametrize("N,M,m,prec", [([32, 32, 32], 60000, 6, "f32"), ([32, 32, 32], 30000, 6, "f64"),
                                        ([64, 48], 20000, 5, "f64"), ([256], 3000, 4, "f32")])
def test_spread_noalloc_matches_plan_spread_twice(N, M, m, prec):
    from cunfft_gb300 import _native as nat
    from cunfft_gb300.nfft import NFFT

    lib = nat.lib()
    fn = _noalloc(lib)
    dev = torch.device("cuda:0")
    cd = torch.complex128 if prec == "f64" else torch.complex64
    d = len(N)
    Na = (ctypes.c_int64 * d)(*N)
    stream = torch.cuda.current_stream(dev)
    rng = np.random.default_rng(M + m)
    # the status word starts non-zero: the call must clear it before the kernels run
    status = torch.full((1,), 99, dtype=torch.int32, device=dev)
    for call in range(2):
        x = torch.from_numpy(rng.uniform(-0.5, 0.5, (M, d))).to(dev)
        f = torch.from_numpy(rng.uniform(-1, 1, M) + 1j * rng.uniform(-1, 1, M)).to(dev, cd)
        plan = NFFT(N, m=m, precision=prec, device=dev).set_nodes(x)
        ref = plan.spread(f)
        g = torch.zeros_like(ref)
        st = fn(d, Na, None, m, plan.precision, M, _vp(x), _vp(f), _vp(g), ctypes.c_void_p(stream.cuda_stream),
                _vp(status) if call == 0 else None)
        assert st == nat.SUCCESS, f"call {call}: status {st}"
        torch.cuda.synchronize()
        err = (torch.linalg.norm(g - ref) / torch.linalg.norm(ref)).item()
        assert err < TOL[prec], f"call {call}: rel l2 {err}"
        if call == 0:
            assert int(status.item()) == 0
        plan.close()


def test_spread_noalloc_empty_call_leaves_grid_unchanged():
    """M = 0 after a call with nodes: no device work on the grid, status cleared."""
    from cunfft_gb300 import _native as nat

    fn = _noalloc(nat.lib())
    dev = torch.device("cuda:0")
    N = [32, 32, 32]
    Na = (ctypes.c_int64 * 3)(*N)
    rng = np.random.default_rng(5)
    M = 20000
    x = torch.from_numpy(rng.uniform(-0.5, 0.5, (M, 3))).to(dev)
    f = torch.from_numpy(rng.uniform(-1, 1, M) + 1j * rng.uniform(-1, 1, M)).to(dev, torch.complex64)
    g = torch.zeros((64, 64, 64), dtype=torch.complex64, device=dev)
    s = ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
    assert fn(3, Na, None, 6, nat.F32, M, _vp(x), _vp(f), _vp(g), s, None) == nat.SUCCESS
    torch.cuda.synchronize()
    before = g.clone()
    status = torch.full((1,), 7, dtype=torch.int32, device=dev)
    assert fn(3, Na, None, 6, nat.F32, 0, None, None, _vp(g), s, _vp(status)) == nat.SUCCESS
    torch.cuda.synchronize()
    assert torch.equal(g, before)
    assert int(status.item()) == 0


def test_spread_noalloc_rejects_oversized_requests():
    from cunfft_gb300 import _native as nat

    fn = _noalloc(nat.lib())
    N = (ctypes.c_int64 * 1)(64)
    # more nodes than the fixed scratch holds: rejected before any device work
    assert fn(1, N, None, 6, nat.F32, (1 << 20) + 1, ctypes.c_void_p(1), ctypes.c_void_p(1),
              ctypes.c_void_p(1), None, None) == nat.INVALID_ARGUMENT
    # more tiles than the scratch holds (512^3 grid, 8 x 8 x 16 tiles: 131072)
    N3 = (ctypes.c_int64 * 3)(256, 256, 256)
    assert fn(3, N3, None, 6, nat.F32, 10, ctypes.c_void_p(1), ctypes.c_void_p(1),
              ctypes.c_void_p(1), None, None) == nat.INVALID_ARGUMENT
