"""cunfft_x_spread_noalloc: spreading for callers that cannot allocate device memory.

The entry point keeps its scratch in a fixed array inside the library instead
of plan-owned allocations, for callers such as code captured into CUDA graphs or
frameworks that own all device memory.  This test calls it through the C ABI
twice in a row (the second call reuses the scratch the first one left behind)
and compares each result with the plan-based spreading entry point
cunfft_x_spread, within the tolerances of the other parity tests.  The file is
collected last on purpose.
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
                   ctypes.c_int, ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    return fn


@pytest.mark.parametrize("N,M,m,prec", [([32, 32, 32], 60000, 6, "f32"), ([64, 48], 20000, 5, "f64"),
                                        ([256], 3000, 4, "f32")])
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
    for call in range(2):
        x = torch.from_numpy(rng.uniform(-0.5, 0.5, (M, d))).to(dev)
        f = torch.from_numpy(rng.uniform(-1, 1, M) + 1j * rng.uniform(-1, 1, M)).to(dev, cd)
        plan = NFFT(N, m=m, precision=prec, device=dev).set_nodes(x)
        ref = plan.spread(f)
        g = torch.zeros_like(ref)
        st = fn(d, Na, None, m, plan.precision, M, ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(f.data_ptr()),
                ctypes.c_void_p(g.data_ptr()), ctypes.c_void_p(stream.cuda_stream))
        assert st == nat.SUCCESS, f"call {call}: status {st}"
        torch.cuda.synchronize()
        err = (torch.linalg.norm(g - ref) / torch.linalg.norm(ref)).item()
        assert err < TOL[prec], f"call {call}: rel l2 {err}"
        plan.close()


def test_spread_noalloc_rejects_oversized_requests():
    from cunfft_gb300 import _native as nat

    fn = _noalloc(nat.lib())
    N = (ctypes.c_int64 * 1)(64)
    # more nodes than the fixed scratch holds: rejected before any device work
    assert fn(1, N, None, 6, nat.F32, (1 << 20) + 1, ctypes.c_void_p(1), ctypes.c_void_p(1),
              ctypes.c_void_p(1), None) == nat.INVALID_ARGUMENT
