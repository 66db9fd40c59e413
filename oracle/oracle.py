"""ctypes bindings to the C oracle (oracle/cunfft_oracle.c).

Test infrastructure: a CPU FP64 restatement of the CUNFFT method and the
direct NDFT.  Arrays are numpy: nodes ``x`` float64 of shape (M, d);
coefficients complex128 of shape N (row-major, dim 0 slowest); samples
complex128 of shape (M,).
"""
import ctypes
import os

import numpy as np

from .build import LIB, build_oracle

_lib = None
_i64 = ctypes.c_int64
_pd = ctypes.POINTER(ctypes.c_double)
_pi64 = ctypes.POINTER(ctypes.c_int64)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build_oracle()
        L = ctypes.CDLL(LIB)
        L.orc_drand48_default_state.restype = ctypes.c_uint64
        L.orc_drand48_fill.argtypes = [ctypes.POINTER(ctypes.c_uint64), _pd, _i64]
        L.orc_example_data.argtypes = [ctypes.POINTER(ctypes.c_uint64), _i64, _pd, _i64, _pd]
        L.orc_next_pow2.restype = _i64
        L.orc_next_pow2.argtypes = [_i64]
        L.orc_params.argtypes = [ctypes.c_int, _pi64, _pi64, ctypes.c_int, _pd, _pd, _pd]
        L.orc_fg_exp_l.argtypes = [_pd, ctypes.c_double, ctypes.c_int]
        L.orc_window_start.restype = _i64
        L.orc_window_start.argtypes = [ctypes.c_double, _i64, ctypes.c_int]
        for name in ("orc_roc_forward", "orc_roc_adjoint"):
            getattr(L, name).argtypes = [ctypes.c_int, _pi64, _pi64, ctypes.c_int, _pd, _pd]
        L.orc_fft.argtypes = [ctypes.c_int, _pi64, _pd, ctypes.c_int]
        for name in ("orc_interp", "orc_spread", "orc_nfft_forward", "orc_nfft_adjoint"):
            getattr(L, name).argtypes = [ctypes.c_int, _pi64, _pi64, ctypes.c_int, _i64, _pd, _pd, _pd]
        for name in ("orc_ndft_forward", "orc_ndft_adjoint"):
            getattr(L, name).argtypes = [ctypes.c_int, _pi64, _i64, _pd, _pd, _pd]
        L.orc_ndft_forward_subset.argtypes = [ctypes.c_int, _pi64, _i64, _pi64, _pd, _pd, _pd]
        L.orc_ndft_adjoint_subset.argtypes = [ctypes.c_int, _pi64, _i64, _pd, _pd, _i64, _pi64, _pd]
        L.orc_error_l_infty.restype = ctypes.c_double
        L.orc_error_l_infty.argtypes = [_pd, _pd, _i64]
        L.orc_num_threads.restype = ctypes.c_int
        L.orc_set_window.argtypes = [ctypes.c_int]
        L.orc_get_window.restype = ctypes.c_int
        _lib = L
    return _lib


WINDOWS = {"gaussian": 0, "es": 1}


class _window:
    """Select the restated method's window for one call (the reference's Gaussian
    otherwise); the C oracle keeps it in a global."""

    def __init__(self, window):
        self.w = WINDOWS[window]

    def __enter__(self):
        lib().orc_set_window(self.w)

    def __exit__(self, *exc):
        lib().orc_set_window(0)


def _dp(a):
    return a.ctypes.data_as(_pd)


def _ip(a):
    return a.ctypes.data_as(_pi64)


def _dims(N):
    return np.ascontiguousarray(np.array(N, dtype=np.int64).reshape(-1))


def default_n(N):
    """n_t = 2 * next_pow2(N_t) (src/cunfft.cu:296-299)."""
    return [2 * int(lib().orc_next_pow2(int(v))) for v in N]


def params(N, n, m):
    N, n = _dims(N), _dims(n)
    d = len(N)
    sigma, b, fac = np.zeros(d), np.zeros(d), np.zeros(d)
    lib().orc_params(d, _ip(N), _ip(n), m, _dp(sigma), _dp(b), _dp(fac))
    return sigma, b, fac


def fg_exp_l(b, W):
    out = np.zeros(W)
    lib().orc_fg_exp_l(_dp(out), float(b), int(W))
    return out


def window_start(x, n, m):
    return int(lib().orc_window_start(float(x), int(n), int(m)))


class Drand48:
    """POSIX drand48 stream starting from the default (unseeded) state."""

    def __init__(self, state=None):
        self.state = ctypes.c_uint64(lib().orc_drand48_default_state() if state is None else state)

    def draw(self, count):
        out = np.empty(count, dtype=np.float64)
        lib().orc_drand48_fill(ctypes.byref(self.state), _dp(out), count)
        return out


def reference_example_data(N, M, adjoint=False, skip_generations=0):
    """Inputs of the reference drivers (src/cuda_util.cpp:151-171) from glibc's
    unseeded drand48 stream: ``ncoef`` (re, im) pairs (f_hat for the forward
    test, f for the adjoint test), then x = drand48() - 0.5 for M*d values.
    ``skip_generations`` earlier repetitions of the same draw precede them (the
    reference driver logs the tenth of ten repetitions: skip_generations=9)."""
    d = len(N)
    ncoef = int(M) if adjoint else int(np.prod(N))
    coef = np.empty(2 * ncoef, dtype=np.float64)
    x = np.empty(int(M) * d, dtype=np.float64)
    st = ctypes.c_uint64(lib().orc_drand48_default_state())
    for _ in range(int(skip_generations) + 1):
        lib().orc_example_data(ctypes.byref(st), ncoef, _dp(coef), x.size, _dp(x))
    return x.reshape(int(M), d), coef.view(np.complex128)


def _c(a):
    return np.ascontiguousarray(a, dtype=np.complex128)


def _r(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def roc_forward(fhat, N, n, m, window="gaussian"):
    N, n = _dims(N), _dims(n)
    fh = _c(fhat).reshape(-1)
    g = np.zeros(int(np.prod(n)), dtype=np.complex128)
    with _window(window):
        lib().orc_roc_forward(len(N), _ip(N), _ip(n), m, _dp(fh.view(np.float64)), _dp(g.view(np.float64)))
    return g.reshape(tuple(n))


def roc_adjoint(g, N, n, m, window="gaussian"):
    N, n = _dims(N), _dims(n)
    gg = _c(g).reshape(-1)
    fh = np.zeros(int(np.prod(N)), dtype=np.complex128)
    with _window(window):
        lib().orc_roc_adjoint(len(N), _ip(N), _ip(n), m, _dp(gg.view(np.float64)), _dp(fh.view(np.float64)))
    return fh.reshape(tuple(N))


def fft(a, sign):
    a = _c(a).copy()
    n = _dims(a.shape)
    lib().orc_fft(len(n), _ip(n), _dp(a.reshape(-1).view(np.float64)), int(sign))
    return a


def interp(x, g, N, n, m, window="gaussian"):
    N, n = _dims(N), _dims(n)
    x = _r(x).reshape(-1, len(N))
    gg = _c(g).reshape(-1)
    f = np.zeros(x.shape[0], dtype=np.complex128)
    with _window(window):
        lib().orc_interp(len(N), _ip(N), _ip(n), m, x.shape[0], _dp(x), _dp(gg.view(np.float64)),
                     _dp(f.view(np.float64)))
    return f


def spread(x, f, N, n, m, window="gaussian"):
    N, n = _dims(N), _dims(n)
    x = _r(x).reshape(-1, len(N))
    ff = _c(f).reshape(-1)
    g = np.zeros(int(np.prod(n)), dtype=np.complex128)
    with _window(window):
        lib().orc_spread(len(N), _ip(N), _ip(n), m, x.shape[0], _dp(x), _dp(ff.view(np.float64)),
                     _dp(g.view(np.float64)))
    return g.reshape(tuple(n))


def nfft_forward(x, fhat, N, n=None, m=6, window="gaussian"):
    N = _dims(N)
    n = _dims(default_n(N) if n is None else n)
    x = _r(x).reshape(-1, len(N))
    fh = _c(fhat).reshape(-1)
    f = np.zeros(x.shape[0], dtype=np.complex128)
    with _window(window):
        lib().orc_nfft_forward(len(N), _ip(N), _ip(n), m, x.shape[0], _dp(x),
                           _dp(fh.view(np.float64)), _dp(f.view(np.float64)))
    return f


def nfft_adjoint(x, f, N, n=None, m=6, window="gaussian"):
    N = _dims(N)
    n = _dims(default_n(N) if n is None else n)
    x = _r(x).reshape(-1, len(N))
    ff = _c(f).reshape(-1)
    fh = np.zeros(int(np.prod(N)), dtype=np.complex128)
    with _window(window):
        lib().orc_nfft_adjoint(len(N), _ip(N), _ip(n), m, x.shape[0], _dp(x),
                           _dp(ff.view(np.float64)), _dp(fh.view(np.float64)))
    return fh.reshape(tuple(int(v) for v in N))


def ndft_forward(x, fhat, N):
    N = _dims(N)
    x = _r(x).reshape(-1, len(N))
    fh = _c(fhat).reshape(-1)
    f = np.zeros(x.shape[0], dtype=np.complex128)
    lib().orc_ndft_forward(len(N), _ip(N), x.shape[0], _dp(x), _dp(fh.view(np.float64)),
                           _dp(f.view(np.float64)))
    return f


def ndft_adjoint(x, f, N):
    N = _dims(N)
    x = _r(x).reshape(-1, len(N))
    ff = _c(f).reshape(-1)
    fh = np.zeros(int(np.prod(N)), dtype=np.complex128)
    lib().orc_ndft_adjoint(len(N), _ip(N), x.shape[0], _dp(x), _dp(ff.view(np.float64)),
                           _dp(fh.view(np.float64)))
    return fh.reshape(tuple(int(v) for v in N))


def ndft_forward_subset(x, fhat, N, idx):
    N = _dims(N)
    x = _r(x).reshape(-1, len(N))
    idx = np.ascontiguousarray(idx, dtype=np.int64)
    fh = _c(fhat).reshape(-1)
    f = np.zeros(idx.size, dtype=np.complex128)
    lib().orc_ndft_forward_subset(len(N), _ip(N), idx.size, _ip(idx), _dp(x),
                                  _dp(fh.view(np.float64)), _dp(f.view(np.float64)))
    return f


def ndft_adjoint_subset(x, f, N, kidx):
    N = _dims(N)
    x = _r(x).reshape(-1, len(N))
    kidx = np.ascontiguousarray(kidx, dtype=np.int64)
    ff = _c(f).reshape(-1)
    out = np.zeros(kidx.size, dtype=np.complex128)
    lib().orc_ndft_adjoint_subset(len(N), _ip(N), x.shape[0], _dp(x), _dp(ff.view(np.float64)),
                                  kidx.size, _ip(kidx), _dp(out.view(np.float64)))
    return out


def error_l_infty(ref, y):
    a = _c(ref).reshape(-1)
    b = _c(y).reshape(-1)
    return float(lib().orc_error_l_infty(_dp(a.view(np.float64)), _dp(b.view(np.float64)), a.size))


def rel_l2(ref, y):
    ref = np.asarray(ref).reshape(-1)
    y = np.asarray(y).reshape(-1)
    return float(np.linalg.norm(ref - y) / np.linalg.norm(ref))


def num_threads():
    return int(lib().orc_num_threads())
