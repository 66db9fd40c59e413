"""The CPU oracle against the reference's own known answers.

The reference ships no stored vectors; its result logs record, for inputs
drawn from glibc's drand48 stream, the error E_inf of its FP64 NFFT against
its direct NDFT (tests/golden/make_kats.py explains the inputs).  Reproducing
those values to 4-5 digits pins the oracle's window-start rule, tap weights,
roll-off factors, FFT signs and layouts to the reference's.
"""
import json
import os

import numpy as np
import pytest

import oracle as O

GOLD = os.path.join(os.path.dirname(__file__), "golden", "kats.json")
KATS = json.load(open(GOLD))["kats"]
# NDFT cost bound for the default CPU run: M * N_total terms
SMALL = [k for k in KATS if k["M"] * int(np.prod(k["N"])) <= 3e7]


def _id(k):
    return f"{k['direction'][:3]}-m{k['m']}-d{k['d']}-N{k['N'][0]}"


def kat_tolerance(k):
    # m=6 values are ~1e-7 and reproduce to <1e-4 relative; m=12 values are
    # ~1e-12, where FP64 rounding of the sums moves the fourth digit.
    return 1e-3 if k["m"] <= 8 else 1e-2


def test_kat_fixture_complete():
    assert len(KATS) >= 90
    have = {(k["direction"], k["m"], k["d"]) for k in KATS}
    for direction in ("forward", "adjoint"):
        for m in (6, 12):
            for d in (1, 2, 3):
                assert (direction, m, d) in have


def test_drand48_matches_libc():
    import ctypes
    import subprocess
    import sys
    code = ("import ctypes;L=ctypes.CDLL('libc.so.6');L.drand48.restype=ctypes.c_double;"
            "print(repr([L.drand48() for _ in range(6)]))")
    out = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, check=True).stdout
    ref = eval(out)
    assert list(O.Drand48().draw(6)) == ref


@pytest.mark.parametrize("k", SMALL, ids=_id)
def test_oracle_reproduces_reference_kat(k):
    x, c = O.reference_example_data(k["N"], k["M"], k["direction"] == "adjoint", k["skip_generations"])
    if k["direction"] == "forward":
        e = O.error_l_infty(O.ndft_forward(x, c, k["N"]), O.nfft_forward(x, c, k["N"], m=k["m"]))
    else:
        e = O.error_l_infty(O.ndft_adjoint(x, c, k["N"]), O.nfft_adjoint(x, c, k["N"], m=k["m"]))
    assert abs(e / k["e_inf"] - 1.0) < kat_tolerance(k), (e, k["e_inf"])


def test_kat_inputs_are_the_tenth_repetition():
    """The same KAT fails with the first repetition's inputs: the fixture's
    skip_generations is load-bearing."""
    k = next(k for k in KATS if k["direction"] == "forward" and k["m"] == 6 and k["N"] == [64, 64])
    x, c = O.reference_example_data(k["N"], k["M"], False, 0)
    e = O.error_l_infty(O.ndft_forward(x, c, k["N"]), O.nfft_forward(x, c, k["N"], m=6))
    assert abs(e / k["e_inf"] - 1.0) > 0.05


def test_window_start_rule():
    n, m = 128, 6
    # round-to-nearest-even, minus signbit, minus m
    assert O.window_start(0.3, n, m) == 38 - 6
    assert O.window_start(-0.3, n, m) == -38 - 1 - 6
    assert O.window_start(0.0, n, m) == -6
    assert O.window_start(-0.0, n, m) == -7          # signbit(-0.0) = 1
    assert O.window_start(2.5 / n, n, m) == 2 - 6     # tie rounds to even
    assert O.window_start(3.5 / n, n, m) == 4 - 6
    assert O.window_start(-0.5, n, m) == -64 - 1 - 6


def test_params_match_reference_formulas():
    sigma, b, fac = O.params([64, 32], [128, 64], 6)
    assert np.allclose(sigma, [2.0, 2.0])
    assert np.allclose(b, 2 * 2 / (2 * 2 - 1) * 6 / np.pi)
    assert np.allclose(fac, np.pi ** 2 * b / np.array([128.0, 64.0]) ** 2)
    fg = O.fg_exp_l(b[0], 14)
    assert np.allclose(fg, np.exp(-np.arange(14) ** 2 / b[0]), rtol=1e-13)


@pytest.mark.parametrize("shape", [(32,), (16, 8), (4, 8, 16), (12,), (6, 10)])
def test_oracle_fft_matches_numpy(shape):
    rng = np.random.default_rng(1)
    a = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
    fwd = O.fft(a, -1)
    inv = O.fft(a, +1)
    assert np.allclose(fwd, np.fft.fftn(a), atol=1e-12 * np.abs(a).sum())
    assert np.allclose(inv, np.fft.ifftn(a) * a.size, atol=1e-12 * np.abs(a).sum())


@pytest.mark.parametrize("N", [[32], [16, 8], [8, 4, 8]])
def test_oracle_adjointness(N):
    """<A fhat, f> == <fhat, A^H f> for the NFFT pair and the NDFT pair."""
    rng = np.random.default_rng(7)
    M = 50
    x = rng.uniform(-0.5, 0.5, (M, len(N)))
    fh = rng.standard_normal(N) + 1j * rng.standard_normal(N)
    f = rng.standard_normal(M) + 1j * rng.standard_normal(M)
    for fwd, adj in ((O.nfft_forward, O.nfft_adjoint), (O.ndft_forward, O.ndft_adjoint)):
        lhs = np.vdot(f, fwd(x, fh, N))
        rhs = np.vdot(adj(x, f, N), fh)
        assert abs(lhs - rhs) < 1e-10 * abs(lhs)


def test_oracle_ndft_subset_matches_full():
    rng = np.random.default_rng(3)
    N = [8, 6]
    x = rng.uniform(-0.5, 0.5, (40, 2))
    fh = rng.standard_normal(N) + 1j * rng.standard_normal(N)
    f = rng.standard_normal(40) + 1j * rng.standard_normal(40)
    idx = np.array([0, 5, 39])
    assert np.allclose(O.ndft_forward_subset(x, fh, N, idx), O.ndft_forward(x, fh, N)[idx])
    kidx = np.array([0, 7, 47])
    assert np.allclose(O.ndft_adjoint_subset(x, f, N, kidx), O.ndft_adjoint(x, f, N).reshape(-1)[kidx])


def test_oracle_odd_and_small_grids():
    """Windows wider than the grid (2m+2 > n) wrap several times; odd N uses
    k in [-floor(N/2), ceil(N/2))."""
    rng = np.random.default_rng(5)
    for N, m in (([8], 12), ([8, 8], 12), ([7], 4), ([5, 6], 3)):
        x = rng.uniform(-0.5, 0.5, (30, len(N)))
        fh = rng.standard_normal(N) + 1j * rng.standard_normal(N)
        ref = O.ndft_forward(x, fh, N)
        got = O.nfft_forward(x, fh, N, m=m)
        assert O.rel_l2(ref, got) < 5e-3


@pytest.mark.parametrize("N,n", [([10], [24]), ([31], [45]), ([12, 20], [24, 50]), ([15, 9], [30, 27]),
                                 ([6, 5, 7], [12, 15, 14])])
def test_oracle_general_grid_sizes(N, n):
    """Non-power-of-two oversampled grids (true modulo wrap, direct DFT on those lengths):
    the NFFT pair stays an accurate approximation of the NDFT pair and stays adjoint."""
    rng = np.random.default_rng(sum(n))
    M = 60
    x = rng.uniform(-0.5, 0.5, (M, len(N)))
    fh = rng.standard_normal(N) + 1j * rng.standard_normal(N)
    f = rng.standard_normal(M) + 1j * rng.standard_normal(M)
    sigma = min(a / b for a, b in zip(n, N))
    tol = 1e-5 if sigma >= 2 else 1e-3
    assert O.rel_l2(O.ndft_forward(x, fh, N), O.nfft_forward(x, fh, N, n=n)) < tol
    assert O.rel_l2(O.ndft_adjoint(x, f, N), O.nfft_adjoint(x, f, N, n=n)) < tol
    lhs = np.vdot(f, O.nfft_forward(x, fh, N, n=n))
    rhs = np.vdot(O.nfft_adjoint(x, f, N, n=n), fh)
    assert abs(lhs - rhs) < 1e-10 * abs(lhs)


@pytest.mark.parametrize("N,m,tol", [([64], 6, 1e-10), ([16, 24], 6, 1e-10), ([8, 10, 12], 6, 1e-10),
                                     ([32], 4, 1e-6), ([16, 16], 8, 1e-12)])
def test_oracle_es_window_against_ndft(N, m, tol):
    """The ES window (exponential of semicircle, roll-off by quadrature) is pinned to
    the direct NDFT: about 1e-12 at m = 6, sigma = 2, where the reference's Gaussian
    stops near 1e-6; the pair stays adjoint."""
    rng = np.random.default_rng(m + len(N))
    M = 120
    x = rng.uniform(-0.5, 0.5, (M, len(N)))
    fh = rng.standard_normal(N) + 1j * rng.standard_normal(N)
    f = rng.standard_normal(M) + 1j * rng.standard_normal(M)
    fw = O.nfft_forward(x, fh, N, m=m, window="es")
    ad = O.nfft_adjoint(x, f, N, m=m, window="es")
    assert O.rel_l2(O.ndft_forward(x, fh, N), fw) < tol
    assert O.rel_l2(O.ndft_adjoint(x, f, N), ad) < tol
    assert abs(np.vdot(f, fw) - np.vdot(ad, fh)) < 1e-10 * abs(np.vdot(f, fw))
    # the window selection does not leak into later Gaussian calls
    assert O.lib().orc_get_window() == 0
    assert O.rel_l2(O.ndft_forward(x, fh, N), O.nfft_forward(x, fh, N, m=m)) > 10 * tol
