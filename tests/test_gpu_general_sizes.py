"""Oversampled grids of any size (not only powers of two) and odd bandwidths.

The reference wraps window indices with &(n-1) (src/cunfft_kernel.cu:590, :768,
:1036), so it needs power-of-two n; here any n >= N is accepted.  Every result is
compared with the oracle on the same n (the oracle wraps by true modulo and runs a
direct DFT on non-power-of-two lengths), and the approximation against the direct
NDFT at sigma = 2.
"""
import numpy as np
import pytest

import oracle as O

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

TOL64 = 1e-12   # FP64 form against the FP64 oracle on identical inputs (relative l2)
TOL32 = 1e-5    # FP32 form against the FP64 oracle


@pytest.fixture(scope="module")
def dev():
    from cunfft_gb300 import _native
    _native.lib()
    return torch.device("cuda:0")


def _rand(shape, rng):
    return rng.uniform(-1, 1, shape) + 1j * rng.uniform(-1, 1, shape)


CASES = [
    ([10], [24]), ([33], [70]), ([31], [45]),                  # 1D: even n, odd N, odd n
    ([12, 20], [24, 50]), ([15, 9], [30, 27]),                 # 2D: 50 = 2 x 25, odd N and odd n
    ([12, 10, 20], [24, 30, 40]),                              # 3D, last size divisible by 8
    ([9, 11, 13], [18, 22, 26]),                               # 3D, last size even only
    ([10, 10, 11], [20, 21, 27]),                              # 3D, odd sizes
]


@pytest.mark.parametrize("N,n", CASES)
@pytest.mark.parametrize("prec", ["f64", "f32"])
def test_general_sizes_match_oracle(dev, N, n, prec):
    from cunfft_gb300.nfft import NFFT
    rng = np.random.default_rng(sum(n) + len(prec))
    d, M = len(N), 3000
    x = rng.uniform(-0.5, 0.5, (M, d))
    x[:10] = -0.5
    x[10:20] = np.nextafter(0.5, 0)
    fh, f = _rand(N, rng), _rand(M, rng)
    tol = TOL64 if prec == "f64" else TOL32
    p = NFFT(N, n=n, m=4, precision=prec, device=dev).set_nodes(torch.from_numpy(x).to(dev))
    assert p.n == n
    got_f = p.forward(torch.from_numpy(fh).to(dev)).cpu().numpy()
    got_fh = p.adjoint(torch.from_numpy(f).to(dev)).cpu().numpy()
    p.synchronize()
    assert O.rel_l2(O.nfft_forward(x, fh, N, n=n, m=4), got_f) < tol
    assert O.rel_l2(O.nfft_adjoint(x, f, N, n=n, m=4), got_fh) < tol
    p.close()


@pytest.mark.parametrize("N,n", [([12, 10, 20], [24, 30, 40]), ([9, 11, 13], [18, 22, 26]),
                                 ([10, 10, 11], [20, 21, 27])])
def test_general_sizes_every_kernel_form(dev, N, n):
    """FP32 3D: each spreading and interpolation form the plan offers, on grids whose
    last size is divisible by 8, only even, or odd (the tensor-core forms' 16-byte pairs
    and boxes need the even / divisible-by-8 row length)."""
    from cunfft_gb300.nfft import NFFT
    rng = np.random.default_rng(sum(n))
    M = 5000
    x = rng.uniform(-0.5, 0.5, (M, 3))
    f = _rand(M, rng)
    p = NFFT(N, n=n, m=5, precision="f32", device=dev).set_nodes(torch.from_numpy(x).to(dev))
    ref_g = O.spread(x, f, N, n, 5)
    ft = torch.from_numpy(f).to(dev)
    assert p.spread_kernel() == "tensor"
    for k in ("tensor", "register", "shared"):
        p.set_spread_kernel(k)
        assert p.spread_kernel() == k
        assert O.rel_l2(ref_g, p.spread(ft).cpu().numpy()) < TOL32, k
        p.synchronize()
    p.set_spread_kernel("auto")
    g = _rand(n, rng)
    gt = torch.from_numpy(g).to(dev).to(torch.complex64)
    ref_f = O.interp(x, g, N, n, 5)
    kinds = ["tensor", "shared"] if n[2] % 8 == 0 else ["shared"]
    assert p.interp_kernel() == kinds[0]
    for k in kinds:
        p.set_interp_kernel(k)
        assert O.rel_l2(ref_f, p.interp(gt).cpu().numpy()) < TOL32, k
        p.synchronize()
    p.close()


@pytest.mark.parametrize("T0", [1, 2, 4, 8, 16])
def test_partial_tiles(dev, T0):
    """n_0 = 30 and n_1 = 20 are not multiples of the tile extents: the last tile of each
    dimension is partial."""
    from cunfft_gb300.nfft import NFFT
    rng = np.random.default_rng(40 + T0)
    N, n, M = [15, 10, 24], [30, 20, 48], 8000
    x = rng.uniform(-0.5, 0.5, (M, 3))
    fh, f = _rand(N, rng), _rand(M, rng)
    for prec, tol in (("f32", TOL32), ("f64", TOL64)):
        p = NFFT(N, n=n, m=6, precision=prec, device=dev).set_nodes(torch.from_numpy(x).to(dev))
        p.set_tiling([T0])
        assert O.rel_l2(O.nfft_forward(x, fh, N, n=n), p.forward(torch.from_numpy(fh).to(dev)).cpu().numpy()) < tol
        assert O.rel_l2(O.nfft_adjoint(x, f, N, n=n), p.adjoint(torch.from_numpy(f).to(dev)).cpu().numpy()) < tol
        p.synchronize()
        p.close()


def test_general_sizes_batched_uneven(dev):
    from cunfft_gb300.nfft import NFFT
    rng = np.random.default_rng(50)
    N, n, Ms = [14, 18], [28, 36], [900, 0, 2500]
    xs = [rng.uniform(-0.5, 0.5, (M, 2)) for M in Ms]
    fhs = [_rand(N, rng) for _ in Ms]
    fs = [_rand(M, rng) for M in Ms]
    p = NFFT(N, n=n, m=6, precision="f64", batch=3, device=dev)
    p.set_nodes(torch.from_numpy(np.concatenate(xs)).to(dev), M_inst=Ms)
    got_f = p.forward(torch.from_numpy(np.stack(fhs)).to(dev)).cpu().numpy()
    got_fh = p.adjoint(torch.from_numpy(np.concatenate(fs)).to(dev)).cpu().numpy()
    off = np.concatenate([[0], np.cumsum(Ms)])
    for i in range(3):
        if Ms[i]:
            assert O.rel_l2(O.nfft_forward(xs[i], fhs[i], N, n=n), got_f[off[i]:off[i + 1]]) < TOL64
            assert O.rel_l2(O.nfft_adjoint(xs[i], fs[i], N, n=n), got_fh[i]) < TOL64
        else:
            assert np.abs(got_fh[i]).max() == 0
    p.close()


def test_general_sizes_accuracy_against_ndft(dev):
    """sigma = 2 on non-power-of-two grids keeps the window's accuracy (m = 6)."""
    from cunfft_gb300.nfft import NFFT
    rng = np.random.default_rng(60)
    N, n, M = [12, 10, 20], [24, 20, 40], 2000
    x = rng.uniform(-0.5, 0.5, (M, 3))
    fh, f = _rand(N, rng), _rand(M, rng)
    p = NFFT(N, n=n, m=6, precision="f64", device=dev).set_nodes(torch.from_numpy(x).to(dev))
    assert O.rel_l2(O.ndft_forward(x, fh, N), p.forward(torch.from_numpy(fh).to(dev)).cpu().numpy()) < 1e-5
    assert O.rel_l2(O.ndft_adjoint(x, f, N), p.adjoint(torch.from_numpy(f).to(dev)).cpu().numpy()) < 1e-5
    p.close()


def test_general_sizes_node_gradient(dev):
    """Derivative-of-Gaussian gridding on a non-power-of-two grid against the NDFT gradient."""
    from cunfft_gb300.nfft import NFFT
    rng = np.random.default_rng(70)
    N, n, M = [10, 12], [30, 36], 300
    x = rng.uniform(-0.45, 0.45, (M, 2))
    fh = rng.standard_normal(N) + 1j * rng.standard_normal(N)
    gf = rng.standard_normal(M) + 1j * rng.standard_normal(M)
    p = NFFT(N, n=n, m=12, device=dev).set_nodes(torch.from_numpy(x).to(dev))
    got = p.node_gradient(torch.from_numpy(fh).to(dev), torch.from_numpy(gf).to(dev)).cpu().numpy()
    ks = np.meshgrid(*[np.arange(-(v // 2), v - v // 2) for v in N], indexing="ij")
    ref = np.zeros((M, 2))
    for t in range(2):
        ref[:, t] = (np.conj(gf) * O.ndft_forward(x, (-2j * np.pi * ks[t]) * fh, N)).real
    assert np.linalg.norm(got - ref) / np.linalg.norm(ref) < 1e-9
    p.close()


def test_reference_api_guru_non_power_of_two(dev):
    """cunfft_initGuru with a user grid the reference itself cannot take (n = 3 N)."""
    from cunfft_gb300.abi import ReferencePlan
    rng = np.random.default_rng(80)
    N, n, M = [16, 20], [48, 60], 700
    x = rng.uniform(-0.5, 0.5, (M, 2))
    fh = _rand(N, rng).reshape(-1)
    p = ReferencePlan(N, M, n=n)
    p.x[:] = x
    p.f_hat[:] = fh
    p.copyDataToDevice()
    p.cunfft_transform()
    p.copyDataToHost()
    p.check()
    assert O.rel_l2(O.nfft_forward(x, fh, N, n=n), p.f) < TOL64
    p.cunfft_finalize()
