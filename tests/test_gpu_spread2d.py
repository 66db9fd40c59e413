"""The 2D FP32 tensor-core spreading kernel (k_spread2_tm: A = w0 in tensor memory, B =
w1 f in shared memory, FP16 hi/lo x 3, bulk FP32 reductions) against the shared-tile
kernel and the FP64 oracle: every window width, outer tile extents, small, odd and
non-power-of-two grids (the atomic fallbacks), clustered and boundary nodes, batched
uneven instances, the ES window and caller grids that are only 8-byte aligned.
Reference: the 2D adjoint gridding kernelConvWithGauss_adjoint_2d (src/cunfft_kernel.cu:842-878)."""
import numpy as np
import pytest

import oracle as O

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

TOL32 = 1e-5  # FP32 form vs the FP64 oracle (relative l2), as the parity tests


@pytest.fixture(scope="module")
def dev():
    from cunfft_gb300 import _native
    _native.lib()
    return torch.device("cuda:0")


def _rand(shape, rng):
    return rng.uniform(-1, 1, shape) + 1j * rng.uniform(-1, 1, shape)


def _check_kinds(p, x, f, N, m, tol=TOL32, window="gaussian"):
    """The tensor and shared-tile kernels' grids against the oracle's, and the adjoint."""
    ft = torch.from_numpy(f).to(p.device)
    ref = O.spread(x, f, N, p.n, m, window=window)
    for k in ("tensor", "shared"):
        p.set_spread_kernel(k)
        assert p.spread_kernel() == k
        g = p.spread(ft)
        p.synchronize()  # raises on a device-side check failure
        err = O.rel_l2(ref, g.cpu().numpy())
        assert err < tol, (k, err)
    p.set_spread_kernel("auto")
    assert p.spread_kernel() == "tensor"
    assert O.rel_l2(O.nfft_adjoint(x, f, N, n=p.n, m=m, window=window), p.adjoint(ft).cpu()) < tol


@pytest.mark.parametrize("m", [1, 2, 3, 4, 5, 6, 7])
def test_spread2d_every_width(dev, m):
    from cunfft_gb300.nfft import NFFT
    rng = np.random.default_rng(200 + m)
    N, M = [64, 48], 30000
    x = rng.uniform(-0.5, 0.5, (M, 2))
    f = _rand(M, rng)
    p = NFFT(N, m=m, precision="f32", device=dev).set_nodes(torch.from_numpy(x).to(dev))
    assert p.tiling()["T"][:2] == [64, 64]
    _check_kinds(p, x, f, N, m)
    p.close()


@pytest.mark.parametrize("T0", [1, 8, 16, 32, 64])
def test_spread2d_outer_tile_extents(dev, T0):
    from cunfft_gb300.nfft import NFFT
    rng = np.random.default_rng(40 + T0)
    N, M = [128, 64], 25000
    x = rng.uniform(-0.5, 0.5, (M, 2))
    f = _rand(M, rng)
    p = NFFT(N, m=6, precision="f32", device=dev).set_nodes(torch.from_numpy(x).to(dev))
    p.set_tiling([T0])
    assert p.tiling()["T"][0] == T0
    _check_kinds(p, x, f, N, 6)
    p.close()


@pytest.mark.parametrize("N,n", [([8, 8], None), ([4, 64], None), ([64, 4], None), ([33, 45], [70, 90]),
                                 ([33, 45], [71, 91]), ([40, 100], [80, 202])])
def test_spread2d_small_odd_and_general_grids(dev, N, n):
    """Rows shorter than the padded tile (the columns wrap more than once), odd row lengths
    and odd or non-power-of-two grid sizes take the kernel's atomic paths."""
    from cunfft_gb300.nfft import NFFT
    rng = np.random.default_rng(sum(N))
    M = 5000
    x = rng.uniform(-0.5, 0.5, (M, 2))
    f = _rand(M, rng)
    m = 3 if N[0] <= 8 or N[1] <= 8 else 6
    p = NFFT(N, n=n, m=m, precision="f32", device=dev).set_nodes(torch.from_numpy(x).to(dev))
    _check_kinds(p, x, f, N, m, tol=5 * TOL32)
    p.close()


def test_spread2d_clustered_and_boundary_nodes(dev):
    """Many nodes in a few tiles (chains of work items on one tile, partial batches), nodes
    on -1/2, just below +1/2 and at -0.0."""
    from cunfft_gb300.nfft import NFFT
    rng = np.random.default_rng(55)
    N, M = [128, 128], 60001
    x = np.clip(rng.normal(0.05, 0.01, (M, 2)), -0.5, 0.4999)
    x[:50] = -0.5
    x[50:100] = np.nextafter(0.5, 0)
    x[100:150] = -0.0
    f = _rand(M, rng)
    p = NFFT(N, m=6, precision="f32", device=dev).set_nodes(torch.from_numpy(x).to(dev))
    _check_kinds(p, x, f, N, 6)
    p.close()


def test_spread2d_batched_uneven(dev):
    from cunfft_gb300.nfft import NFFT
    rng = np.random.default_rng(66)
    N, Ms = [64, 64], [7000, 0, 1234, 1]
    xs = [rng.uniform(-0.5, 0.5, (M, 2)) for M in Ms]
    fs = [_rand(M, rng) for M in Ms]
    p = NFFT(N, m=5, precision="f32", batch=4, device=dev)
    p.set_nodes(torch.from_numpy(np.concatenate(xs)).to(dev), M_inst=Ms)
    assert p.spread_kernel() == "tensor"
    ft = torch.from_numpy(np.concatenate(fs)).to(dev)
    ref = np.stack([O.spread(xs[i], fs[i], N, p.n, 5) for i in range(4)])
    for k in ("tensor", "shared"):
        p.set_spread_kernel(k)
        err = O.rel_l2(ref, p.spread(ft).cpu().numpy())
        p.synchronize()
        assert err < TOL32, (k, err)
    p.close()


def test_spread2d_es_window(dev):
    from cunfft_gb300.nfft import NFFT
    rng = np.random.default_rng(77)
    N, M = [64, 64], 20000
    x = rng.uniform(-0.5, 0.5, (M, 2))
    f = _rand(M, rng)
    p = NFFT(N, m=6, precision="f32", device=dev, window="es").set_nodes(torch.from_numpy(x).to(dev))
    _check_kinds(p, x, f, N, 6, window="es")
    p.close()


def test_spread2d_grid_alignments(dev):
    """A caller grid that starts 8 bytes into its buffer takes the 8-byte paths."""
    from cunfft_gb300.nfft import NFFT
    rng = np.random.default_rng(88)
    N, M = [64, 64], 20000
    x = rng.uniform(-0.5, 0.5, (M, 2))
    f = _rand(M, rng)
    p = NFFT(N, m=6, precision="f32", device=dev).set_nodes(torch.from_numpy(x).to(dev))
    ref = O.spread(x, f, N, p.n, 6)
    ft = torch.from_numpy(f).to(dev).to(torch.complex64)
    ntot = int(np.prod(p.n))
    buf = torch.zeros(ntot + 1, dtype=torch.complex64, device=dev)
    g = buf[1:].view(p.n)
    assert g.data_ptr() % 16 == 8
    for k in ("tensor", "shared"):
        p.set_spread_kernel(k)
        g.zero_()
        p.spread(ft, g)
        p.synchronize()
        assert O.rel_l2(ref, g.cpu().numpy()) < TOL32, k
        assert buf[0].item() == 0
    p.close()
