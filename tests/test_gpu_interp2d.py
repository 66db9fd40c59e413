"""The 2D FP32 tensor-core interpolation kernel (k_interp2_tc: nodes binned by 16 x 16
sub-tiles of window starts, A = w1 in shared memory, B = the sub-tile's FP16 hi/lo rows by
TMA, FP16 hi/lo x 3 into tensor memory) against the shared-tile kernel and the FP64
oracle: every window width, outer tile extents, small, odd and non-power-of-two grids,
clustered and boundary nodes, batched uneven instances, the ES window, grids that are only
8-byte aligned, and the binning's sub-tile order.
Reference: the 2D forward gridding kernelConvWithGauss_2d (src/cunfft_kernel.cu:667-712)."""
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


def _check_kinds(p, x, N, m, rng, tol=TOL32, window="gaussian", kinds=("tensor", "shared")):
    """Both kernels' samples from one random grid against the oracle's, and the forward."""
    g = _rand(([p.batch] if p.batch > 1 else []) + p.n, rng)
    gt = torch.from_numpy(g).to(p.device).to(torch.complex64)
    ref = O.interp(x, g, N, p.n, m, window=window)
    for k in kinds:
        p.set_interp_kernel(k)
        assert p.interp_kernel() == k
        f = p.interp(gt)
        p.synchronize()  # raises on a device-side check failure
        err = O.rel_l2(ref, f.cpu().numpy())
        assert err < tol, (k, err)
    p.set_interp_kernel("auto")
    assert p.interp_kernel() == kinds[0]
    fh = _rand(N, rng)
    ref_f = O.nfft_forward(x, fh, N, n=p.n, m=m, window=window)
    assert O.rel_l2(ref_f, p.forward(torch.from_numpy(fh).to(p.device)).cpu()) < tol


@pytest.mark.parametrize("m", [1, 2, 3, 4, 5, 6, 7])
def test_interp2d_every_width(dev, m):
    from cunfft_gb300.nfft import NFFT
    rng = np.random.default_rng(300 + m)
    N, M = [64, 48], 30000
    x = rng.uniform(-0.5, 0.5, (M, 2))
    p = NFFT(N, m=m, precision="f32", device=dev).set_nodes(torch.from_numpy(x).to(dev))
    assert p.interp_kernel() == "tensor"
    _check_kinds(p, x, N, m, rng)
    p.close()


@pytest.mark.parametrize("T0", [1, 4, 16, 32, 64])
def test_interp2d_outer_tile_extents(dev, T0):
    """Sub-tiles of min(T0, 16) rows."""
    from cunfft_gb300.nfft import NFFT
    rng = np.random.default_rng(60 + T0)
    N, M = [128, 64], 25000
    x = rng.uniform(-0.5, 0.5, (M, 2))
    p = NFFT(N, m=6, precision="f32", device=dev).set_nodes(torch.from_numpy(x).to(dev))
    p.set_tiling([T0])
    assert p.tiling()["T"][0] == T0
    _check_kinds(p, x, N, 6, rng)
    p.close()


@pytest.mark.parametrize("N,n", [([8, 8], None), ([64, 8], None), ([33, 45], [70, 96]),
                                 ([33, 45], [71, 96]), ([40, 100], [80, 208])])
def test_interp2d_small_odd_and_general_grids(dev, N, n):
    """Rows shorter than the tile, odd and non-power-of-two row counts (partial last tiles
    and sub-tiles), and non-power-of-two row lengths divisible by 8."""
    from cunfft_gb300.nfft import NFFT
    rng = np.random.default_rng(sum(N) + 7)
    M = 5000
    x = rng.uniform(-0.5, 0.5, (M, 2))
    m = 3 if N[0] <= 8 or N[1] <= 8 else 6
    p = NFFT(N, n=n, m=m, precision="f32", device=dev).set_nodes(torch.from_numpy(x).to(dev))
    _check_kinds(p, x, N, m, rng, tol=5 * TOL32)
    p.close()


@pytest.mark.parametrize("N,n", [([64, 4], None), ([33, 45], [70, 90])])
def test_interp2d_unsupported_grids_take_the_shared_kernel(dev, N, n):
    """Rows shorter than 16 columns, or a row length not divisible by 8: the plan keeps
    the shared-tile kernel."""
    from cunfft_gb300._native import CunfftError
    from cunfft_gb300.nfft import NFFT
    rng = np.random.default_rng(9)
    x = rng.uniform(-0.5, 0.5, (3000, 2))
    p = NFFT(N, n=n, m=3, precision="f32", device=dev).set_nodes(torch.from_numpy(x).to(dev))
    assert p.interp_kernel() == "shared"
    with pytest.raises(CunfftError):
        p.set_interp_kernel("tensor")
    _check_kinds(p, x, N, 3, rng, tol=5 * TOL32, kinds=("shared",))
    p.close()


def test_interp2d_clustered_and_boundary_nodes(dev):
    """Many nodes in a few sub-tiles (chains of 128-node items), nodes on -1/2, just below
    +1/2 and at -0.0."""
    from cunfft_gb300.nfft import NFFT
    rng = np.random.default_rng(56)
    N, M = [128, 128], 60001
    x = np.clip(rng.normal(0.05, 0.01, (M, 2)), -0.5, 0.4999)
    x[:50] = -0.5
    x[50:100] = np.nextafter(0.5, 0)
    x[100:150] = -0.0
    p = NFFT(N, m=6, precision="f32", device=dev).set_nodes(torch.from_numpy(x).to(dev))
    _check_kinds(p, x, N, 6, rng)
    p.close()


def test_interp2d_batched_uneven(dev):
    from cunfft_gb300.nfft import NFFT
    rng = np.random.default_rng(67)
    N, Ms = [64, 64], [7000, 0, 1234, 1]
    xs = [rng.uniform(-0.5, 0.5, (M, 2)) for M in Ms]
    p = NFFT(N, m=5, precision="f32", batch=4, device=dev)
    p.set_nodes(torch.from_numpy(np.concatenate(xs)).to(dev), M_inst=Ms)
    assert p.interp_kernel() == "tensor"
    g = _rand([4] + p.n, rng)
    gt = torch.from_numpy(g).to(dev).to(torch.complex64)
    ref = np.concatenate([O.interp(xs[i], g[i], N, p.n, 5) for i in range(4)])
    for k in ("tensor", "shared"):
        p.set_interp_kernel(k)
        err = O.rel_l2(ref, p.interp(gt).cpu().numpy())
        p.synchronize()
        assert err < TOL32, (k, err)
    p.close()


def test_interp2d_es_window(dev):
    from cunfft_gb300.nfft import NFFT
    rng = np.random.default_rng(78)
    N, M = [64, 64], 20000
    x = rng.uniform(-0.5, 0.5, (M, 2))
    p = NFFT(N, m=6, precision="f32", device=dev, window="es").set_nodes(torch.from_numpy(x).to(dev))
    _check_kinds(p, x, N, 6, rng, window="es")
    p.close()


def test_interp2d_grid_alignments(dev):
    """A caller grid that starts 8 bytes into its buffer takes the split's 8-byte loads."""
    from cunfft_gb300.nfft import NFFT
    rng = np.random.default_rng(89)
    N, M = [64, 64], 20000
    x = rng.uniform(-0.5, 0.5, (M, 2))
    p = NFFT(N, m=6, precision="f32", device=dev).set_nodes(torch.from_numpy(x).to(dev))
    g = _rand(p.n, rng)
    ref = O.interp(x, g, N, p.n, 6)
    ntot = int(np.prod(p.n))
    buf = torch.zeros(ntot + 1, dtype=torch.complex64, device=dev)
    gv = buf[1:].view(p.n)
    gv.copy_(torch.from_numpy(g).to(torch.complex64))
    assert gv.data_ptr() % 16 == 8
    for k in ("tensor", "shared"):
        p.set_interp_kernel(k)
        out = torch.empty(M, dtype=torch.complex64, device=dev)
        p.interp(gv, out=out)
        p.synchronize()
        assert O.rel_l2(ref, out.cpu().numpy()) < TOL32, k
    p.close()


def test_interp2d_sub_tile_binning(dev):
    """The binning orders each tile's nodes by 16 x 16 sub-tile of window starts: the same
    node set gives the same samples through every tiling and both kernels, and the
    spreading (which reads tile-level items over the same order) still matches."""
    from cunfft_gb300.nfft import NFFT
    rng = np.random.default_rng(90)
    N, M = [64, 64], 40000
    x = rng.uniform(-0.5, 0.5, (M, 2))
    f = _rand(M, rng)
    p = NFFT(N, m=6, precision="f32", device=dev).set_nodes(torch.from_numpy(x).to(dev))
    ref_s = O.spread(x, f, N, p.n, 6)
    assert O.rel_l2(ref_s, p.spread(torch.from_numpy(f).to(dev)).cpu().numpy()) < TOL32
    g = _rand(p.n, rng)
    gt = torch.from_numpy(g).to(dev).to(torch.complex64)
    ref = O.interp(x, g, N, p.n, 6)
    for T0 in (64, 16, 2):
        p.set_tiling([T0])
        assert O.rel_l2(ref, p.interp(gt).cpu().numpy()) < TOL32, T0
        assert O.rel_l2(ref_s, p.spread(torch.from_numpy(f).to(dev)).cpu().numpy()) < TOL32, T0
    p.synchronize()
    p.close()
