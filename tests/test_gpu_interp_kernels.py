"""The 3D FP32 interpolation kernels (tensor-core 3xTF32 and shared-tile) against the
oracle; kernel selection through the extension API."""
import numpy as np
import pytest

import oracle as O

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

TOL32 = 1e-5     # FP32 form vs the FP64 oracle (relative l2), as the parity tests


@pytest.fixture(scope="module")
def dev():
    from cunfft_gb300 import _native
    _native.lib()
    return torch.device("cuda:0")


def _rand(shape, rng):
    return rng.uniform(-1, 1, shape) + 1j * rng.uniform(-1, 1, shape)


def _interp_kinds(p, g, kinds):
    """Samples interpolated from grid g by each requested kernel."""
    out = {}
    for k in kinds:
        p.set_interp_kernel(k)
        assert p.interp_kernel() == k
        out[k] = p.interp(g).clone()
        p.synchronize()  # raises on a device-side check failure
    p.set_interp_kernel("auto")
    return out


def _agree(outs, ref, tol=TOL32):
    for k, v in outs.items():
        err = O.rel_l2(ref, v.cpu().numpy())
        assert err < tol, (k, err)


def _grid(p, rng, dev):
    g = _rand(([p.batch] if p.batch > 1 else []) + p.n, rng)
    return g, torch.from_numpy(g).to(dev).to(torch.complex64)


@pytest.mark.parametrize("m", [1, 2, 3, 4, 5, 6, 7])
def test_interp_kernels_every_width(dev, m):
    from cunfft_gb300.nfft import NFFT
    rng = np.random.default_rng(200 + m)
    N, M = [32, 32, 32], 30000
    x = rng.uniform(-0.5, 0.5, (M, 3))
    p = NFFT(N, m=m, precision="f32", device=dev).set_nodes(torch.from_numpy(x).to(dev))
    assert p.interp_kernel() == "tensor"
    g, gt = _grid(p, rng, dev)
    _agree(_interp_kinds(p, gt, ["tensor", "shared"]), O.interp(x, g, N, p.n, m))
    fh = _rand(N, rng)
    assert O.rel_l2(O.nfft_forward(x, fh, N, m=m), p.forward(torch.from_numpy(fh).to(dev)).cpu()) < TOL32
    p.close()


@pytest.mark.parametrize("T0", [1, 2, 4, 8, 16])
def test_interp_kernels_outer_tile_extents(dev, T0):
    from cunfft_gb300.nfft import NFFT
    rng = np.random.default_rng(17 + T0)
    N, M = [16, 32, 64], 20000
    x = rng.uniform(-0.5, 0.5, (M, 3))
    p = NFFT(N, m=6, precision="f32", device=dev).set_nodes(torch.from_numpy(x).to(dev))
    p.set_tiling([T0])
    assert p.tiling()["T"][0] == T0
    g, gt = _grid(p, rng, dev)
    _agree(_interp_kinds(p, gt, ["tensor", "shared"]), O.interp(x, g, N, p.n, 6))
    p.close()


@pytest.mark.parametrize("N", [[4, 4, 4], [8, 2, 16], [2, 8, 4], [64, 8, 4]])
def test_interp_kernels_small_and_ragged_grids(dev, N):
    """Grids smaller than the padded tile: rows and columns wrap onto themselves."""
    from cunfft_gb300.nfft import NFFT
    rng = np.random.default_rng(sum(N) + 1)
    M = 3000
    x = rng.uniform(-0.5, 0.5, (M, 3))
    p = NFFT(N, m=3, precision="f32", device=dev).set_nodes(torch.from_numpy(x).to(dev))
    g, gt = _grid(p, rng, dev)
    _agree(_interp_kinds(p, gt, ["tensor", "shared"]), O.interp(x, g, N, p.n, 3))
    p.close()


def test_interp_kernels_clustered_and_boundary_nodes(dev):
    """Thousands of nodes in a few tiles: work items of up to 1024 nodes, i.e. several
    128-node batches per tile, and partial batches; nodes on -1/2, below +1/2, -0.0."""
    from cunfft_gb300.nfft import NFFT
    rng = np.random.default_rng(6)
    N, M = [32, 32, 32], 40001
    x = np.clip(rng.normal(0.1, 0.02, (M, 3)), -0.5, 0.4999)
    x[:50] = -0.5
    x[50:100] = np.nextafter(0.5, 0)
    x[100:150] = -0.0
    p = NFFT(N, m=6, precision="f32", device=dev).set_nodes(torch.from_numpy(x).to(dev))
    g, gt = _grid(p, rng, dev)
    _agree(_interp_kinds(p, gt, ["tensor", "shared"]), O.interp(x, g, N, p.n, 6))
    p.close()


def test_interp_kernels_batched_uneven(dev):
    from cunfft_gb300.nfft import NFFT
    rng = np.random.default_rng(12)
    N, Ms = [16, 16, 16], [5000, 0, 1234]
    xs = [rng.uniform(-0.5, 0.5, (M, 3)) for M in Ms]
    p = NFFT(N, m=5, precision="f32", batch=3, device=dev)
    p.set_nodes(torch.from_numpy(np.concatenate(xs)).to(dev), M_inst=Ms)
    g, gt = _grid(p, rng, dev)
    ref = np.concatenate([O.interp(xs[i], g[i], N, p.n, 5) for i in range(3)])
    _agree(_interp_kinds(p, gt, ["tensor", "shared"]), ref)
    p.close()


def test_interp_tensor_few_nodes(dev):
    from cunfft_gb300.nfft import NFFT
    rng = np.random.default_rng(14)
    N = [16, 16, 16]
    for M in (1, 7, 129, 300):
        x = rng.uniform(-0.5, 0.5, (M, 3))
        p = NFFT(N, precision="f32", device=dev).set_nodes(torch.from_numpy(x).to(dev))
        g, gt = _grid(p, rng, dev)
        _agree(_interp_kinds(p, gt, ["tensor", "shared"]), O.interp(x, g, N, p.n, 6))
        p.close()


def test_interp_kernel_graph_follows_choice(dev):
    from cunfft_gb300.nfft import NFFT
    rng = np.random.default_rng(15)
    N, M = [32, 32, 32], 20000
    x = rng.uniform(-0.5, 0.5, (M, 3))
    fh = torch.from_numpy(_rand(N, rng)).to(dev).to(torch.complex64)
    p = NFFT(N, precision="f32", device=dev).set_nodes(torch.from_numpy(x).to(dev))
    out = torch.empty(M, dtype=torch.complex64, device=dev)
    outs = {}
    for k in ("tensor", "shared"):
        p.set_interp_kernel(k)
        p.forward_graph(fh, out)
        outs[k] = out.clone()
    torch.cuda.synchronize()
    ref = O.nfft_forward(x, fh.cpu().numpy().astype(np.complex128), N)
    for k, v in outs.items():
        assert O.rel_l2(ref, v.cpu().numpy()) < TOL32, k
    p.close()


def test_interp_kernel_selection_rules(dev):
    from cunfft_gb300._native import CunfftError
    from cunfft_gb300.nfft import NFFT
    x3 = torch.rand(100, 3, dtype=torch.float64, device=dev) - 0.5
    # FP64; a 2D grid whose inner tile is narrower than the 16-column sub-tiles; 3D with
    # a last size below 8
    for prec, N, x in (("f64", [16, 16, 16], x3), ("f32", [32, 4], x3[:, :2].contiguous()),
                       ("f32", [8, 8, 1], x3)):
        p = NFFT(N, precision=prec, device=dev).set_nodes(x)
        assert p.interp_kernel() == "shared"
        with pytest.raises(CunfftError):
            p.set_interp_kernel("tensor")
        assert p.interp_kernel() == "shared"
        p.close()
    p = NFFT([16, 16, 16], m=8, precision="f32", device=dev).set_nodes(x3)   # 2m+2 = 18 > 16
    assert p.interp_kernel() == "shared"
    p.close()
    p = NFFT([32, 32], precision="f32", device=dev).set_nodes(x3[:, :2].contiguous())
    assert p.interp_kernel() == "tensor"
    p.close()
    p = NFFT([32, 32, 32], precision="f32", device=dev).set_nodes(x3)
    assert p.interp_kernel() == "tensor"
    p.set_tiling([16])
    assert p.interp_kernel() == "tensor"
    p.set_interp_kernel("shared")
    p.set_tiling([8])
    assert p.interp_kernel() == "shared"
    p.set_interp_kernel("auto")
    assert p.interp_kernel() == "tensor"
    with pytest.raises(KeyError):
        p.set_interp_kernel("bogus")
    p.close()


def test_autotune_chooses_both_kernels(dev):
    from cunfft_gb300.nfft import NFFT
    rng = np.random.default_rng(22)
    N, M = [32, 32, 32], 50000
    x = rng.uniform(-0.5, 0.5, (M, 3))
    fh = _rand(N, rng)
    p = NFFT(N, precision="f32", device=dev).set_nodes(torch.from_numpy(x).to(dev))
    t = p.autotune(reps=1)
    assert t["interp"] in ("tensor", "shared") and t["spread"] in ("tensor", "register", "shared")
    assert O.rel_l2(O.nfft_forward(x, fh, N), p.forward(torch.from_numpy(fh).to(dev)).cpu()) < TOL32
    p.synchronize()
    p.close()
