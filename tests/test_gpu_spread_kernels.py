"""The 3D FP32 spreading kernels (tensor-core FP16 hi + lo, register-tile, shared-tile)
against each other and the oracle; kernel selection through the extension API."""
import numpy as np
import pytest

import oracle as O

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

TOL32 = 1e-5     # FP32 form vs the FP64 oracle (relative l2), as the parity tests
TOL_KERN = 5e-6  # FP32 spreading kernels against each other (graph replay test)


@pytest.fixture(scope="module")
def dev():
    from cunfft_gb300 import _native
    _native.lib()
    return torch.device("cuda:0")


def _rand(shape, rng):
    return rng.uniform(-1, 1, shape) + 1j * rng.uniform(-1, 1, shape)


def _spread_kinds(p, f, kinds):
    """Grid of each requested spreading kernel (then back to the automatic choice)."""
    out = {}
    for k in kinds:
        p.set_spread_kernel(k)
        assert p.spread_kernel() == k
        out[k] = p.spread(f).clone()
        p.synchronize()  # raises on a device-side check failure
    p.set_spread_kernel("auto")
    return out


def _agree(grids, ref, tol=TOL32):
    """Every kernel's grid against the FP64 oracle grid."""
    for k, g in grids.items():
        err = O.rel_l2(ref, g.cpu().numpy())
        assert err < tol, (k, err)


@pytest.mark.parametrize("m", [1, 2, 3, 4, 5, 6, 7])
def test_spread_kernels_agree_every_width(dev, m):
    from cunfft_gb300.nfft import NFFT
    rng = np.random.default_rng(100 + m)
    N, M = [32, 32, 32], 30000
    x = rng.uniform(-0.5, 0.5, (M, 3))
    f = _rand(M, rng)
    p = NFFT(N, m=m, precision="f32", device=dev).set_nodes(torch.from_numpy(x).to(dev))
    assert p.spread_kernel() == "tensor"
    ft = torch.from_numpy(f).to(dev)
    _agree(_spread_kinds(p, ft, ["tensor", "register", "shared"]), O.spread(x, f, N, p.n, m))
    assert O.rel_l2(O.nfft_adjoint(x, f, N, m=m), p.adjoint(ft).cpu()) < TOL32
    p.close()


@pytest.mark.parametrize("T0", [1, 2, 4, 8, 16])
def test_spread_kernels_outer_tile_extents(dev, T0):
    from cunfft_gb300.nfft import NFFT
    rng = np.random.default_rng(7 + T0)
    N, M = [16, 32, 64], 20000
    x = rng.uniform(-0.5, 0.5, (M, 3))
    f = _rand(M, rng)
    p = NFFT(N, m=6, precision="f32", device=dev).set_nodes(torch.from_numpy(x).to(dev))
    p.set_tiling([T0])
    assert p.tiling()["T"][0] == T0
    kinds = ["tensor", "shared"] + (["register"] if T0 <= 8 else [])
    ft = torch.from_numpy(f).to(dev)
    _agree(_spread_kinds(p, ft, kinds), O.spread(x, f, N, p.n, 6))
    assert O.rel_l2(O.nfft_adjoint(x, f, N), p.adjoint(ft).cpu()) < TOL32
    p.close()


@pytest.mark.parametrize("N", [[4, 4, 4], [8, 2, 16], [2, 8, 4], [64, 8, 4]])
def test_spread_kernels_small_and_ragged_grids(dev, N):
    """Grids smaller than the fixed inner tile (8 x 16): the padded tile wraps onto itself."""
    from cunfft_gb300.nfft import NFFT
    rng = np.random.default_rng(sum(N))
    M = 3000
    x = rng.uniform(-0.5, 0.5, (M, 3))
    f = _rand(M, rng)
    p = NFFT(N, m=3, precision="f32", device=dev).set_nodes(torch.from_numpy(x).to(dev))
    ft = torch.from_numpy(f).to(dev)
    _agree(_spread_kinds(p, ft, ["tensor", "register", "shared"]), O.spread(x, f, N, p.n, 3), 5 * TOL32)
    assert O.rel_l2(O.nfft_adjoint(x, f, N, m=3), p.adjoint(ft).cpu()) < 5 * TOL32
    p.close()


def test_spread_kernels_clustered_and_boundary_nodes(dev):
    """Many nodes in a few tiles (long work-item chains, partial batches), nodes on -1/2,
    just below +1/2 and at -0.0."""
    from cunfft_gb300.nfft import NFFT
    rng = np.random.default_rng(5)
    N, M = [32, 32, 32], 40001
    x = np.clip(rng.normal(0.1, 0.02, (M, 3)), -0.5, 0.4999)
    x[:50] = -0.5
    x[50:100] = np.nextafter(0.5, 0)
    x[100:150] = -0.0
    f = _rand(M, rng)
    p = NFFT(N, m=6, precision="f32", device=dev).set_nodes(torch.from_numpy(x).to(dev))
    ft = torch.from_numpy(f).to(dev)
    _agree(_spread_kinds(p, ft, ["tensor", "register", "shared"]), O.spread(x, f, N, p.n, 6))
    assert O.rel_l2(O.nfft_adjoint(x, f, N), p.adjoint(ft).cpu()) < TOL32
    p.close()


def test_spread_kernels_batched_uneven(dev):
    from cunfft_gb300.nfft import NFFT
    rng = np.random.default_rng(11)
    N, Ms = [16, 16, 16], [5000, 0, 1234]
    xs = [rng.uniform(-0.5, 0.5, (M, 3)) for M in Ms]
    fs = [_rand(M, rng) for M in Ms]
    p = NFFT(N, m=5, precision="f32", batch=3, device=dev)
    p.set_nodes(torch.from_numpy(np.concatenate(xs)).to(dev), M_inst=Ms)
    ft = torch.from_numpy(np.concatenate(fs)).to(dev)
    ref = np.stack([O.spread(xs[i], fs[i], N, p.n, 5) for i in range(3)])
    _agree(_spread_kinds(p, ft, ["tensor", "register", "shared"]), ref)
    got = p.adjoint(ft).cpu().numpy()
    for i in range(3):
        if Ms[i]:
            assert O.rel_l2(O.nfft_adjoint(xs[i], fs[i], N, m=5), got[i]) < TOL32
        else:
            assert np.abs(got[i]).max() == 0
    p.close()


def test_spread_tensor_few_nodes(dev):
    """1, 7 and 17 nodes: partial batches of the 16-node staging."""
    from cunfft_gb300.nfft import NFFT
    rng = np.random.default_rng(13)
    N = [16, 16, 16]
    for M in (1, 7, 17):
        x = rng.uniform(-0.5, 0.5, (M, 3))
        f = _rand(M, rng)
        p = NFFT(N, precision="f32", device=dev).set_nodes(torch.from_numpy(x).to(dev))
        ft = torch.from_numpy(f).to(dev)
        _agree(_spread_kinds(p, ft, ["tensor", "shared"]), O.spread(x, f, N, p.n, 6))
        assert O.rel_l2(O.nfft_adjoint(x, f, N), p.adjoint(ft).cpu()) < TOL32
        p.close()


def test_spread_kernel_graph_follows_choice(dev):
    from cunfft_gb300.nfft import NFFT
    rng = np.random.default_rng(12)
    N, M = [32, 32, 32], 20000
    x = rng.uniform(-0.5, 0.5, (M, 3))
    f = torch.from_numpy(_rand(M, rng)).to(dev).to(torch.complex64)
    p = NFFT(N, precision="f32", device=dev).set_nodes(torch.from_numpy(x).to(dev))
    out = torch.empty(N, dtype=torch.complex64, device=dev)
    outs = {}
    for k in ("tensor", "register", "shared"):
        p.set_spread_kernel(k)
        p.adjoint_graph(f, out)
        outs[k] = out.clone()
    torch.cuda.synchronize()
    ref = p.adjoint(f).cpu().numpy()
    for k, v in outs.items():
        assert O.rel_l2(ref, v.cpu().numpy()) < TOL_KERN, k
    p.close()


def test_spread_kernel_selection_rules(dev):
    from cunfft_gb300._native import CunfftError
    from cunfft_gb300.nfft import NFFT
    x3 = torch.rand(100, 3, dtype=torch.float64, device=dev) - 0.5
    # FP64 plans and 2D plans with 2m+2 > 16: only the shared-tile kernel
    for prec, N, x, m in (("f64", [16, 16, 16], x3, 6), ("f32", [32, 32], x3[:, :2].contiguous(), 8)):
        p = NFFT(N, m=m, precision=prec, device=dev).set_nodes(x)
        assert p.spread_kernel() == "shared"
        for k in ("register", "tensor"):
            with pytest.raises(CunfftError):
                p.set_spread_kernel(k)
        assert p.spread_kernel() == "shared"
        p.close()
    # 2D FP32 with 2m+2 <= 16: the 2D tensor-core kernel (tiles up to 64 x 64), no register form
    p = NFFT([128, 128], precision="f32", device=dev).set_nodes(x3[:, :2].contiguous())
    assert p.spread_kernel() == "tensor"
    with pytest.raises(CunfftError):
        p.set_spread_kernel("register")
    p.set_tiling([128])                 # beyond the kernel's 64-row outer extent: shared
    assert p.spread_kernel() == "shared"
    p.set_tiling([32])
    assert p.spread_kernel() == "tensor"
    p.close()
    # 2m+2 = 18 > 16
    p = NFFT([16, 16, 16], m=8, precision="f32", device=dev).set_nodes(x3)
    assert p.spread_kernel() == "shared"
    p.close()
    p = NFFT([32, 32, 32], precision="f32", device=dev).set_nodes(x3)
    assert p.spread_kernel() == "tensor"
    p.set_spread_kernel("register")
    assert p.spread_kernel() == "register"
    p.set_tiling([16])                  # the register kernel stops at 8: shared, request kept
    assert p.spread_kernel() == "shared"
    p.set_tiling([4])
    assert p.spread_kernel() == "register"
    p.set_spread_kernel("auto")
    assert p.spread_kernel() == "tensor"
    p.set_tiling([16])
    assert p.spread_kernel() == "tensor"
    p.set_spread_kernel("shared")
    p.set_tiling([8])
    assert p.spread_kernel() == "shared"
    with pytest.raises(KeyError):
        p.set_spread_kernel("bogus")
    p.close()


def test_autotune_picks_a_kernel_and_stays_correct(dev):
    from cunfft_gb300.nfft import NFFT
    rng = np.random.default_rng(21)
    N, M = [32, 32, 32], 50000
    x = rng.uniform(-0.5, 0.5, (M, 3))
    f = _rand(M, rng)
    p = NFFT(N, precision="f32", device=dev).set_nodes(torch.from_numpy(x).to(dev))
    t = p.autotune(reps=1)
    assert t["spread"] in ("tensor", "register", "shared")
    assert O.rel_l2(O.nfft_adjoint(x, f, N), p.adjoint(torch.from_numpy(f).to(dev)).cpu()) < TOL32
    p.synchronize()
    p.close()


@pytest.mark.parametrize("T0", [8, 16])
def test_tensor_spreading_grid_alignments(dev, T0):
    """The tensor-memory-operand form (T0 = 8 at m = 6) adds its staged rows to the grid
    with 16-byte bulk reductions when the grid is 16-byte aligned and falls back to
    atomics otherwise; T0 = 16 runs the shared-memory-operand form.  A grid that starts
    8 bytes into its buffer, and a batched grid (instances ntot apart), match the oracle."""
    from cunfft_gb300.nfft import NFFT
    rng = np.random.default_rng(300 + T0)
    N, M = [32, 32, 32], 20000
    x = rng.uniform(-0.5, 0.5, (M, 3))
    f = _rand(M, rng)
    p = NFFT(N, precision="f32", device=dev).set_nodes(torch.from_numpy(x).to(dev))
    p.set_tiling([T0])
    assert p.spread_kernel() == "tensor"
    ref = O.spread(x, f, N, p.n, 6)
    ft = torch.from_numpy(f).to(dev).to(torch.complex64)
    ntot = int(np.prod(p.n))
    buf = torch.zeros(ntot + 1, dtype=torch.complex64, device=dev)
    g = buf[1:].view(p.n)
    assert g.data_ptr() % 16 == 8
    for k in ("tensor", "register", "shared") if T0 <= 8 else ("tensor", "shared"):
        p.set_spread_kernel(k)
        g.zero_()
        p.spread(ft, g)
        p.synchronize()
        assert O.rel_l2(ref, g.cpu().numpy()) < TOL32, k
        assert buf[0].item() == 0
    p.set_spread_kernel("auto")
    assert O.rel_l2(ref, p.spread(ft).cpu().numpy()) < TOL32
    # interpolation from a grid that starts 8 bytes into its buffer
    gv = _rand(p.n, rng).astype(np.complex64)
    g.copy_(torch.from_numpy(gv).to(dev))
    ref_f = O.interp(x, gv.astype(np.complex128), N, p.n, 6)
    for k in ("tensor", "shared"):
        p.set_interp_kernel(k)
        assert O.rel_l2(ref_f, p.interp(g).cpu().numpy()) < TOL32, k
        p.synchronize()
    p.set_interp_kernel("auto")
    p.close()
    # two instances with different node sets: instance i's grid starts at i ntot
    xs = [rng.uniform(-0.5, 0.5, (Mi, 3)) for Mi in (7000, 11000)]
    fs = [_rand(len(xi), rng) for xi in xs]
    pb = NFFT(N, precision="f32", batch=2, device=dev)
    pb.set_nodes(torch.from_numpy(np.concatenate(xs)).to(dev), M_inst=[len(xi) for xi in xs])
    pb.set_tiling([T0])
    gb = pb.spread(torch.from_numpy(np.concatenate(fs)).to(dev).to(torch.complex64)).cpu().numpy()
    for i in range(2):
        assert O.rel_l2(O.spread(xs[i], fs[i], N, pb.n, 6), gb[i]) < TOL32
    pb.close()
