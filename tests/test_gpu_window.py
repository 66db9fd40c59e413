"""The ES window (exponential of semicircle) behind cunfft_x_set_window: parity with
the oracle's ES restatement, accuracy against the direct NDFT, every gridding
kernel form, switching windows on a plan with bound nodes and captured graphs."""
import numpy as np
import pytest

import oracle as O

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

TOL64 = 1e-12   # FP64 form against the FP64 oracle, same window (relative l2)
TOL32 = 1e-5    # FP32 form against the FP64 oracle
NDFT64 = 1e-10  # FP64 ES form against the direct NDFT at m = 6, sigma = 2


@pytest.fixture(scope="module")
def dev():
    from cunfft_gb300 import _native
    _native.lib()
    return torch.device("cuda:0")


def _rand(shape, rng):
    return rng.uniform(-1, 1, shape) + 1j * rng.uniform(-1, 1, shape)


@pytest.mark.parametrize("N", [[64], [16, 24], [12, 10, 16]])
def test_es_fp64_matches_oracle_and_ndft(dev, N):
    from cunfft_gb300.nfft import NFFT
    rng = np.random.default_rng(len(N))
    d, M = len(N), 1500
    x = rng.uniform(-0.5, 0.5, (M, d))
    x[:5] = -0.5
    fh, f = _rand(N, rng), _rand(M, rng)
    p = NFFT(N, precision="f64", window="es", device=dev).set_nodes(torch.from_numpy(x).to(dev))
    assert p.window() == "es"
    got_f = p.forward(torch.from_numpy(fh).to(dev)).cpu().numpy()
    got_fh = p.adjoint(torch.from_numpy(f).to(dev)).cpu().numpy()
    assert O.rel_l2(O.nfft_forward(x, fh, N, window="es"), got_f) < TOL64
    assert O.rel_l2(O.nfft_adjoint(x, f, N, window="es"), got_fh) < TOL64
    assert O.rel_l2(O.ndft_forward(x, fh, N), got_f) < NDFT64
    assert O.rel_l2(O.ndft_adjoint(x, f, N), got_fh) < NDFT64
    p.close()


@pytest.mark.parametrize("m", [1, 2, 3, 4, 5, 6, 7])
def test_es_fp32_every_kernel_every_width(dev, m):
    """3D FP32: the tensor-core, register and shared spreading and the tensor-core and
    shared interpolation against the oracle's ES grids, at every width they cover."""
    from cunfft_gb300.nfft import NFFT
    rng = np.random.default_rng(300 + m)
    N, M = [32, 32, 32], 20000
    x = rng.uniform(-0.5, 0.5, (M, 3))
    f = _rand(M, rng)
    p = NFFT(N, m=m, precision="f32", window="es", device=dev).set_nodes(torch.from_numpy(x).to(dev))
    ft = torch.from_numpy(f).to(dev)
    ref_g = O.spread(x, f, N, p.n, m, window="es")
    for k in ("tensor", "register", "shared"):
        p.set_spread_kernel(k)
        assert O.rel_l2(ref_g, p.spread(ft).cpu().numpy()) < TOL32, k
        p.synchronize()
    p.set_spread_kernel("auto")
    g = _rand(p.n, rng)
    gt = torch.from_numpy(g).to(dev).to(torch.complex64)
    ref_f = O.interp(x, g, N, p.n, m, window="es")
    for k in ("tensor", "shared"):
        p.set_interp_kernel(k)
        assert O.rel_l2(ref_f, p.interp(gt).cpu().numpy()) < TOL32, k
        p.synchronize()
    p.close()


def test_es_fp32_transforms_against_ndft(dev):
    from cunfft_gb300.nfft import NFFT
    rng = np.random.default_rng(7)
    N, M = [16, 32, 32], 30000
    x = rng.uniform(-0.5, 0.5, (M, 3))
    fh, f = _rand(N, rng), _rand(M, rng)
    p = NFFT(N, precision="f32", window="es", device=dev).set_nodes(torch.from_numpy(x).to(dev))
    assert p.spread_kernel() == "tensor" and p.interp_kernel() == "tensor"
    idx = rng.choice(M, 500, replace=False)
    got_f = p.forward(torch.from_numpy(fh).to(dev)).cpu().numpy()
    assert O.rel_l2(O.ndft_forward(x[idx], fh, N), got_f[idx]) < TOL32
    got_fh = p.adjoint(torch.from_numpy(f).to(dev)).cpu().numpy()
    assert O.rel_l2(O.nfft_adjoint(x, f, N, window="es"), got_fh) < TOL32
    p.close()


def test_window_switch_with_bound_nodes_and_graphs(dev):
    """Switching the window keeps the node binding, and captured graphs follow."""
    from cunfft_gb300.nfft import NFFT
    rng = np.random.default_rng(8)
    N, M = [16, 16, 16], 8000
    x = rng.uniform(-0.5, 0.5, (M, 3))
    fh = _rand(N, rng)
    fht = torch.from_numpy(fh).to(dev).to(torch.complex64)
    p = NFFT(N, precision="f32", device=dev).set_nodes(torch.from_numpy(x).to(dev))
    out = torch.empty(M, dtype=torch.complex64, device=dev)
    res = {}
    for w in ("gaussian", "es", "gaussian", "es"):
        p.set_window(w)
        assert p.window() == w
        p.forward_graph(fht, out)
        res.setdefault(w, []).append(out.clone())
        res[w].append(p.forward(fht).clone())
    torch.cuda.synchronize()
    for w, outs in res.items():
        ref = O.nfft_forward(x, fh, N, window=w)
        for o in outs:
            assert O.rel_l2(ref, o.cpu().numpy()) < TOL32, w
    with pytest.raises(KeyError):
        p.set_window("kaiser")
    p.close()


def test_es_batched_general_sizes(dev):
    from cunfft_gb300.nfft import NFFT
    rng = np.random.default_rng(9)
    N, n, Ms = [14, 18], [28, 36], [700, 0, 1300]
    xs = [rng.uniform(-0.5, 0.5, (M, 2)) for M in Ms]
    fhs = [_rand(N, rng) for _ in Ms]
    p = NFFT(N, n=n, precision="f64", batch=3, window="es", device=dev)
    p.set_nodes(torch.from_numpy(np.concatenate(xs)).to(dev), M_inst=Ms)
    got = p.forward(torch.from_numpy(np.stack(fhs)).to(dev)).cpu().numpy()
    off = np.concatenate([[0], np.cumsum(Ms)])
    for i in range(3):
        if Ms[i]:
            seg = got[off[i]:off[i + 1]]
            assert O.rel_l2(O.nfft_forward(xs[i], fhs[i], N, n=n, window="es"), seg) < TOL64
            assert O.rel_l2(O.ndft_forward(xs[i], fhs[i], N), seg) < NDFT64
    p.close()


def test_es_node_gradient(dev):
    """Derivative-of-ES gridding against the FP64 NDFT gradient."""
    from cunfft_gb300.nfft import NFFT
    rng = np.random.default_rng(10)
    N, M = [12, 16], 300
    x = rng.uniform(-0.45, 0.45, (M, 2))
    fh = rng.standard_normal(N) + 1j * rng.standard_normal(N)
    gf = rng.standard_normal(M) + 1j * rng.standard_normal(M)
    p = NFFT(N, window="es", device=dev).set_nodes(torch.from_numpy(x).to(dev))
    got = p.node_gradient(torch.from_numpy(fh).to(dev), torch.from_numpy(gf).to(dev)).cpu().numpy()
    ks = np.meshgrid(*[np.arange(-(v // 2), v - v // 2) for v in N], indexing="ij")
    ref = np.zeros((M, 2))
    for t in range(2):
        ref[:, t] = (np.conj(gf) * O.ndft_forward(x, (-2j * np.pi * ks[t]) * fh, N)).real
    assert np.linalg.norm(got - ref) / np.linalg.norm(ref) < 1e-8
    p.close()
