"""Range of the tensor-core kernels' FP16 hi/lo operands: the power-of-two scaling
(spreading: from the call's largest sample component; interpolation: per padded grid
plane) keeps FP32 accuracy for inputs far outside FP16's range, for planes of very
different magnitude, and for all-zero inputs."""
import numpy as np
import pytest

import oracle as O

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

TOL32 = 1e-5    # FP32 form against the FP64 oracle (relative l2)


@pytest.fixture(scope="module")
def dev():
    from cunfft_gb300 import _native
    _native.lib()
    return torch.device("cuda:0")


def _rand(shape, rng):
    return rng.uniform(-1, 1, shape) + 1j * rng.uniform(-1, 1, shape)


def _plan(dev, N, x):
    from cunfft_gb300.nfft import NFFT
    p = NFFT(N, precision="f32", device=dev).set_nodes(torch.from_numpy(x).to(dev))
    assert p.spread_kernel() == "tensor" and p.interp_kernel() == "tensor"
    return p


@pytest.mark.parametrize("scale", [1e20, 1e-20, 3e4, 1.0])
def test_spread_sample_magnitudes(dev, scale):
    rng = np.random.default_rng(int(abs(np.log10(scale))) + 1)
    N, M = [16, 16, 32], 20000
    x = rng.uniform(-0.5, 0.5, (M, 3))
    f = _rand(M, rng) * scale
    p = _plan(dev, N, x)
    got = p.spread(torch.from_numpy(f).to(dev).to(torch.complex64)).cpu().numpy()
    ref = O.spread(x, f.astype(np.complex64).astype(np.complex128), N, p.n, 6)
    assert O.rel_l2(ref, got) < TOL32
    p.close()


def test_spread_mixed_sample_magnitudes(dev):
    """Samples spanning 12 orders of magnitude: the largest set the scale; the grid's
    relative error stays at the FP32 level."""
    rng = np.random.default_rng(5)
    N, M = [16, 16, 32], 20000
    x = rng.uniform(-0.5, 0.5, (M, 3))
    f = _rand(M, rng) * np.where(rng.uniform(size=M) < 0.5, 1e6, 1e-6)
    p = _plan(dev, N, x)
    got = p.spread(torch.from_numpy(f).to(dev).to(torch.complex64)).cpu().numpy()
    ref = O.spread(x, f.astype(np.complex64).astype(np.complex128), N, p.n, 6)
    assert O.rel_l2(ref, got) < TOL32
    p.close()


@pytest.mark.parametrize("scale", [1e30, 1e-30, 1.0])
def test_interp_grid_magnitudes(dev, scale):
    rng = np.random.default_rng(int(abs(np.log10(scale))) + 7)
    N, M = [16, 16, 32], 20000
    x = rng.uniform(-0.5, 0.5, (M, 3))
    p = _plan(dev, N, x)
    g = (_rand(p.n, rng) * scale).astype(np.complex64)
    got = p.interp(torch.from_numpy(g).to(dev)).cpu().numpy()
    ref = O.interp(x, g.astype(np.complex128), N, p.n, 6)
    assert O.rel_l2(ref, got) < TOL32
    p.close()


def test_interp_planes_of_different_magnitudes(dev):
    """Every grid plane scaled by its own factor between 1e-15 and 1e15 (each plane
    carries its own FP16 scale); each node's relative error against the oracle (its
    value is dominated by the largest plane in its window) stays at the FP32 level."""
    rng = np.random.default_rng(9)
    N, M = [16, 16, 32], 20000
    x = rng.uniform(-0.5, 0.5, (M, 3))
    p = _plan(dev, N, x)
    pscale = 10.0 ** rng.uniform(-15, 15, p.n[0])
    g = (_rand(p.n, rng) * pscale[:, None, None]).astype(np.complex64)
    got = p.interp(torch.from_numpy(g).to(dev)).cpu().numpy()
    ref = O.interp(x, g.astype(np.complex128), N, p.n, 6)
    rel = np.abs(got - ref) / np.abs(ref)
    assert np.percentile(rel, 99) < TOL32
    p.close()


def test_zero_inputs(dev):
    rng = np.random.default_rng(11)
    N, M = [16, 16, 32], 5000
    x = rng.uniform(-0.5, 0.5, (M, 3))
    p = _plan(dev, N, x)
    g = p.spread(torch.zeros(M, dtype=torch.complex64, device=dev))
    assert torch.count_nonzero(g).item() == 0
    f = p.interp(torch.zeros(p.n, dtype=torch.complex64, device=dev))
    assert torch.count_nonzero(f).item() == 0
    fh = p.forward(torch.zeros(N, dtype=torch.complex64, device=dev))
    assert torch.count_nonzero(fh).item() == 0
    p.synchronize()
    p.close()
