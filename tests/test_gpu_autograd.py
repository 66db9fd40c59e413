"""Differentiable NFFT: gradients w.r.t. coefficients and node positions.

Checked against central finite differences (h = 1e-6) of the same FP64 NFFT and
against the FP64 NDFT gradient d f_j / d x_{j,t} = sum_k (-2 pi i k_t) f_hat_k e^{-2 pi i k.x_j}.
"""
import numpy as np
import pytest

import oracle as O

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def dev():
    from cunfft_gb300 import _native
    _native.lib()
    return torch.device("cuda:0")


def _ndft_grad_x(x, fh, N, gf):
    """Re(conj(gf_j) * d f_j/d x_{j,t}) with the FP64 NDFT (oracle), spectral derivative."""
    d = len(N)
    ks = np.meshgrid(*[np.arange(-(n // 2), n - n // 2) for n in N], indexing="ij")
    out = np.zeros((x.shape[0], d))
    for t in range(d):
        dfh = (-2j * np.pi * ks[t]) * fh
        df = O.ndft_forward(x, dfh, N)
        out[:, t] = (np.conj(gf) * df).real
    return out


@pytest.mark.parametrize("N,M", [([32], 200), ([16, 16], 300), ([8, 8, 8], 200)])
def test_node_gradient_matches_ndft_gradient(dev, N, M):
    from cunfft_gb300.nfft import NFFT

    rng = np.random.default_rng(len(N))
    x = rng.uniform(-0.45, 0.45, (M, len(N)))
    fh = rng.standard_normal(N) + 1j * rng.standard_normal(N)
    gf = rng.standard_normal(M) + 1j * rng.standard_normal(M)
    p = NFFT(N, m=12, device=dev).set_nodes(torch.from_numpy(x).to(dev))
    got = p.node_gradient(torch.from_numpy(fh).to(dev), torch.from_numpy(gf).to(dev)).cpu().numpy()
    ref = _ndft_grad_x(x, fh, N, gf)
    assert np.linalg.norm(got - ref) / np.linalg.norm(ref) < 1e-9
    p.close()


def test_autograd_function_gradients(dev):
    from cunfft_gb300.autograd import nfft
    from cunfft_gb300.nfft import NFFT

    rng = np.random.default_rng(0)
    N, M = [16, 16], 400
    x0 = rng.uniform(-0.45, 0.45, (M, 2))
    fh0 = rng.standard_normal(N) + 1j * rng.standard_normal(N)
    y = torch.from_numpy(O.ndft_forward(x0 + rng.normal(0, 1e-3, x0.shape), fh0, N)).to(dev)
    plan = NFFT(N, m=6, device=dev)
    x = torch.from_numpy(x0).to(dev).requires_grad_(True)
    fh = torch.from_numpy(fh0).to(dev).requires_grad_(True)
    loss = (nfft(x, fh, plan=plan) - y).abs().pow(2).sum()
    loss.backward()
    # coefficient gradient: dL/d conj(fh) convention of torch = A^H (2 (A fh - y))
    r = O.nfft_forward(x0, fh0, N) - y.cpu().numpy()
    g_fh = O.nfft_adjoint(x0, 2 * r, N)
    assert np.linalg.norm(fh.grad.cpu().numpy() - g_fh) / np.linalg.norm(g_fh) < 1e-10
    # node gradient against central finite differences of the loss (h = 1e-6)
    h = 1e-6
    gx = x.grad.cpu().numpy()
    for j, t in [(0, 0), (17, 1), (123, 0), (399, 1)]:
        xp, xm = x0.copy(), x0.copy()
        xp[j, t] += h
        xm[j, t] -= h
        lp = np.sum(np.abs(O.nfft_forward(xp, fh0, N) - y.cpu().numpy()) ** 2)
        lm = np.sum(np.abs(O.nfft_forward(xm, fh0, N) - y.cpu().numpy()) ** 2)
        fd = (lp - lm) / (2 * h)
        assert abs(fd - gx[j, t]) <= 1e-5 * max(1.0, abs(fd)), (j, t, fd, gx[j, t])
    plan.close()


def test_autograd_fp32_plan(dev):
    from cunfft_gb300.autograd import nfft

    rng = np.random.default_rng(1)
    N, M = [32, 32], 1000
    x = torch.from_numpy(rng.uniform(-0.5, 0.5, (M, 2))).to(dev).requires_grad_(True)
    fh = torch.from_numpy(rng.standard_normal(N) + 1j * rng.standard_normal(N)).to(dev, torch.complex64)
    fh.requires_grad_(True)
    out = nfft(x, fh)
    assert out.dtype == torch.complex64
    out.abs().pow(2).sum().backward()
    assert x.grad is not None and torch.isfinite(x.grad).all()
    assert fh.grad is not None and fh.grad.dtype == torch.complex64
