"""Host-buffer transforms (cunfft_x_forward_host / cunfft_x_adjoint_host): copies on
the plan's copy streams, overlapped with its kernels, give the device path's results."""
import numpy as np
import pytest

import oracle as O

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

TOL32 = 1e-5
TOL64 = 1e-12


@pytest.fixture(scope="module")
def dev():
    from cunfft_gb300 import _native
    _native.lib()
    return torch.device("cuda:0")


def _c(shape, rng, dtype):
    return torch.from_numpy(rng.uniform(-1, 1, shape) + 1j * rng.uniform(-1, 1, shape)).to(dtype)


@pytest.mark.parametrize("prec,tol", [("f32", TOL32), ("f64", TOL64)])
def test_host_path_back_to_back_rounds(dev, prec, tol):
    """Two forward/adjoint rounds with new nodes and inputs, issued without any wait in
    between, match the device path on the same inputs (and so the oracle)."""
    from cunfft_gb300.nfft import NFFT
    rng = np.random.default_rng(31)
    N, M = [16, 32, 32], 20000
    cd = torch.complex64 if prec == "f32" else torch.complex128
    p = NFFT(N, precision=prec, device=dev)
    rounds = []
    for r in range(2):
        x = torch.from_numpy(rng.uniform(-0.5, 0.5, (M, 3))).pin_memory()
        fh = _c(N, rng, cd).pin_memory()
        f = _c(M, rng, cd).pin_memory()
        out_f = torch.empty(M, dtype=cd).pin_memory()
        out_fh = torch.empty(N, dtype=cd).pin_memory()
        p.forward_host(fh, out_f, x=x)
        p.adjoint_host(f, out_fh)
        rounds.append((x, fh, f, out_f, out_fh))
    p.synchronize()
    ref = NFFT(N, precision=prec, device=dev)
    for x, fh, f, out_f, out_fh in rounds:
        ref.set_nodes(x.to(dev))
        rf = ref.forward(fh.to(dev)).cpu().numpy()
        rh = ref.adjoint(f.to(dev)).cpu().numpy()
        assert O.rel_l2(rf, out_f.numpy()) < tol
        assert O.rel_l2(rh, out_fh.numpy()) < tol
    xo, fho = rounds[1][0].numpy(), rounds[1][1].numpy().astype(np.complex128)
    assert O.rel_l2(O.nfft_forward(xo, fho, N), rounds[1][3].numpy()) < max(tol, 1e-12)
    p.close()
    ref.close()


def test_host_path_batched_uneven_f64(dev):
    from cunfft_gb300.nfft import NFFT
    rng = np.random.default_rng(32)
    N, Ms = [32, 32], [3000, 0, 517]
    M = sum(Ms)
    p = NFFT(N, precision="f64", batch=3, device=dev)
    x = torch.from_numpy(rng.uniform(-0.5, 0.5, (M, 2))).pin_memory()
    fh = _c([3] + N, rng, torch.complex128).pin_memory()
    f = _c(M, rng, torch.complex128).pin_memory()
    out_f = torch.empty(M, dtype=torch.complex128).pin_memory()
    out_fh = torch.empty([3] + N, dtype=torch.complex128).pin_memory()
    p.forward_host(fh, out_f, x=x, M_inst=Ms)
    p.adjoint_host(f, out_fh)
    p.synchronize()
    xs = np.split(x.numpy(), np.cumsum(Ms)[:-1])
    fs = np.split(f.numpy(), np.cumsum(Ms)[:-1])
    outs = np.split(out_f.numpy(), np.cumsum(Ms)[:-1])
    for i in range(3):
        if Ms[i]:
            assert O.rel_l2(O.nfft_forward(xs[i], fh[i].numpy(), N), outs[i]) < TOL64
            assert O.rel_l2(O.nfft_adjoint(xs[i], fs[i], N), out_fh[i].numpy()) < TOL64
        else:
            assert np.abs(out_fh[i].numpy()).max() == 0
    p.close()


def test_host_path_on_device_bound_nodes(dev):
    """x = None keeps nodes bound through the device API."""
    from cunfft_gb300.nfft import NFFT
    rng = np.random.default_rng(33)
    N, M = [16, 16, 16], 5000
    x = torch.from_numpy(rng.uniform(-0.5, 0.5, (M, 3))).to(dev)
    p = NFFT(N, precision="f32", device=dev).set_nodes(x)
    fh = _c(N, rng, torch.complex64).pin_memory()
    f = _c(M, rng, torch.complex64).pin_memory()
    out_f = torch.empty(M, dtype=torch.complex64).pin_memory()
    out_fh = torch.empty(N, dtype=torch.complex64).pin_memory()
    p.adjoint_host(f, out_fh)
    p.forward_host(fh, out_f)
    p.synchronize()
    assert O.rel_l2(p.forward(fh.to(dev)).cpu().numpy(), out_f.numpy()) < TOL32
    assert O.rel_l2(p.adjoint(f.to(dev)).cpu().numpy(), out_fh.numpy()) < TOL32
    p.close()


def test_host_path_errors(dev):
    from cunfft_gb300._native import CunfftError
    from cunfft_gb300.nfft import NFFT
    p = NFFT([16, 16], precision="f32", device=dev)
    f = torch.zeros(10, dtype=torch.complex64)
    with pytest.raises(ValueError):
        p.adjoint_host(f, torch.zeros(16 * 16, dtype=torch.complex64))  # no nodes: M = 0 != 10
    p.M = 10
    with pytest.raises(CunfftError):
        p.adjoint_host(f, torch.zeros([16, 16], dtype=torch.complex64))  # library: nodes not set
    with pytest.raises(ValueError):
        p.forward_host(torch.zeros([16, 16], dtype=torch.complex128), torch.zeros(10, dtype=torch.complex64))
    p.close()
