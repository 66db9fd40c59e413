"""Parity cases at the benchmark configurations other than the headline 3D one.

1. 2D N=64^2, n=128^2, m=6, M=4096 uniform nodes (FP64), against the CPU direct NDFT.
3. 2D clustered nodes, N=512^2, n=1024^2, m=6: 512 radial spokes x 1024 samples plus
   2^18 Gaussian (std 0.02) nodes at the origin; FP64 against the oracle NFFT, FP32
   against the FP64 result, both against the FP64 NDFT on subsamples.
4. Batched 2D adjoint + forward, 64 instances, N=256^2, n=512^2, m=5, per-instance
   M log-uniform in [1e3, 1e6], FP32, replayed from captured CUDA graphs; error
   against the FP64 NDFT on 2048 nodes / 2048 coefficients per instance.
5. Differentiable 2D NFFT, N=256^2, m=6, M=2^18 float64 nodes: gradients of
   ||A(x) f_hat - y||^2 against finite differences (h = 1e-6) and the FP64 NDFT.
Inputs are seeded synthetic data with the configurations' shapes and distributions.
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


def _crand(shape, rng):
    return rng.uniform(-1, 1, shape) + 1j * rng.uniform(-1, 1, shape)


def _rel(ref, got):
    ref = torch.as_tensor(ref).to(torch.complex128).reshape(-1)
    got = torch.as_tensor(got).to(ref.device, torch.complex128).reshape(-1)
    return (torch.linalg.norm(ref - got) / torch.linalg.norm(ref)).item()


def test_config1_2d_small_against_cpu_ndft(dev):
    from cunfft_gb300.nfft import NFFT

    rng = np.random.default_rng(101)
    N, M = [64, 64], 4096
    x = rng.uniform(-0.5, 0.5, (M, 2))
    fh, f = _crand(N, rng), _crand(M, rng)
    p = NFFT(N, m=6, device=dev).set_nodes(torch.from_numpy(x).to(dev))
    got_f = p.forward(torch.from_numpy(fh).to(dev)).cpu().numpy()
    got_fh = p.adjoint(torch.from_numpy(f).to(dev)).cpu().numpy()
    assert O.rel_l2(O.nfft_forward(x, fh, N), got_f) < 1e-12
    assert O.rel_l2(O.nfft_adjoint(x, f, N), got_fh) < 1e-12
    e_f = O.rel_l2(O.ndft_forward(x, fh, N), got_f)
    e_a = O.rel_l2(O.ndft_adjoint(x, f, N), got_fh)
    assert e_f < 5e-6 and e_a < 5e-6, (e_f, e_a)  # the Gaussian window at m = 6 (~1e-6)
    p.close()


def _clustered_nodes(rng):
    spokes, samples = 512, 1024
    theta = np.pi * np.arange(spokes) / spokes
    r = -0.5 + np.arange(samples) / samples
    rad = np.stack([np.outer(np.cos(theta), r).ravel(), np.outer(np.sin(theta), r).ravel()], axis=1)
    g = rng.normal(0.0, 0.02, (1 << 18, 2))
    g = np.mod(g + 0.5, 1.0) - 0.5
    return np.concatenate([rad, g])


def test_config3_clustered_2d(dev):
    from cunfft_gb300.nfft import NFFT

    rng = np.random.default_rng(303)
    N = [512, 512]
    x = _clustered_nodes(rng)
    M = x.shape[0]
    assert M == 786432
    fh, f = _crand(N, rng), _crand(M, rng)
    xt = torch.from_numpy(x).to(dev)
    p64 = NFFT(N, m=6, device=dev).set_nodes(xt)
    f64 = p64.forward(torch.from_numpy(fh).to(dev))
    fh64 = p64.adjoint(torch.from_numpy(f).to(dev))
    assert _rel(O.nfft_forward(x, fh, N), f64.cpu()) < 1e-12
    assert _rel(O.nfft_adjoint(x, f, N), fh64.cpu()) < 1e-12
    p32 = NFFT(N, m=6, precision="f32", device=dev).set_nodes(xt)
    f32 = p32.forward(torch.from_numpy(fh).to(dev))
    fh32 = p32.adjoint(torch.from_numpy(f).to(dev))
    # the FP32 form against the FP64 form on identical inputs: the FP32 gridding's own error
    # (measured 3.6e-7 forward, 9.1e-7 adjoint), below the window's ~1e-6 against the NDFT
    assert _rel(f64, f32) < 2e-6 and _rel(fh64, fh32) < 2e-6
    # FP64 NDFT on subsamples: 2048 nodes (forward), 2048 coefficients (adjoint)
    idx = torch.from_numpy(rng.choice(M, 2048, replace=False)).to(dev)
    sub = NFFT(N, m=6, device=dev).set_nodes(xt[idx].contiguous())
    nd = sub.ndft_forward(torch.from_numpy(fh).to(dev))
    assert _rel(nd, f32[idx]) < 1e-5
    kidx = torch.from_numpy(rng.choice(N[0] * N[1], 2048, replace=False)).to(dev)
    nda = p64.ndft_adjoint_at(torch.from_numpy(f).to(dev), kidx)
    assert _rel(nda, fh32.reshape(-1)[kidx]) < 1e-5
    for p in (p64, p32, sub):
        p.close()


def test_config4_batched_uneven_graph(dev):
    from cunfft_gb300.nfft import NFFT

    rng = np.random.default_rng(404)
    B, N, m = 64, [256, 256], 5
    Ms = np.round(10 ** rng.uniform(3, 6, B)).astype(np.int64)
    xs = [rng.uniform(-0.5, 0.5, (int(k), 2)) for k in Ms]
    x = torch.from_numpy(np.concatenate(xs)).to(dev)
    fh = torch.from_numpy(_crand([B] + N, rng)).to(dev)
    f = torch.from_numpy(_crand(int(Ms.sum()), rng)).to(dev)
    stream = torch.cuda.Stream(dev)  # a capturable (non-default) stream
    stream.wait_stream(torch.cuda.current_stream(dev))
    with torch.cuda.stream(stream):
        p = NFFT(N, m=m, precision="f32", batch=B, device=dev).set_nodes(x, Ms.tolist())
        fh32, f32 = fh.to(torch.complex64), f.to(torch.complex64)
        out_f = torch.empty(int(Ms.sum()), dtype=torch.complex64, device=dev)
        out_fh = torch.empty([B] + N, dtype=torch.complex64, device=dev)
        p.adjoint_graph(f32, out_fh)      # captures
        p.forward_graph(fh32, out_f)      # captures
        ref_fh = p.adjoint(f32).clone()
        ref_f = p.forward(fh32).clone()
        out_fh.zero_()
        out_f.zero_()
        p.adjoint_graph(f32, out_fh)      # replays
        p.forward_graph(fh32, out_f)      # replays
    stream.synchronize()
    assert _rel(ref_fh, out_fh) < 1e-6 and _rel(ref_f, out_f) < 1e-6
    # FP64 NDFT: 2048 nodes per instance (forward), 2048 coefficients per instance (adjoint)
    sub_idx, off = [], 0
    for k in Ms:
        sub_idx.append(off + rng.choice(int(k), min(2048, int(k)), replace=False))
        off += int(k)
    sub_counts = [len(s) for s in sub_idx]
    sidx = torch.from_numpy(np.concatenate(sub_idx)).to(dev)
    sub = NFFT(N, m=m, batch=B, device=dev).set_nodes(x[sidx].contiguous(), sub_counts)
    nd_f = sub.ndft_forward(fh)
    assert _rel(nd_f, out_f[sidx]) < 1e-5
    full = NFFT(N, m=m, batch=B, device=dev).set_nodes(x, Ms.tolist())
    kidx = torch.from_numpy(rng.choice(N[0] * N[1], 2048, replace=False)).to(dev)
    nd_h = full.ndft_adjoint_at(f, kidx).reshape(B, -1)
    got_h = out_fh.reshape(B, -1)[:, kidx]
    assert _rel(nd_h, got_h) < 1e-5
    # the FP32 replay against the FP64 form on the same instances (measured 2.8e-7 forward,
    # 6.3e-7 adjoint)
    assert _rel(full.forward(fh), out_f) < 2e-6
    assert _rel(full.adjoint(f), out_fh) < 2e-6
    for q in (p, sub, full):
        q.close()


def test_config5_autograd_2d(dev):
    from cunfft_gb300.autograd import NFFTFunction
    from cunfft_gb300.nfft import NFFT

    rng = np.random.default_rng(505)
    N, M, m = [256, 256], 1 << 18, 6
    x0 = rng.uniform(-0.5, 0.5, (M, 2))
    fh0 = (rng.standard_normal(N) + 1j * rng.standard_normal(N)) / np.sqrt(2)
    xpert = np.mod(x0 + rng.normal(0, 1e-3, x0.shape) + 0.5, 1.0) - 0.5
    fhd = torch.from_numpy(fh0).to(dev)
    y = NFFT(N, m=m, device=dev).set_nodes(torch.from_numpy(xpert).to(dev)).forward(fhd)
    plan = NFFT(N, m=m, device=dev)
    x = torch.from_numpy(x0).to(dev).requires_grad_(True)
    fh = fhd.clone().requires_grad_(True)
    loss = (NFFTFunction.apply(x, fh, plan) - y).abs().pow(2).sum()
    loss.backward()
    with torch.no_grad():
        r = plan.set_nodes(x.detach()).forward(fhd) - y
        g_fh = plan.adjoint(2 * r)
    assert _rel(g_fh, fh.grad) < 1e-12
    # node gradient: central differences of the loss (only node j's term changes)
    one = NFFT(N, m=m, device=dev)
    gx = x.grad.cpu().numpy()
    for j, t in [(0, 0), (777, 1), (123456, 0), (M - 1, 1)]:
        vals = []
        for s in (+1, -1):
            xj = x0[j:j + 1].copy()
            xj[0, t] += s * 1e-6
            fj = one.set_nodes(torch.from_numpy(xj).to(dev)).forward(fhd)
            vals.append((fj - y[j]).abs().pow(2).sum().item())
        fd = (vals[0] - vals[1]) / 2e-6
        assert abs(fd - gx[j, t]) <= 1e-5 * max(1.0, abs(fd)), (j, t, fd, gx[j, t])
    # against the FP64 NDFT gradient on 512 nodes: Re(conj(2 r_j) * sum_k (-2 pi i k_t) f_hat_k e^{-2 pi i k x_j})
    idx = rng.choice(M, 512, replace=False)
    sub = NFFT(N, m=m, device=dev).set_nodes(torch.from_numpy(x0[idx]).to(dev))
    k = [torch.arange(-(n // 2), n - n // 2, device=dev, dtype=torch.float64) for n in N]
    kk = torch.meshgrid(*k, indexing="ij")
    ref = np.zeros((512, 2))
    rj = r[torch.from_numpy(idx).to(dev)]
    for t in range(2):
        dfh = (-2j * np.pi) * kk[t] * fhd
        df = sub.ndft_forward(dfh)
        ref[:, t] = (torch.conj(2 * rj) * df).real.cpu().numpy()
    got = gx[idx]
    assert np.linalg.norm(got - ref) / np.linalg.norm(ref) < 1e-4
    for q in (plan, one, sub):
        q.close()
