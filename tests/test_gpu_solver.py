"""Inverse NFFT (CG on the normal equations) over the GB300 forward/adjoint pair."""
import numpy as np
import pytest

import oracle as O

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("N,M,prec,tol", [([64], 512, "f64", 1e-5), ([32, 32], 4096, "f64", 1e-5),
                                          ([16, 16, 16], 20000, "f32", 1e-4)])
def test_cgne_recovers_coefficients(N, M, prec, tol):
    from cunfft_gb300.nfft import NFFT
    from cunfft_gb300.solver import cgne

    dev = torch.device("cuda:0")
    rng = np.random.default_rng(len(N) * 7 + M)
    x = rng.uniform(-0.5, 0.5, (M, len(N)))
    fh = rng.standard_normal(N) + 1j * rng.standard_normal(N)
    f = O.ndft_forward(x, fh, N)  # exact samples
    plan = NFFT(N, m=6, precision=prec, device=dev).set_nodes(torch.from_numpy(x).to(dev))
    sol, hist = cgne(plan, torch.from_numpy(f).to(dev), iters=60, tol=1e-9)
    assert hist[-1] < hist[0]
    err = np.linalg.norm(sol.cpu().numpy().astype(np.complex128) - fh) / np.linalg.norm(fh)
    assert err < tol, (err, hist[-5:])
    plan.close()


def _ndft_matrix(x, N):
    """Dense A[j, k] = exp(-2 pi i k . x_j), k over I_N row-major (last dim fastest)."""
    grids = np.meshgrid(*[np.arange(-(n // 2), n - n // 2) for n in N], indexing="ij")
    k = np.stack([g.reshape(-1) for g in grids], axis=1)
    return np.exp(-2j * np.pi * (x @ k.T))


def test_cgne_weighted_regularised_matches_dense_solve():
    """Underdetermined, clustered nodes with random weights and a Tikhonov term:
    the CG solution against numpy's dense solve of the same normal equations."""
    from cunfft_gb300.nfft import NFFT
    from cunfft_gb300.solver import cgne

    dev = torch.device("cuda:0")
    rng = np.random.default_rng(3)
    N, M, lam = [16, 16], 150, 5.0
    x = rng.normal(0, 0.15, (M, 2)).clip(-0.5, 0.4999)
    w = rng.uniform(0.5, 2.0, M)
    f = rng.standard_normal(M) + 1j * rng.standard_normal(M)
    A = _ndft_matrix(x, N)
    ref = np.linalg.solve(A.conj().T @ (w[:, None] * A) + lam * np.eye(A.shape[1]), A.conj().T @ (w * f))
    plan = NFFT(N, device=dev).set_nodes(torch.from_numpy(x).to(dev))
    sol, hist = cgne(plan, torch.from_numpy(f).to(dev), iters=300, weights=torch.from_numpy(w).to(dev),
                     lam=lam, tol=1e-12)
    assert hist[-1] < 1e-7, hist[-5:]
    err = np.linalg.norm(sol.cpu().numpy().reshape(-1) - ref) / np.linalg.norm(ref)
    assert err < 1e-5, err
    plan.close()
