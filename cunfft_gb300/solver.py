"""Inverse NFFT: reconstruct Fourier coefficients from nonuniform samples.

The reference's README promises "the nonequispaced fast Fourier transform and
its inversion" (README:1) but ships no solver.  This module adds one as a caller
of the GB300 forward/adjoint pair: conjugate gradients on the normal equations
of the first kind,

    min_fhat || W^(1/2) (A fhat - f) ||_2^2 + lam ||fhat||_2^2
    (A^H W A + lam I) fhat = A^H W f,

with optional sample weights W (e.g. density compensation) and Tikhonov term
lam.  Every iteration costs one forward and one adjoint NFFT on the plan's
nodes; the vector algebra runs as torch operations on the same stream.
"""
import torch


def cgne(plan, f, iters=20, weights=None, lam=0.0, fhat0=None, tol=0.0, callback=None):
    """Solve (A^H W A + lam I) fhat = A^H W f by conjugate gradients.

    plan: an ``NFFT`` with nodes bound; f: samples (M,) of the plan's dtype;
    weights: optional nonnegative (M,) real weights; returns (fhat, history),
    history the relative residual ||A^H W (f - A fhat) - lam fhat|| / ||A^H W f||
    per iteration.
    """
    cd = plan.cdtype
    f = f.to(cd)
    w = None if weights is None else weights.to(f.real.dtype)
    shape = plan._coef_shape()

    def normal_op(v):
        av = plan.forward(v)
        if w is not None:
            av = av * w
        out = plan.adjoint(av)
        if lam:
            out = out + lam * v
        return out

    b = plan.adjoint(f * w if w is not None else f)
    x = torch.zeros(shape, dtype=cd, device=f.device) if fhat0 is None else fhat0.to(cd).clone()
    r = b - normal_op(x) if fhat0 is not None else b.clone()
    p = r.clone()
    rr = torch.vdot(r.reshape(-1), r.reshape(-1)).real
    bnorm = torch.linalg.norm(b.reshape(-1))
    hist = []
    for _ in range(int(iters)):
        ap = normal_op(p)
        alpha = rr / torch.vdot(p.reshape(-1), ap.reshape(-1)).real
        x = x + alpha * p
        r = r - alpha * ap
        rr_new = torch.vdot(r.reshape(-1), r.reshape(-1)).real
        rel = (torch.sqrt(rr_new) / bnorm).item()
        hist.append(rel)
        if callback is not None:
            callback(x, rel)
        if rel <= tol:
            break
        p = r + (rr_new / rr) * p
        rr = rr_new
    return x, hist
