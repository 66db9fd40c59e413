"""Differentiable NFFT: torch.autograd.Function over the GB300 kernels.

forward:  f = A(x) f_hat        (NFFT, cunfft_x_forward)
backward: grad_f_hat = A(x)^H grad_f          (adjoint NFFT, cunfft_x_adjoint)
          grad_x[j, t] = Re(conj(grad_f_j) d f_j / d x_{j,t})
                        (derivative-of-Gaussian gridding, cunfft_x_node_gradient)
These are PyTorch's conventions for a C-linear map of complex f_hat and a
real-valued node tensor.  The reference has no differentiable transform.
"""
import torch

from .nfft import NFFT


class NFFTFunction(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x, fhat, plan):
        plan.set_nodes(x.detach())
        f = plan.forward(fhat.detach())
        ctx.save_for_backward(x, fhat)
        ctx.plan = plan
        return f

    @staticmethod
    def backward(ctx, grad_f):
        x, fhat = ctx.saved_tensors
        plan = ctx.plan
        if plan.x is None or plan.x.data_ptr() != x.data_ptr():
            plan.set_nodes(x.detach())
        grad_f = grad_f.contiguous()
        gx = gfh = None
        if ctx.needs_input_grad[1]:
            gfh = plan.adjoint(grad_f).reshape(fhat.shape).to(fhat.dtype)
        if ctx.needs_input_grad[0]:
            gx = plan.node_gradient(fhat.detach(), grad_f).reshape(x.shape)
        return gx, gfh, None


def nfft(x, fhat, N=None, m=6, precision=None, plan=None):
    """f = A(x) f_hat with autograd support for x and f_hat."""
    if plan is None:
        N = list(fhat.shape) if N is None else list(N)
        if precision is None:
            precision = "f64" if fhat.dtype == torch.complex128 else "f32"
        plan = NFFT(N, m=m, precision=precision, device=fhat.device)
    return NFFTFunction.apply(x, fhat, plan)
