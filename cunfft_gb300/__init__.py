"""cunfft_gb300 -- GB300-native Gaussian-window NFFT (d = 1..3) behind CUNFFT's plan API.

The compute path is the in-tree CUDA library ``libcunfft.so`` (sm_103a):
  - ``cunfft_gb300.abi.ReferencePlan``: the reference's C plan API (cunfft.h);
  - ``cunfft_gb300.nfft.NFFT``: the extension API on torch CUDA tensors
    (runtime m, FP32 form, batched instances, streams);
  - ``cunfft_gb300.autograd.nfft``: differentiable forward transform.
There is no CPU fallback: importing a submodule that needs the library raises
when it has not been built.
"""
from ._native import CunfftError, lib  # noqa: F401

__all__ = ["CunfftError", "lib", "NFFT", "ReferencePlan", "nfft"]


def __getattr__(name):
    if name == "NFFT":
        from .nfft import NFFT
        return NFFT
    if name == "ReferencePlan":
        from .abi import ReferencePlan
        return ReferencePlan
    if name == "nfft":
        from .autograd import nfft
        return nfft
    raise AttributeError(name)
