"""Python front end of the extension API (include/cunfft_x.h) for torch CUDA tensors.

``NFFT`` wraps one cunfft_x plan: d-variate NFFT (d = 1..3, Gaussian or ES window) in
FP64 (the reference's form) or FP32 (FP32 gridding and FFT, FP64 node
reduction and roll-off factors), for ``batch`` instances with uneven node
counts.  Tensors stay on the device; calls run on the plan's CUDA stream, which
defaults to torch's current stream so they order with surrounding torch work.

Layouts (as the reference): nodes ``x`` float64 (M, d) in [-0.5, 0.5);
coefficients (batch, *N) row-major with frequency k_t at index k_t + N_t//2;
samples (M,).
"""
import ctypes

import torch

from . import _native as nat


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None and t.numel() > 0 else ctypes.c_void_p(0)


class NFFT:
    def __init__(self, N, n=None, m=6, precision="f64", batch=1, device=None, stream=None, window="gaussian"):
        self._host_refs = []  # host tensors in flight in host-buffer transforms
        self._lib = nat.lib()
        self.N = [int(v) for v in N]
        self.d = len(self.N)
        if not 1 <= self.d <= 3:
            raise ValueError("d must be 1, 2 or 3")
        self.m = int(m)
        self.batch = int(batch)
        self.precision = {"f64": nat.F64, "f32": nat.F32, "float64": nat.F64, "float32": nat.F32}[precision]
        self.cdtype = torch.complex128 if self.precision == nat.F64 else torch.complex64
        self.device = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        with torch.cuda.device(self.device):
            if stream is None:
                stream = torch.cuda.current_stream(self.device)
            self.stream = stream
            Na = (ctypes.c_int64 * self.d)(*self.N)
            na = (ctypes.c_int64 * self.d)(*(n if n is not None else [0] * self.d))
            h = ctypes.c_void_p()
            st = self._lib.cunfft_x_plan_create(ctypes.byref(h), self.d, Na, na, self.m, self.precision,
                                                self.batch, ctypes.c_void_p(stream.cuda_stream))
            nat.check(st)
        self._h = h
        self.n = self._grid_sizes(n)
        self.N_total = 1
        for v in self.N:
            self.N_total *= v
        self.x = None
        self.M_inst = [0] * self.batch
        self.M = 0
        if window != "gaussian":
            self.set_window(window)

    def _grid_sizes(self, n):
        if n is not None:
            return [int(v) for v in n]
        out = []
        for v in self.N:
            p = 1
            while p < v:
                p <<= 1
            out.append(2 * p)
        return out

    # ------------------------------------------------------------------ nodes
    def set_nodes(self, x, M_inst=None):
        """Bind nodes: x float64 CUDA tensor (sum M_i, d); M_inst per-instance counts."""
        if x.dtype != torch.float64 or not x.is_cuda:
            raise TypeError("nodes must be a float64 CUDA tensor")
        x = x.contiguous().reshape(-1, self.d)
        M = x.shape[0]
        if M_inst is None:
            if self.batch != 1:
                raise ValueError("M_inst is required for batched plans")
            M_inst = [M]
        M_inst = [int(v) for v in M_inst]
        if len(M_inst) != self.batch or sum(M_inst) != M:
            raise ValueError("M_inst must have one count per instance summing to x.shape[0]")
        arr = (ctypes.c_int64 * self.batch)(*M_inst)
        nat.check(self._lib.cunfft_x_set_nodes(self._h, _ptr(x), arr), self._h)
        self.x = x  # keep the storage alive: the plan reads it
        self.M_inst = M_inst
        self.M = M
        return self

    # ------------------------------------------------------------ transforms
    def _coef(self, fhat):
        fhat = fhat.to(self.cdtype).contiguous()
        if fhat.numel() != self.batch * self.N_total:
            raise ValueError("f_hat has the wrong size")
        return fhat

    def _samples(self, f):
        f = f.to(self.cdtype).contiguous()
        if f.numel() != self.M:
            raise ValueError("f has the wrong size")
        return f

    def _coef_shape(self):
        return ([self.batch] if self.batch > 1 else []) + self.N

    def forward(self, fhat, out=None):
        fhat = self._coef(fhat)
        f = out if out is not None else torch.empty(self.M, dtype=self.cdtype, device=self.device)
        nat.check(self._lib.cunfft_x_forward(self._h, _ptr(fhat), _ptr(f)), self._h)
        return f

    def adjoint(self, f, out=None):
        f = self._samples(f)
        fh = out if out is not None else torch.empty(self._coef_shape(), dtype=self.cdtype, device=self.device)
        nat.check(self._lib.cunfft_x_adjoint(self._h, _ptr(f), _ptr(fh)), self._h)
        return fh

    # ------------------------------------------------ host buffers, overlapped copies
    def _host(self, t, dtype, numel, what):
        if t.is_cuda or t.dtype != dtype or not t.is_contiguous() or t.numel() != numel:
            raise ValueError(f"{what} must be a contiguous CPU {dtype} tensor of {numel} elements (pinned for overlap)")
        return t

    def forward_host(self, fhat, out, x=None, M_inst=None):
        """Forward transform between CPU tensors with the copies overlapped with the
        plan's kernels: x (float64, sum M_i x d; None keeps the bound nodes), fhat in,
        out (samples) written.  Asynchronous: keep the tensors alive and the inputs
        unchanged until synchronize(); pin them (tensor.pin_memory()) for overlap."""
        arr = None
        if x is not None:
            M = x.numel() // self.d
            self._host(x, torch.float64, M * self.d, "x")
            if M_inst is None:
                if self.batch != 1:
                    raise ValueError("M_inst is required for batched plans")
                M_inst = [M]
            M_inst = [int(v) for v in M_inst]
            if len(M_inst) != self.batch or sum(M_inst) != M:
                raise ValueError("M_inst must have one count per instance summing to the node count")
            arr = (ctypes.c_int64 * self.batch)(*M_inst)
            self.M_inst, self.M, self.x = M_inst, M, None
        self._host(fhat, self.cdtype, self.batch * self.N_total, "fhat")
        self._host(out, self.cdtype, self.M, "out")
        nat.check(self._lib.cunfft_x_forward_host(self._h, _ptr(x), arr, _ptr(fhat), _ptr(out)), self._h)
        self._host_refs.extend([x, fhat, out])
        return out

    def adjoint_host(self, f, out):
        """Adjoint between CPU tensors on the bound nodes (see forward_host)."""
        self._host(f, self.cdtype, self.M, "f")
        self._host(out, self.cdtype, self.batch * self.N_total, "out")
        nat.check(self._lib.cunfft_x_adjoint_host(self._h, _ptr(f), _ptr(out)), self._h)
        self._host_refs.extend([f, out])
        return out

    def forward_graph(self, fhat, out):
        """forward() replayed from a captured CUDA graph (fixed buffers fhat, out)."""
        fhat = self._coef(fhat)
        nat.check(self._lib.cunfft_x_forward_graph(self._h, _ptr(fhat), _ptr(out)), self._h)
        return out

    def adjoint_graph(self, f, out):
        """adjoint() replayed from a captured CUDA graph (fixed buffers f, out)."""
        f = self._samples(f)
        nat.check(self._lib.cunfft_x_adjoint_graph(self._h, _ptr(f), _ptr(out)), self._h)
        return out

    def ndft_forward(self, fhat):
        fhat = fhat.to(torch.complex128).contiguous()
        f = torch.empty(self.M, dtype=torch.complex128, device=self.device)
        nat.check(self._lib.cunfft_x_ndft_forward(self._h, _ptr(fhat), _ptr(f)), self._h)
        return f

    def ndft_adjoint(self, f):
        f = f.to(torch.complex128).contiguous()
        fh = torch.empty(self._coef_shape(), dtype=torch.complex128, device=self.device)
        nat.check(self._lib.cunfft_x_ndft_adjoint(self._h, _ptr(f), _ptr(fh)), self._h)
        return fh

    def ndft_adjoint_at(self, f, kidx):
        """Adjoint NDFT at the row-major coefficient indices kidx (int64 CUDA tensor)."""
        f = f.to(torch.complex128).contiguous()
        kidx = kidx.to(device=self.device, dtype=torch.int64).contiguous()
        out = torch.empty(self.batch * kidx.numel(), dtype=torch.complex128, device=self.device)
        nat.check(self._lib.cunfft_x_ndft_adjoint_at(self._h, _ptr(f), _ptr(kidx), kidx.numel(), _ptr(out)),
                  self._h)
        return out

    def node_gradient(self, fhat, grad_f):
        fhat = self._coef(fhat)
        grad_f = self._samples(grad_f)
        gx = torch.empty(self.M, self.d, dtype=torch.float64, device=self.device)
        nat.check(self._lib.cunfft_x_node_gradient(self._h, _ptr(fhat), _ptr(grad_f), _ptr(gx)), self._h)
        return gx

    def interp(self, g, out=None):
        g = g.to(self.cdtype).contiguous()
        f = out if out is not None else torch.empty(self.M, dtype=self.cdtype, device=self.device)
        nat.check(self._lib.cunfft_x_interp(self._h, _ptr(g), _ptr(f)), self._h)
        return f

    def spread(self, f, g=None):
        f = self._samples(f)
        if g is None:
            g = torch.zeros(([self.batch] if self.batch > 1 else []) + self.n, dtype=self.cdtype, device=self.device)
        nat.check(self._lib.cunfft_x_spread(self._h, _ptr(f), _ptr(g)), self._h)
        return g

    # ---------------------------------------------------------------- tuning
    def set_tiling(self, T=None, chunk=0):
        arr = (ctypes.c_int * 3)(*((list(T) + [0, 0, 0])[:3] if T else [0, 0, 0]))
        nat.check(self._lib.cunfft_x_set_tiling(self._h, arr, int(chunk)), self._h)

    def tiling(self):
        T = (ctypes.c_int * 3)()
        chunk, threads = ctypes.c_int(), ctypes.c_int()
        nat.check(self._lib.cunfft_x_get_tiling(self._h, T, ctypes.byref(chunk), ctypes.byref(threads)))
        return {"T": list(T)[: self.d], "chunk": chunk.value, "threads": threads.value, "spread": self.spread_kernel(),
                "interp": self.interp_kernel()}

    WINDOWS = {"gaussian": 0, "es": 1}

    def set_window(self, window):
        """Gridding window: "gaussian" (the reference's) or "es" (exponential of
        semicircle, about 1e-12 relative error at m = 6, sigma = 2)."""
        nat.check(self._lib.cunfft_x_set_window(self._h, self.WINDOWS[window]), self._h)
        return self

    def window(self):
        k = ctypes.c_int()
        nat.check(self._lib.cunfft_x_get_window(self._h, ctypes.byref(k)))
        return {v: n for n, v in self.WINDOWS.items()}[k.value]

    SPREAD_KERNELS = {"auto": 0, "shared": 1, "register": 2, "global": 3, "tensor": 4}

    def set_spread_kernel(self, kind="auto"):
        """Request the spreading kernel: "auto", "shared", "register" or "tensor"."""
        nat.check(self._lib.cunfft_x_set_spread_kernel(self._h, self.SPREAD_KERNELS[kind]), self._h)

    def spread_kernel(self):
        """Spreading kernel in use: "shared", "register", "tensor" or "global"."""
        k = ctypes.c_int()
        nat.check(self._lib.cunfft_x_get_spread_kernel(self._h, ctypes.byref(k)))
        return {v: n for n, v in self.SPREAD_KERNELS.items()}[k.value]

    INTERP_KERNELS = {"auto": 0, "shared": 1, "global": 3, "tensor": 4}

    def set_interp_kernel(self, kind="auto"):
        """Request the interpolation kernel: "auto", "shared" or "tensor"."""
        nat.check(self._lib.cunfft_x_set_interp_kernel(self._h, self.INTERP_KERNELS[kind]), self._h)

    def interp_kernel(self):
        """Interpolation kernel in use: "shared", "tensor" or "global"."""
        k = ctypes.c_int()
        nat.check(self._lib.cunfft_x_get_interp_kernel(self._h, ctypes.byref(k)))
        return {v: n for n, v in self.INTERP_KERNELS.items()}[k.value]

    def autotune(self, reps=3):
        nat.check(self._lib.cunfft_x_autotune(self._h, int(reps)), self._h)
        return self.tiling()

    def stage_times(self):
        v = [ctypes.c_double() for _ in range(4)]
        nat.check(self._lib.cunfft_x_stage_times(self._h, *[ctypes.byref(a) for a in v]), self._h)
        return dict(zip(("bin", "roc", "fft", "conv"), (a.value for a in v)))

    def check_wait_timeout(self):
        """Run a kernel whose bounded completion wait gives up (about 1 ms): the next
        synchronize() raises CunfftError with CUNFFT_X_DEVICE_CHECK_FAILED."""
        nat.check(self._lib.cunfft_x_check_wait_timeout(self._h), self._h)

    def synchronize(self):
        nat.check(self._lib.cunfft_x_synchronize(self._h), self._h)
        self._host_refs = []  # host buffers of finished host-buffer transforms

    def grid(self):
        """The plan's oversampled grid as a tensor view (batch, *n)."""
        ptr = self._lib.cunfft_x_grid(self._h)
        numel = self.batch
        for v in self.n:
            numel *= v
        return _wrap_device_pointer(ptr, numel, self.cdtype, self.device).reshape(
            ([self.batch] if self.batch > 1 else []) + self.n)

    def close(self):
        if getattr(self, "_h", None):
            self._lib.cunfft_x_plan_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _wrap_device_pointer(ptr, numel, dtype, device):
    """A tensor that aliases device memory owned by the library (no copy)."""
    class _CudaArray:
        def __init__(self, p, nbytes):
            self.__cuda_array_interface__ = {"shape": (nbytes,), "typestr": "|u1", "data": (p, False),
                                             "version": 3}
    itemsize = torch.empty((), dtype=dtype).element_size()
    raw = torch.as_tensor(_CudaArray(ptr, numel * itemsize), device=device)
    return raw.view(dtype)
