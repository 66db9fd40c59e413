"""Python mirror of the reference's plan API, bound to the drop-in C ABI.

``ReferencePlan`` drives libcunfft.so exactly as a reference program drives
CUNFFT (src/simpleTest.cpp, Tests/Scripts/simpleTest.cpp): cunfft_init, write
plan.x / plan.f_hat on the host, copyDataToDevice, cunfft_transform,
copyDataToHost, cunfft_finalize.  The host arrays are numpy views of the
plan's pinned buffers.
"""
import ctypes

import numpy as np

from . import _native as nat


class ReferencePlan:
    def __init__(self, N, M, n=None, flags=None, m=None):
        self.lib = nat.lib()
        self.plan = nat.CunfftPlan()
        self.ref = ctypes.byref(self.plan)
        d = len(N)
        Na = (ctypes.c_ssize_t * d)(*[int(v) for v in N])
        if m is not None:
            nat.check(self.lib.cunfft_x_set_default_cutoff(int(m)))
        try:
            if n is None and flags is None:
                self.lib.cunfft_init(self.ref, d, Na, int(M))
            else:
                if n is None:
                    n = [2 * int(self.lib.next_power_of_2(int(v))) for v in N]
                na = (ctypes.c_ssize_t * d)(*[int(v) for v in n])
                fl = nat.CUFFT_INIT | nat.CUFFT_BOTH if flags is None else int(flags)
                self.lib.cunfft_initGuru(self.ref, d, Na, int(M), na, fl)
        finally:
            if m is not None:
                self.lib.cunfft_x_set_default_cutoff(6)
        self.status()
        self.d = d
        self.closed = False

    # host views over the plan's pinned arrays
    def _cview(self, ptr, count):
        if count == 0:
            return np.zeros(0, dtype=np.complex128)
        buf = (ctypes.c_double * (2 * count)).from_address(ctypes.addressof(ptr.contents))
        return np.frombuffer(buf, dtype=np.complex128, count=count)

    @property
    def x(self):
        cnt = self.plan.M_total * self.plan.d
        if cnt == 0:
            return np.zeros((0, self.plan.d))
        buf = (ctypes.c_double * cnt).from_address(ctypes.addressof(self.plan.x.contents))
        return np.frombuffer(buf, dtype=np.float64, count=cnt).reshape(self.plan.M_total, self.plan.d)

    @property
    def f_hat(self):
        return self._cview(self.plan.f_hat, self.plan.N_total)

    @property
    def f(self):
        return self._cview(self.plan.f, self.plan.M_total)

    @property
    def g(self):
        return self._cview(self.plan.g, self.plan.n_total)

    @property
    def times(self):
        t = self.plan.CUNFFTTimes
        return {k: getattr(t, k) for k, _ in nat.NFFTTimeSpec._fields_}

    def status(self):
        return self.lib.cunfft_x_last_error(self.ref)

    def check(self):
        s = self.status()
        if s != nat.SUCCESS:
            raise nat.CunfftError(s, "plan API call failed")

    # reference API, one method per entry point
    def copyDataToDevice(self):
        self.lib.copyDataToDevice(self.ref)

    def copyDataToDeviceAd(self):
        self.lib.copyDataToDeviceAd(self.ref)

    def copyDataToHost(self):
        self.lib.copyDataToHost(self.ref)

    def copyDataToHostAd(self):
        self.lib.copyDataToHostAd(self.ref)

    def copy_f_ToHost(self):
        out = np.zeros(self.plan.M_total, dtype=np.complex128)
        self.lib.copy_f_ToHost(self.ref, out.ctypes.data_as(ctypes.POINTER(nat.GpuComplex)))
        return out

    def copy_f_hat_ToHost(self):
        out = np.zeros(self.plan.N_total, dtype=np.complex128)
        self.lib.copy_f_hat_ToHost(self.ref, out.ctypes.data_as(ctypes.POINTER(nat.GpuComplex)))
        return out

    def copy_x_toHost(self):
        out = np.zeros(self.plan.M_total * self.plan.d, dtype=np.float64)
        self.lib.copy_x_toHost(self.ref, out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
        return out.reshape(self.plan.M_total, self.plan.d)

    def copy_g_ToHost(self):
        self.lib.copy_g_ToHost(self.ref)

    def cunfft_transform(self):
        self.lib.cunfft_transform(self.ref)

    def cunfft_adjoint(self):
        self.lib.cunfft_adjoint(self.ref)

    def cundft_transform(self):
        self.lib.cundft_transform(self.ref)

    def cundft_adjoint(self):
        self.lib.cundft_adjoint(self.ref)

    def cunfft_reinit(self):
        self.lib.cunfft_reinit(self.ref)

    def cunfft_reinitAd(self):
        self.lib.cunfft_reinitAd(self.ref)

    def getExampleData_uniDistr(self):
        self.lib.getExampleData_uniDistr(self.ref)

    def getExampleDataAd_uniDistr(self):
        self.lib.getExampleDataAd_uniDistr(self.ref)

    def cunfft_finalize(self):
        if not self.closed:
            self.lib.cunfft_finalize(self.ref)
            self.closed = True

    def __del__(self):
        try:
            self.cunfft_finalize()
        except Exception:
            pass
