"""ctypes binding of libcunfft.so (the in-tree GB300 library).

Loading fails loudly when the library has not been built: there is no CPU or
eager fallback for any transform.
"""
import ctypes
import os

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "libcunfft.so")

_lib = None

# --- status codes (include/cunfft_x.h) ---
SUCCESS = 0
INVALID_ARGUMENT = 1
ALLOC_FAILED = 2
CUFFT_ERROR = 3
CUDA_ERROR = 4
NODES_NOT_SET = 5
UNSUPPORTED = 6
DEVICE_CHECK_FAILED = 7

F64 = 0
F32 = 1


class CunfftError(RuntimeError):
    def __init__(self, status, message=""):
        self.status = status
        super().__init__(f"cunfft status {status} ({status_string(status)}): {message}")


# --- the drop-in ABI structs (include/cunfft_typedefs.h) ---
class NFFTTimeSpec(ctypes.Structure):
    _fields_ = [("runTime", ctypes.c_double), ("time_ROC", ctypes.c_double), ("time_CONV", ctypes.c_double),
                ("time_FFT", ctypes.c_double), ("time_COPY_IN", ctypes.c_double),
                ("time_COPY_OUT", ctypes.c_double), ("time_else", ctypes.c_double)]


class GpuComplex(ctypes.Structure):
    _fields_ = [("x", ctypes.c_double), ("y", ctypes.c_double)]


class KData(ctypes.Structure):
    _fields_ = [("N", ctypes.c_ssize_t * 3), ("n", ctypes.c_ssize_t * 3), ("b", ctypes.c_double * 3),
                ("bsqrt", ctypes.c_double * 3), ("fac", ctypes.c_double * 3), ("sigma", ctypes.c_double * 3)]


class CunfftPlan(ctypes.Structure):
    """Field-for-field mirror of cunfft_plan."""
    _fields_ = [
        ("N_total", ctypes.c_ssize_t), ("M_total", ctypes.c_ssize_t), ("d", ctypes.c_int),
        ("N", ctypes.POINTER(ctypes.c_ssize_t)), ("x", ctypes.POINTER(ctypes.c_double)),
        ("f_hat", ctypes.POINTER(GpuComplex)), ("f", ctypes.POINTER(GpuComplex)),
        ("sigma", ctypes.POINTER(ctypes.c_double)), ("n", ctypes.POINTER(ctypes.c_ssize_t)),
        ("n_total", ctypes.c_ssize_t), ("m", ctypes.c_int), ("b", ctypes.POINTER(ctypes.c_double)),
        ("g", ctypes.POINTER(GpuComplex)), ("g_hat", ctypes.POINTER(GpuComplex)),
        ("fg_exp_l_cpu", ctypes.POINTER(ctypes.c_double)),
        ("g_gpu", ctypes.c_void_p), ("fhat_gpu", ctypes.c_void_p), ("x_gpu", ctypes.c_void_p),
        ("f_gpu", ctypes.c_void_p), ("fft_forward", ctypes.c_int), ("fft_backward", ctypes.c_int),
        ("CUNFFTTimes", NFFTTimeSpec), ("flags", ctypes.c_uint),
    ]


CUFFT_INIT = 1 << 0
CUFFT_BOTH = 1 << 1
CUFFT_FORW = 1 << 2
CUFFT_BACKW = 1 << 3

# Every C symbol declared in include/cunfft.h, include/cunfft_x.h and include/cunfft_util.h.
ABI_SYMBOLS = [
    "warmUp_createPlan", "copyDataToDevice", "copyDataToDeviceAd", "copyDataToHost", "copyDataToHostAd",
    "copy_f_hat_ToHost", "copy_f_ToHost", "copy_g_ToHost", "copy_x_toHost", "cunfft_transform",
    "cunfft_adjoint", "cunfft_initPlan", "cunfft_freePlan", "cunfft_initDevicePara", "cunfft_init",
    "cunfft_initGuru", "cunfft_initHelp", "cunfft_reinit", "cunfft_reinitAd", "cunfft_finalize",
    "cunfft_finalizeDevice", "resetCUNFFTTimes", "cundft_transform", "cundft_adjoint", "nfft_init_fg_exp_l",
    "setProperties", "resetDevice", "cunfft_x_last_error", "cunfft_x_set_default_cutoff",
]
X_SYMBOLS = [
    "cunfft_x_plan_create", "cunfft_x_plan_destroy", "cunfft_x_set_nodes", "cunfft_x_forward",
    "cunfft_x_adjoint", "cunfft_x_forward_graph", "cunfft_x_adjoint_graph", "cunfft_x_ndft_forward", "cunfft_x_ndft_adjoint", "cunfft_x_ndft_adjoint_at",
    "cunfft_x_node_gradient",
    "cunfft_x_interp", "cunfft_x_spread", "cunfft_x_set_stream", "cunfft_x_get_stream", "cunfft_x_set_tiling",
    "cunfft_x_autotune", "cunfft_x_get_tiling", "cunfft_x_stage_times", "cunfft_x_synchronize",
    "cunfft_x_last_message", "cunfft_x_status_string", "cunfft_x_grid", "cunfft_x_version",
    "cunfft_x_spread_noalloc", "cunfft_x_set_spread_kernel", "cunfft_x_get_spread_kernel",
    "cunfft_x_set_window", "cunfft_x_get_window",
    "cunfft_x_set_interp_kernel", "cunfft_x_get_interp_kernel", "cunfft_x_forward_host", "cunfft_x_adjoint_host",
    "cunfft_x_check_wait_timeout",
]
UTIL_SYMBOLS = [
    "showTimes", "getGPUMemProps_ToStdout", "showCPUMemUse", "showCoeff_double", "showCoeff_cuComplex",
    "prod_int", "next_power_of_2", "createFourierCoeff_clustered", "createFourierCoeff_uniDistr",
    "createFourierCoeff_null", "getExampleData_clustered", "getExampleData_uniDistr",
    "getExampleDataAd_uniDistr", "getExampleData_null", "setExampleData", "l_infty", "compute_error_l_infty",
    "findDevice",
]


def lib():
    """Load libcunfft.so and declare its prototypes."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(f"{LIB_PATH} is missing: build it first "
                          "(python -c 'import __graft_entry__ as g; g.build()')")
    L = ctypes.CDLL(LIB_PATH)
    vp, i64p, dp = ctypes.c_void_p, ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_double)
    pp = ctypes.POINTER(ctypes.c_void_p)
    ip = ctypes.POINTER(ctypes.c_int)
    sig = {
        "cunfft_x_plan_create": (ctypes.c_int, [pp, ctypes.c_int, i64p, i64p, ctypes.c_int, ctypes.c_int,
                                                ctypes.c_int, vp]),
        "cunfft_x_plan_destroy": (ctypes.c_int, [vp]),
        "cunfft_x_set_nodes": (ctypes.c_int, [vp, vp, i64p]),
        "cunfft_x_forward": (ctypes.c_int, [vp, vp, vp]),
        "cunfft_x_adjoint": (ctypes.c_int, [vp, vp, vp]),
        "cunfft_x_forward_graph": (ctypes.c_int, [vp, vp, vp]),
        "cunfft_x_adjoint_graph": (ctypes.c_int, [vp, vp, vp]),
        "cunfft_x_spread_noalloc": (ctypes.c_int, [ctypes.c_int, i64p, i64p, ctypes.c_int, ctypes.c_int,
                                                   ctypes.c_int64, vp, vp, vp, vp, vp]),
        "cunfft_x_ndft_forward": (ctypes.c_int, [vp, vp, vp]),
        "cunfft_x_ndft_adjoint": (ctypes.c_int, [vp, vp, vp]),
        "cunfft_x_ndft_adjoint_at": (ctypes.c_int, [vp, vp, vp, ctypes.c_int64, vp]),
        "cunfft_x_node_gradient": (ctypes.c_int, [vp, vp, vp, vp]),
        "cunfft_x_interp": (ctypes.c_int, [vp, vp, vp]),
        "cunfft_x_spread": (ctypes.c_int, [vp, vp, vp]),
        "cunfft_x_set_stream": (ctypes.c_int, [vp, vp]),
        "cunfft_x_get_stream": (vp, [vp]),
        "cunfft_x_set_tiling": (ctypes.c_int, [vp, ip, ctypes.c_int]),
        "cunfft_x_autotune": (ctypes.c_int, [vp, ctypes.c_int]),
        "cunfft_x_get_tiling": (ctypes.c_int, [vp, ip, ip, ip]),
        "cunfft_x_set_spread_kernel": (ctypes.c_int, [vp, ctypes.c_int]),
        "cunfft_x_set_window": (ctypes.c_int, [vp, ctypes.c_int]),
        "cunfft_x_get_window": (ctypes.c_int, [vp, ip]),
        "cunfft_x_get_spread_kernel": (ctypes.c_int, [vp, ip]),
        "cunfft_x_set_interp_kernel": (ctypes.c_int, [vp, ctypes.c_int]),
        "cunfft_x_get_interp_kernel": (ctypes.c_int, [vp, ip]),
        "cunfft_x_forward_host": (ctypes.c_int, [vp, vp, i64p, vp, vp]),
        "cunfft_x_adjoint_host": (ctypes.c_int, [vp, vp, vp]),
        "cunfft_x_stage_times": (ctypes.c_int, [vp, dp, dp, dp, dp]),
        "cunfft_x_synchronize": (ctypes.c_int, [vp]),
        "cunfft_x_check_wait_timeout": (ctypes.c_int, [vp]),
        "cunfft_x_last_message": (ctypes.c_char_p, [vp]),
        "cunfft_x_status_string": (ctypes.c_char_p, [ctypes.c_int]),
        "cunfft_x_grid": (vp, [vp]),
        "cunfft_x_version": (ctypes.c_char_p, []),
        "cunfft_x_last_error": (ctypes.c_int, [ctypes.POINTER(CunfftPlan)]),
        "cunfft_x_set_default_cutoff": (ctypes.c_int, [ctypes.c_int]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    P = ctypes.POINTER(CunfftPlan)
    sp = ctypes.POINTER(ctypes.c_ssize_t)
    for name in ("copyDataToDevice", "copyDataToDeviceAd", "copyDataToHost", "copyDataToHostAd", "copy_g_ToHost",
                 "cunfft_transform", "cunfft_adjoint", "cunfft_freePlan", "cunfft_initDevicePara", "cunfft_initHelp",
                 "cunfft_reinit", "cunfft_reinitAd", "cunfft_finalize", "cunfft_finalizeDevice", "cundft_transform",
                 "cundft_adjoint", "getExampleData_uniDistr", "getExampleDataAd_uniDistr", "getExampleData_null",
                 "getExampleData_clustered", "showCPUMemUse"):
        getattr(L, name).restype = None
        getattr(L, name).argtypes = [P]
    L.copy_f_hat_ToHost.argtypes = [P, ctypes.POINTER(GpuComplex)]
    L.copy_f_ToHost.argtypes = [P, ctypes.POINTER(GpuComplex)]
    L.copy_x_toHost.argtypes = [P, dp]
    for name in ("copy_f_hat_ToHost", "copy_f_ToHost", "copy_x_toHost"):
        getattr(L, name).restype = None
    L.cunfft_init.argtypes = [P, ctypes.c_int, sp, ctypes.c_ssize_t]
    L.cunfft_init.restype = None
    L.cunfft_initGuru.argtypes = [P, ctypes.c_int, sp, ctypes.c_ssize_t, sp, ctypes.c_uint]
    L.cunfft_initGuru.restype = None
    L.cunfft_initPlan.argtypes = [ctypes.c_int, sp, ctypes.POINTER(ctypes.c_int)]
    L.cunfft_initPlan.restype = None
    L.warmUp_createPlan.argtypes = [sp]
    L.warmUp_createPlan.restype = None
    L.resetCUNFFTTimes.argtypes = [ctypes.POINTER(NFFTTimeSpec)]
    L.resetCUNFFTTimes.restype = None
    L.nfft_init_fg_exp_l.argtypes = [dp, ctypes.c_double, ctypes.c_int]
    L.nfft_init_fg_exp_l.restype = None
    L.setProperties.argtypes = [sp, sp, dp, dp, ctypes.c_int, ctypes.POINTER(KData)]
    L.setProperties.restype = None
    L.resetDevice.argtypes = []
    L.resetDevice.restype = None
    L.compute_error_l_infty.argtypes = [ctypes.POINTER(GpuComplex), ctypes.POINTER(GpuComplex), ctypes.c_int]
    L.compute_error_l_infty.restype = ctypes.c_double
    L.next_power_of_2.argtypes = [ctypes.c_ssize_t]
    L.next_power_of_2.restype = ctypes.c_ssize_t
    _lib = L
    return L


def status_string(s):
    try:
        return lib().cunfft_x_status_string(int(s)).decode()
    except Exception:  # pragma: no cover
        return "?"


def check(status, plan_handle=None):
    if status != SUCCESS:
        msg = ""
        if plan_handle:
            m = lib().cunfft_x_last_message(plan_handle)
            msg = m.decode() if m else ""
        raise CunfftError(status, msg)
