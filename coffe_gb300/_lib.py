"""ctypes binding of ``libcoffe_gpu.so`` (the C ABI in ``include/coffe_gpu.h``).

The library is the only compute path: if it is missing or cannot be loaded the
import of this module raises, there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

from . import build as _build

STATUS = {
    0: "COFFE_GPU_OK",
    -1: "COFFE_GPU_EINVAL",
    -2: "COFFE_GPU_ECUDA",
    -3: "COFFE_GPU_ENOMEM",
    -4: "COFFE_GPU_ENONFINITE",
    -5: "COFFE_GPU_ESTATE",
    -6: "COFFE_GPU_ELIMIT",
}

FP64 = 0
MIXED = 1
FP64_FASTALG = 2
DEN = 1
RSD = 2
LEN = 4
ONLY_CROSS = 8
SMALL_R = 1
PK_DEVICE = 2
ASYNC = 4
TABLES_DF = 8
NOALLOC_MAX_OUTPUTS = 1048576
PEAK_FP64 = 0
PEAK_FP32 = 1
PEAK_FP32X2 = 2

# every symbol include/coffe_gpu.h declares
EXPORTS = (
    "coffe_gpu_ctx_create",
    "coffe_gpu_ctx_destroy",
    "coffe_gpu_strerror",
    "coffe_gpu_last_error",
    "coffe_gpu_synchronize",
    "coffe_gpu_set_stream",
    "coffe_gpu_background_init",
    "coffe_gpu_background_set",
    "coffe_gpu_background_get",
    "coffe_gpu_set_bias",
    "coffe_gpu_integral_table_len",
    "coffe_gpu_integrals_init",
    "coffe_gpu_integrals_init_ex",
    "coffe_gpu_integral_get",
    "coffe_gpu_integral_eval",
    "coffe_gpu_multipoles",
    "coffe_gpu_set_flatsky",
    "coffe_gpu_set_lensing_rule",
    "coffe_gpu_multipoles_async",
    "coffe_gpu_multipoles_noalloc",
    "coffe_gpu_corrfunc",
    "coffe_gpu_average_multipoles",
    "coffe_gpu_multipoles_retries",
    "coffe_gpu_multipoles_scaled",
    "coffe_gpu_multipoles_adjoint",
    "coffe_gpu_covariance_integrals",
    "coffe_gpu_covariance_multipoles",
    "coffe_gpu_average_covariance_multipoles",
    "coffe_gpu_set_autotune",
    "coffe_gpu_get_tuning",
    "coffe_gpu_set_tuning",
    "coffe_gpu_launch_count",
    "coffe_gpu_divergent_separations",
    "coffe_gpu_divergent_integral",
    "coffe_gpu_renormalization_grid",
    "coffe_gpu_measure_peak",
    "coffe_gpu_set_kernel_timing",
    "coffe_gpu_kernel_times",
    "coffe_gpu_debug_fail_alloc",
)


class Cosmology(C.Structure):
    _fields_ = [
        ("Omega0_cdm", C.c_double),
        ("Omega0_baryon", C.c_double),
        ("Omega0_gamma", C.c_double),
        ("Omega0_de", C.c_double),
        ("h", C.c_double),
        ("bins", C.c_int),
    ]


class Tuning(C.Structure):
    """coffe_gpu_tuning_t: launch shapes of the table stage and the mixed
    multipole kernel."""
    _fields_ = [
        ("fft_threads", C.c_int),
        ("fft_radix", C.c_int),
        ("fft_swizzle", C.c_int),
        ("spline_group", C.c_int),
        ("lane_threads", C.c_int),
        ("lane_unroll", C.c_int),
        ("fft_threads_fwd", C.c_int),
        ("lane_pack", C.c_int),
        ("fft_fused", C.c_int),
        ("lane_poly", C.c_int),
    ]


class CoffeGpuError(RuntimeError):
    def __init__(self, status: int, what: str, detail: str = ""):
        self.status = status
        super().__init__(f"{what}: {STATUS.get(status, status)} ({detail})")


_lib = None
_p = C.c_void_p
_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)
_lp = C.POINTER(C.c_int64)


def lib_path() -> Path:
    return _build.LIB


def load(build_if_missing: bool = True):
    """Load the library (building it first when it is absent)."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.LIB
    if not path.exists():
        if not build_if_missing:
            raise ImportError(f"{path} is missing: run python -m coffe_gb300.build")
        _build.build()
    L = C.CDLL(str(path))
    L.coffe_gpu_ctx_create.argtypes = [C.c_int, C.POINTER(_p)]
    L.coffe_gpu_ctx_destroy.argtypes = [_p]
    L.coffe_gpu_strerror.argtypes = [C.c_int]
    L.coffe_gpu_strerror.restype = C.c_char_p
    L.coffe_gpu_last_error.argtypes = [_p]
    L.coffe_gpu_last_error.restype = C.c_char_p
    L.coffe_gpu_synchronize.argtypes = [_p]
    L.coffe_gpu_set_stream.argtypes = [_p, _p]
    L.coffe_gpu_background_init.argtypes = [_p, C.POINTER(Cosmology)]
    L.coffe_gpu_background_set.argtypes = [_p, _dp, _dp, _dp, _dp, _dp, _dp, C.c_size_t,
                                           C.c_double, C.c_double]
    L.coffe_gpu_background_get.argtypes = [_p] + [_dp] * 8
    L.coffe_gpu_set_bias.argtypes = [_p, C.c_int, _dp, _dp, C.c_size_t]
    L.coffe_gpu_integral_table_len.argtypes = [C.c_size_t]
    L.coffe_gpu_integral_table_len.restype = C.c_size_t
    L.coffe_gpu_integrals_init.argtypes = [_p, _dp, _dp, C.c_int, C.c_size_t, _ip, _ip, C.c_int,
                                           C.c_size_t, C.c_int, C.c_uint]
    # the per-step entry points take raw addresses (void *): numpy's
    # .ctypes.data_as costs ~3 us per array, a noticeable share of a call
    L.coffe_gpu_integrals_init_ex.argtypes = [_p, _p, _p, C.c_int, C.c_size_t, _p, _p, _p,
                                              C.c_int, C.c_size_t, C.c_int, C.c_uint]
    L.coffe_gpu_set_flatsky.argtypes = [_p, C.c_int, C.c_int]
    L.coffe_gpu_integral_get.argtypes = [_p, C.c_int, C.c_int, _dp, _dp]
    L.coffe_gpu_integral_eval.argtypes = [_p, C.c_int, C.c_int, _dp, C.c_size_t, _dp]
    L.coffe_gpu_multipoles.argtypes = [_p, C.c_int, C.c_int, C.c_double, C.c_int, _p, _p, _p,
                                       _p, C.c_int, _p, _p, C.c_int]
    L.coffe_gpu_multipoles_async.argtypes = [_p, C.c_int, C.c_int, C.c_double, C.c_int,
                                             C.c_int64, _ip, _dp, _lp, _dp, C.c_int, _ip, _dp]
    L.coffe_gpu_set_lensing_rule.argtypes = [_p, C.c_int, C.c_int]
    L.coffe_gpu_multipoles_noalloc.argtypes = [_p, C.c_int, C.c_int, C.c_double, C.c_int,
                                               C.c_int64, _ip, _dp, _lp, _dp, C.c_int, _ip, _dp]
    L.coffe_gpu_multipoles_scaled.argtypes = [_p, C.c_int, C.c_int, C.c_int64, _ip, _dp, _lp, _dp,
                                              C.c_int, _ip, _dp, _dp, _dp]
    L.coffe_gpu_multipoles_adjoint.argtypes = [_p, C.c_int, C.c_int, C.c_int64, _ip, _dp, _lp,
                                               _dp, C.c_int, _ip, _dp, _dp, _dp, _dp, _dp, _dp]
    L.coffe_gpu_covariance_integrals.argtypes = [_p, _dp, _dp, C.c_size_t, C.c_size_t, C.c_int,
                                                 _ip, _ip, _ip, _dp, C.c_int, _dp]
    L.coffe_gpu_covariance_multipoles.argtypes = [_p, C.c_int, _dp, _dp, C.c_size_t, C.c_size_t,
                                                  C.c_int, _dp, _dp, _dp, _dp, _dp, _dp, C.c_int,
                                                  _ip, C.c_int, _dp, _dp]
    L.coffe_gpu_multipoles_retries.argtypes = [_p]
    L.coffe_gpu_multipoles_retries.restype = C.c_longlong
    L.coffe_gpu_corrfunc.argtypes = [_p, C.c_int, C.c_int, C.c_int, _ip, _dp, _lp, _dp,
                                     C.c_int, _dp, _dp, C.c_int]
    L.coffe_gpu_average_multipoles.argtypes = [_p, C.c_int, C.c_int, C.c_double, C.c_int, _ip,
                                               _dp, _dp, _lp, _dp, C.c_int, _ip, C.c_int, _dp,
                                               C.c_int]
    L.coffe_gpu_average_covariance_multipoles.argtypes = (
        L.coffe_gpu_covariance_multipoles.argtypes)
    L.coffe_gpu_set_autotune.argtypes = [_p, C.c_int]
    L.coffe_gpu_get_tuning.argtypes = [_p, C.POINTER(Tuning)]
    L.coffe_gpu_set_tuning.argtypes = [_p, C.POINTER(Tuning)]
    L.coffe_gpu_launch_count.argtypes = [_p]
    L.coffe_gpu_launch_count.restype = C.c_longlong
    L.coffe_gpu_divergent_separations.argtypes = [_dp, C.c_size_t]
    L.coffe_gpu_divergent_separations.restype = C.c_size_t
    L.coffe_gpu_divergent_integral.argtypes = [_p, _dp, _dp, C.c_size_t, C.c_double, C.c_double,
                                               _dp, C.c_size_t, _dp, _dp]
    L.coffe_gpu_renormalization_grid.argtypes = [_p, _dp, _dp, C.c_size_t, C.c_double,
                                                 C.c_double, _dp, C.c_size_t, _dp, C.c_size_t, _dp]
    L.coffe_gpu_measure_peak.argtypes = [_p, C.c_int, _dp]
    L.coffe_gpu_set_kernel_timing.argtypes = [_p, C.c_int]
    L.coffe_gpu_kernel_times.argtypes = [_p, C.POINTER(C.c_char_p), C.POINTER(C.c_longlong),
                                         _dp, C.c_int, C.c_int]
    L.coffe_gpu_debug_fail_alloc.argtypes = [_p, C.c_int]
    _lib = L
    return L
