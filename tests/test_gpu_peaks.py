"""The measured arithmetic rates that bench.py divides the compute-bound kernels'
FLOP/s by (coffe_gpu_measure_peak): positive, and ordered as the hardware is
(FP32 well above FP64 on a GB300)."""
import pytest

pytestmark = pytest.mark.gpu


def test_measured_peaks_are_sane(gpu_ctx):
    p64 = gpu_ctx.measure_peak("fp64")
    p32 = gpu_ctx.measure_peak("fp32")
    p2 = gpu_ctx.measure_peak("fp32x2")
    print(f"FP64 {p64 / 1e12:.3f} TFLOP/s, FP32 {p32 / 1e12:.2f}, FP32x2 {p2 / 1e12:.2f}")
    assert 0 < p64 < p32
    assert p32 > 8 * p64
    assert p2 > 0.5 * p32


def test_measure_peak_rejects_unknown_kind(gpu_ctx):
    from coffe_gb300.api import CoffeGpuError

    with pytest.raises(KeyError):
        gpu_ctx.measure_peak("int8")
    import ctypes as C

    v = C.c_double()
    assert gpu_ctx._L.coffe_gpu_measure_peak(gpu_ctx._ctx, 7, C.byref(v)) == -1
