"""Host-side instrumentation and failure injection through the C ABI:
per-kernel CUDA-event timing (coffe_gpu_set_kernel_timing /
coffe_gpu_kernel_times) and an injected device-allocation failure
(coffe_gpu_debug_fail_alloc), which must surface as COFFE_GPU_ENOMEM from the
call that needed the memory and leave the context usable.  Nothing here faults
or hangs the GPU: the failure is made on the host, in place of cudaMalloc."""
import numpy as np
import pytest

from conftest import H

pytestmark = pytest.mark.gpu


@pytest.fixture()
def fresh_ctx():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from coffe_gb300.api import Context

    ctx = Context(0)
    yield ctx
    ctx.close()


def test_kernel_timing_names_the_launched_kernels(fresh_ctx):
    from coffe_gb300 import workloads

    b = workloads.subset(workloads.cfg3(n_spectra=4), 4)
    ctx = fresh_ctx
    ctx.background_init(0.31, 0.05, 9e-5, H, 10000)
    ctx.set_kernel_timing(True)
    ctx.integrals_init(b.k, b.pk, [(0, 0), (0, 2), (0, 4)], N=4096, precision="mixed",
                       small_r=False)
    ctx.multipoles(b.req_spectrum, b.req_z_mean, b.req_offset, b.sep, b.ls, precision="mixed")
    t = ctx.kernel_times()
    print(t)
    tables = (("fftlog_tables_fused_kernel",) if ctx.tuning()["fft_fused"] else
              ("fftlog_forward_df_kernel", "fftlog_inverse_f32_kernel"))
    lanes = ("mp_poly_kernel",) if ctx.tuning()["lane_poly"] else ("mp_fast_kernel",)
    for name in tables + lanes:
        assert name in t, (name, sorted(t))
        assert t[name][0] >= 1 and t[name][1] > 0
    assert ctx.kernel_times() == {}  # reset by the previous read
    ctx.set_kernel_timing(False)
    ctx.multipoles(b.req_spectrum, b.req_z_mean, b.req_offset, b.sep, b.ls, precision="mixed")
    assert ctx.kernel_times() == {}


@pytest.mark.parametrize("nth", [1, 2, 3])
def test_injected_allocation_failure_is_enomem_and_recoverable(fresh_ctx, nth):
    from coffe_gb300 import workloads
    from coffe_gb300.api import CoffeGpuError

    b = workloads.subset(workloads.cfg3(n_spectra=2), 2)
    ctx = fresh_ctx
    ctx.background_init(0.31, 0.05, 9e-5, H, 10000)
    ctx.debug_fail_alloc(nth)  # a fresh context allocates its table buffers on first use
    with pytest.raises(CoffeGpuError) as ei:
        ctx.integrals_init(b.k, b.pk, [(0, 0), (0, 2), (0, 4)], N=4096, precision="fp64",
                           small_r=False)
    assert ei.value.status == -3
    assert "injected" in str(ei.value)
    # the failure left no half-built state: the same call now succeeds
    ctx.integrals_init(b.k, b.pk, [(0, 0), (0, 2), (0, 4)], N=4096, precision="fp64",
                       small_r=False)
    out = ctx.multipoles(b.req_spectrum, b.req_z_mean, b.req_offset, b.sep, b.ls)
    assert np.isfinite(out).all()


def test_allocation_failure_in_a_multipole_call(fresh_ctx):
    from coffe_gb300 import workloads
    from coffe_gb300.api import CoffeGpuError

    b = workloads.subset(workloads.cfg3(n_spectra=2), 2)
    ctx = fresh_ctx
    ctx.background_init(0.31, 0.05, 9e-5, H, 10000)
    ctx.integrals_init(b.k, b.pk, [(0, 0), (0, 2), (0, 4)], N=4096, precision="fp64",
                       small_r=False)
    ctx.debug_fail_alloc(1)  # the first buffer this call stages its requests in
    with pytest.raises(CoffeGpuError) as ei:
        ctx.multipoles(b.req_spectrum, b.req_z_mean, b.req_offset, b.sep, b.ls)
    assert ei.value.status == -3
    out = ctx.multipoles(b.req_spectrum, b.req_z_mean, b.req_offset, b.sep, b.ls)
    assert np.isfinite(out).all()
