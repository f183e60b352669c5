"""coffe_gpu_multipoles_noalloc against coffe_gpu_multipoles_async, through the C ABI.

The no-allocation entry point exists for callers that cannot let the library
allocate device memory mid-run: processes whose device memory is all pooled up
front (PyTorch's caching allocator, services that reserve their HBM) and callers
that cannot have cudaMalloc/cudaFree synchronise the whole device under other
streams.  It runs the same kernels with scratch taken from a fixed array, so its
results must match the allocating entry point within the parity tolerances used
everywhere else: 1e-10 relative on the FP64 path, 1e-4 on the mixed path, both
with a floor of 1e-3 of the largest |value| of the same request and multipole.

The file is named so that it is collected last; it builds its own context, so it
passes alone in a fresh process as well as after the other GPU tests.
"""
import numpy as np
import pytest

from conftest import H

pytestmark = pytest.mark.gpu

TOL = {"fp64": 1e-10, "mixed": 1e-4}


def _floor(ref, offsets, frac=1e-3):
    fl = np.zeros_like(ref)
    for q in range(len(offsets) - 1):
        lo, hi = offsets[q], offsets[q + 1]
        if hi > lo:
            fl[lo:hi] = frac * np.abs(ref[lo:hi]).max(axis=0)
    return np.maximum(fl, 1e-300)


def _rel_err(got, ref, offsets):
    return np.max(np.abs(got - ref) / np.maximum(np.abs(ref), _floor(ref, offsets)))


@pytest.fixture(scope="module")
def setup():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from coffe_gb300 import workloads
    from coffe_gb300.api import Context

    b = workloads.subset(workloads.cfg3(n_spectra=4), 4)
    ctx = Context(0)
    ctx.background_init(0.31, 0.05, 9e-5, H, 10000)
    dev = torch.device("cuda:0")
    arrays = dict(
        req_spectrum=torch.tensor(b.req_spectrum, dtype=torch.int32, device=dev),
        req_z_mean=torch.tensor(b.req_z_mean, dtype=torch.float64, device=dev),
        req_offset=torch.tensor(b.req_offset, dtype=torch.int64, device=dev),
        sep=torch.tensor(b.sep, dtype=torch.float64, device=dev),
    )
    yield torch, ctx, b, arrays
    ctx.close()


def _run(torch, ctx, b, arrays, precision, ls, noalloc):
    out = torch.full((len(b.sep), len(ls)), float("nan"), dtype=torch.float64, device="cuda:0")
    call = ctx.multipoles_noalloc if noalloc else ctx.multipoles_async
    torch.cuda.synchronize()  # inputs and the NaN fill are on torch's stream
    call(arrays["req_spectrum"], arrays["req_z_mean"], arrays["req_offset"], arrays["sep"],
         len(b.sep), ls, out, precision=precision)
    ctx.synchronize()
    return out.cpu().numpy()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_noalloc_matches_allocating_entry_point(setup, precision):
    torch, ctx, b, arrays = setup
    ctx.integrals_init(b.k, b.pk, [(0, 0), (0, 2), (0, 4)], N=4096, precision=precision,
                       small_r=False)
    ls = (0, 2, 4)
    ref = _run(torch, ctx, b, arrays, precision, ls, noalloc=False)
    assert np.isfinite(ref).all()
    # two calls in a row on the same scratch: the counter and node table are
    # re-initialised by each call
    for call in range(2):
        got = _run(torch, ctx, b, arrays, precision, ls, noalloc=True)
        assert np.isfinite(got).all(), call
        e = _rel_err(got, ref, b.req_offset)
        print(precision, "call", call, "max rel difference", e)
        assert e < TOL[precision], (call, e)
    # a different multipole list rewrites the node table
    ls2 = (2, 0)
    ref2 = _run(torch, ctx, b, arrays, precision, ls2, noalloc=False)
    got2 = _run(torch, ctx, b, arrays, precision, ls2, noalloc=True)
    assert _rel_err(got2, ref2, b.req_offset) < TOL[precision]


def test_noalloc_rejects_calls_beyond_its_scratch(setup):
    """The size check happens on the host before anything is launched."""
    from coffe_gb300 import _lib
    from coffe_gb300.api import CoffeGpuError

    torch, ctx, b, arrays = setup
    ctx.integrals_init(b.k, b.pk, [(0, 0), (0, 2), (0, 4)], N=4096, precision="fp64",
                       small_r=False)
    n_sep = _lib.NOALLOC_MAX_OUTPUTS // 3 + 1
    out = torch.empty((1, 3), dtype=torch.float64, device="cuda:0")
    with pytest.raises(CoffeGpuError) as ei:
        ctx.multipoles_noalloc(arrays["req_spectrum"], arrays["req_z_mean"],
                               arrays["req_offset"], arrays["sep"], n_sep, (0, 2, 4), out)
    assert ei.value.status == -1
    assert "scratch limit" in str(ei.value)


def test_noalloc_retry_path_and_odd_multipoles(setup):
    """Odd multipoles and unequal tracer biases (no mirror rule on either entry
    point) at a tolerance tight enough that first panels fail: the retry counter
    and list in the fixed scratch carry real work, and the results still match."""
    torch, ctx, b, arrays = setup
    z = np.linspace(0.0, 5.0, 11)
    ctx.set_bias(0, z, 1.0 + 0.4 * z)
    ctx.set_bias(1, z, 1.3 + 0.1 * z)
    try:
        ctx.integrals_init(b.k, b.pk, [(0, 0), (0, 2), (0, 4)], N=4096, precision="fp64",
                           small_r=False)
        ls = (1, 2, 3)
        for call in range(2):
            got = _run_eps(torch, ctx, b, arrays, ls, 1e-10, noalloc=True)
            ref = _run_eps(torch, ctx, b, arrays, ls, 1e-10, noalloc=False)
            assert ctx.last_retries() > 0  # the tolerance sends pairs to the retry list
            assert np.isfinite(got).all(), call
            assert _rel_err(got, ref, b.req_offset) < 1e-10, call
    finally:
        one = np.ones(11)
        ctx.set_bias(0, z, one)
        ctx.set_bias(1, z, one)


def _run_eps(torch, ctx, b, arrays, ls, epsrel, noalloc):
    out = torch.full((len(b.sep), len(ls)), float("nan"), dtype=torch.float64, device="cuda:0")
    call = ctx.multipoles_noalloc if noalloc else ctx.multipoles_async
    torch.cuda.synchronize()
    call(arrays["req_spectrum"], arrays["req_z_mean"], arrays["req_offset"], arrays["sep"],
         len(b.sep), ls, out, precision="fp64", epsrel=epsrel)
    ctx.synchronize()
    return out.cpu().numpy()


def test_noalloc_call_leaves_device_memory_unchanged(setup):
    """The contract itself: with the inputs and the output already on the device,
    a call on a multipole list and size this context has not seen before changes
    the device's free memory by nothing."""
    torch, ctx, b, arrays = setup
    ctx.integrals_init(b.k, b.pk, [(0, 0), (0, 2), (0, 4)], N=4096, precision="mixed",
                       small_r=False)
    n = int(b.req_offset[2])  # the first two requests only: a new size
    ls = (4, 2, 0, 6)
    out = torch.full((n, len(ls)), float("nan"), dtype=torch.float64, device="cuda:0")
    offs = arrays["req_offset"][:3].clone()
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    ctx.multipoles_noalloc(arrays["req_spectrum"][:2], arrays["req_z_mean"][:2], offs,
                           arrays["sep"], n, ls, out, precision="mixed")
    ctx.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0, (free0, free1)
    assert torch.isfinite(out).all()
