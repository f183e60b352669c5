"""The host-array multipole call with a page-locked output: the den/rsd kernels
write the results into the caller's memory directly (staged through shared
memory, whole lines over the host link) instead of a device copy and a
download.  Its results equal the pageable-output call's bit for bit, on the
fast mixed kernel, the general mixed kernel (galaxy biases) and FP64; a
non-positive separation still returns EINVAL after the work, and the context
stays usable."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TERMS = ((0, 0), (0, 2), (0, 4))


def test_mapped_output_equals_copied_output():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from coffe_gb300 import workloads
    from coffe_gb300.api import Context, CoffeGpuError

    b = workloads.cfg3(n_spectra=16)
    c = b.cosmo
    ctx = Context(0)
    try:
        ctx.background_init(c.omega_m, c.omega_baryon, c.omega_gamma, c.h, 10000)
        for prec, bias in (("mixed", False), ("fp64", False), ("mixed", True)):  # biases stay set
            if bias:
                z = np.linspace(0.0, 5.0, 64)
                ctx.set_bias(0, z, 1.0 + 0.4 * z)
                ctx.set_bias(1, z, 1.3 + 0.1 * z)
            ctx.integrals_init(b.k, b.pk, TERMS, N=4096, precision=prec, small_r=False)
            for ls in (b.ls, (0, 2), (0, 2, 4, 6, 8)):  # odd and even result counts
                n = len(b.sep) - 3  # a ragged last block
                ro = np.minimum(b.req_offset, n)
                pinned = torch.zeros((n, len(ls)), dtype=torch.float64).pin_memory().numpy()
                got = ctx.multipoles(b.req_spectrum, b.req_z_mean, ro, b.sep[:n], ls,
                                     precision=prec, out=pinned)
                ref = ctx.multipoles(b.req_spectrum, b.req_z_mean, ro, b.sep[:n], ls,
                                     precision=prec)
                assert np.isfinite(ref).all()
                assert np.array_equal(got, ref), (prec, bias, ls)
            bad = b.sep.copy()
            bad[-7] = -1.0
            with pytest.raises(CoffeGpuError) as e:
                ctx.multipoles(b.req_spectrum, b.req_z_mean, b.req_offset, bad, b.ls,
                               precision=prec, out=torch.zeros((len(b.sep), 3),
                               dtype=torch.float64).pin_memory().numpy())
            assert e.value.status == -1 and "positive" in str(e.value)
            again = ctx.multipoles(b.req_spectrum, b.req_z_mean, b.req_offset, b.sep, b.ls,
                                   precision=prec)
            assert np.isfinite(again).all()
    finally:
        ctx.close()



def test_mapped_output_with_lensing_takes_the_copy_path(oracle):
    """With lensing the results are accumulated over several kernels: a
    page-locked output then goes through the device copy, and equals the
    pageable-output call."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from coffe_gb300 import workloads
    from coffe_gb300.api import Context

    c = workloads.cfg1()
    terms = [(0, 0), (0, 2), (0, 4), (1, 1), (1, 3), (2, 0)]
    sep = np.array([20.0, 80.0, 200.0]) / 0.67
    ctx = Context(0)
    try:
        ctx.background_init(0.31, 0.05, 9e-5, 0.67, 10000)
        ctx.integrals_init(c["k"], c["pk"][None, :], terms, N=4096, precision="mixed",
                           small_r=True)
        ctx.set_lensing_rule(16, 32)
        pinned = torch.zeros((len(sep), 3), dtype=torch.float64).pin_memory().numpy()
        got = ctx.multipoles([0], [1.5], [0, len(sep)], sep, (0, 2, 4), contrib=7,
                             precision="mixed", out=pinned)
        ref = ctx.multipoles([0], [1.5], [0, len(sep)], sep, (0, 2, 4), contrib=7,
                             precision="mixed")
        assert np.isfinite(ref).all() and np.array_equal(got, ref)
    finally:
        ctx.close()
