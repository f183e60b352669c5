"""GPU parity of the divergent integral I^4_0 and its renormalisation grid
(integrals.c:773-914) through the C ABI: FP64 against the oracle at 1e-10 on the
reference's fixed separations and on a chi grid, against the reference's golden
files (benchmark_integral8*.dat, tests/test_integrals.c:156-248) at 1e-8 / 1e-5,
and the argument checks."""
import numpy as np
import pytest

from conftest import COFFE_H0, H

pytestmark = pytest.mark.gpu

KMIN, KMAX = 1e-5 * H, 300.0 * H  # the reference's defaults, 1e-5 .. 300 h/Mpc


def test_divergent_integral_matches_oracle_and_golden(gpu_ctx, oracle, class_pk, golden):
    k, pk = class_pk
    sep, res, res0 = gpu_ctx.divergent_integral(k, pk, kmin=KMIN, kmax=KMAX)
    assert len(sep) == 297
    ref, ref0 = oracle.divergent_i40(k, pk, sep, KMIN, KMAX)
    assert np.allclose(res, ref, rtol=1e-10, atol=0)
    assert np.allclose(res0, ref0, rtol=1e-10, atol=1e-12 * np.abs(ref0).max())
    d = golden["integral8"]
    r = d[:, 0] / (COFFE_H0 * H)
    _, got, _ = gpu_ctx.divergent_integral(k, pk, r, kmin=KMIN, kmax=KMAX)
    assert np.allclose(got * (COFFE_H0 * H) ** 4, d[:, 1], rtol=1e-8)


def test_renormalization_grid_matches_oracle_and_golden(gpu_ctx, oracle, class_pk, golden):
    k, pk = class_pk
    ren = golden["integral8_renormalization"]
    n = int(round(np.sqrt(len(ren))))
    chi1 = ren[::n, 0] / (COFFE_H0 * H)
    chi2 = ren[:n, 1] / (COFFE_H0 * H)
    got = gpu_ctx.renormalization_grid(k, pk, chi1, chi2, kmin=KMIN, kmax=KMAX)
    ref = oracle.renormalization_grid(k, pk, chi1, chi2, KMIN, KMAX)
    assert np.allclose(got, ref, rtol=1e-10, atol=0)
    assert np.allclose(got.T * (COFFE_H0 * H) ** 4, ren[:, 2].reshape(n, n), rtol=1e-5)
    # a non-square grid keeps the [chi2, chi1] layout
    g2 = gpu_ctx.renormalization_grid(k, pk, chi1[:5], chi2[:3], kmin=KMIN, kmax=KMAX)
    assert g2.shape == (3, 5) and np.allclose(g2, ref[:3, :5], rtol=1e-10)


def test_divergent_integral_rejects_bad_arguments(gpu_ctx, class_pk):
    from coffe_gb300.api import CoffeGpuError

    k, pk = class_pk
    for kw in (dict(sep=[10.0, -1.0]), dict(sep=[0.0]), dict(kmin=k[0] / 2),
               dict(kmin=1.0, kmax=0.5)):
        with pytest.raises(CoffeGpuError) as e:
            gpu_ctx.divergent_integral(k, pk, **kw)
        assert e.value.status == -1
    with pytest.raises(CoffeGpuError):
        gpu_ctx.renormalization_grid(k, pk, [-1.0, 10.0])
    _, res, _ = gpu_ctx.divergent_integral(k, pk, [50.0], kmin=KMIN, kmax=KMAX)
    assert np.isfinite(res).all()  # the context stays usable
