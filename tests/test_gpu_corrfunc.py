"""GPU parity of the correlation function (corrfunc.c:55-141) through the C ABI:
FP64 against the oracle at 1e-10 and mixed at 1e-4 relative (floor 1e-3 of
the largest |value| of the output), den/rsd and with the lensing line and
plane integrals on a reduced rule; the reference's golden correlation
functions at its rtol 5e-4; the Coffe mirror's bulk output in the reference's
order; and the only-cross switch."""
import numpy as np
import pytest

from conftest import H

pytestmark = pytest.mark.gpu

LENS_TERMS = [(0, 0), (0, 2), (0, 4), (1, 1), (1, 3), (2, 0)]
MUS = np.array([-1.0, -0.7, -0.2, 0.0, 0.3, 0.5, 0.9, 1.0])
DEN, RSD, LEN, ONLY_CROSS = 1, 2, 4, 8


@pytest.fixture(scope="module")
def setup(oracle):
    from coffe_gb300 import workloads

    c = workloads.cfg1()
    k, pk = c["k"], c["pk"]
    bg = oracle.background_nodes(0.31, 0.05, 9e-5, H, 10000)
    m = oracle.Model(bg, H, 0.31)
    for n, l in LENS_TERMS:
        x, y = oracle.integral_table(k, pk, n, l, 4096, with_small_r=True)
        m.set_integral(n, l, x, y)
    sep = [np.array([12.0, 55.0, 140.0]) / H, np.array([30.0, 250.0]) / H]
    return k, pk, m, (0.7, 1.5), sep


def _gpu(ctx, k, pk, prec, zs, sep, contrib, n_x=32):
    ctx.background_init(0.31, 0.05, 9e-5, H, 10000)
    ctx.integrals_init(k, pk[None, :], LENS_TERMS, N=4096, precision=prec, small_r=True)
    ctx.set_lensing_rule(64, n_x)
    offs = np.cumsum([0] + [len(s) for s in sep])
    return ctx.corrfunc([0] * len(zs), zs, offs, np.concatenate(sep), MUS, contrib, prec)


def _oracle(m, zs, sep, contrib, n_x=32):
    rows = [m.corrfunc(contrib, z, MUS[None, :], s[:, None], n_x=n_x).reshape(len(s), len(MUS))
            for z, s in zip(zs, sep)]
    return np.concatenate(rows)


def _rel(got, ref):
    floor = 1e-3 * np.abs(ref).max()
    return np.max(np.abs(got - ref) / np.maximum(np.abs(ref), floor))


@pytest.mark.parametrize("contrib", [DEN, RSD, DEN | RSD, LEN, DEN | RSD | LEN])
def test_corrfunc_fp64_and_mixed_match_oracle(gpu_ctx, setup, contrib):
    k, pk, m, zs, sep = setup
    ref = _oracle(m, zs, sep, contrib)
    for prec, tol in (("fp64", 1e-10), ("mixed", 1e-4)):
        got = _gpu(gpu_ctx, k, pk, prec, zs, sep, contrib)
        e = _rel(got, ref)
        print(contrib, prec, "max rel error", e)
        assert e < tol, (contrib, prec, e)


def test_corrfunc_only_cross(gpu_ctx, setup):
    """Only cross-correlations keep the den-rsd term of the nonintegrated part:
    xi(den+rsd, only cross) = xi(den+rsd) - xi(den) - xi(rsd)."""
    k, pk, _, zs, sep = setup
    both = _gpu(gpu_ctx, k, pk, "fp64", zs, sep, DEN | RSD)
    den = _gpu(gpu_ctx, k, pk, "fp64", zs, sep, DEN)
    rsd = _gpu(gpu_ctx, k, pk, "fp64", zs, sep, RSD)
    cross = _gpu(gpu_ctx, k, pk, "fp64", zs, sep, DEN | RSD | ONLY_CROSS)
    assert np.max(np.abs(cross - (both - den - rsd))) <= 1e-12 * np.abs(both).max()


def test_corrfunc_golden_through_gpu(gpu_ctx, golden, class_pk):
    """The reference's golden correlation functions (z = 1, PkL_CLASS;
    test_coffe.py:235-268) at its rtol 5e-4, FP64."""
    k, pk = class_pk
    gpu_ctx.background_init(0.3, 0.05, 9e-5, H, 10000)
    gpu_ctx.integrals_init(k, pk[None, :], LENS_TERMS, N=8192, precision="fp64", small_r=True)
    gpu_ctx.set_lensing_rule(128, 256)
    mus = (0.0, 0.2, 0.5, 0.8, 0.95)
    sep = golden["den_corrfunc0"][:, 0] / H
    for name, mask in [("den", DEN), ("rsd", RSD), ("std", DEN | RSD), ("len", LEN),
                       ("std_len", DEN | RSD | LEN)]:
        got = gpu_ctx.corrfunc([0], [1.0], [0, len(sep)], sep, mus, mask)
        for i in range(len(mus)):
            ref = golden[f"{name}_corrfunc{i}"]
            assert np.allclose(ref[:, 0], sep * H)
            assert np.allclose(got[:, i], ref[:, 1], rtol=5e-4), (name, mus[i], got[:, i] / ref[:, 1] - 1)


def test_coffe_mirror_corrfunc_bulk(golden, class_pk):
    """Coffe.compute_corrfunc_bulk in the reference's order (z, mu, r) against
    the den+rsd golden files, as the reference's own test reads them."""
    from coffe_gb300.api import Coffe

    k, pk = class_pk
    mus = [0.0, 0.2, 0.5, 0.8, 0.95]
    cosmo = Coffe(sep=np.array([10, 20, 40, 100, 150]) / H, mu=mus, has_density=True,
                  has_rsd=True, integrals_fftlog_sampling=8192)
    try:
        cosmo.set_power_spectrum_linear(k, pk)
        res = cosmo.compute_corrfunc_bulk()
        assert [(r.mu, r.r) for r in res[:6]] == [(0.0, r) for r in cosmo.sep] + [(0.2, cosmo.sep[0])]
        for i, mu in enumerate(mus):
            vals = np.array([r.value for r in res if r.mu == mu])
            assert np.allclose(vals, golden[f"std_corrfunc{i}"][:, 1], rtol=5e-4), mu
        one = cosmo.compute_corrfunc(z=1.0, r=float(cosmo.sep[2]), mu=0.5)
        assert np.isclose(one, golden["std_corrfunc2"][2, 1], rtol=5e-4)
        with pytest.raises(ValueError):
            cosmo.compute_corrfunc(z=1.0, r=50.0, mu=1.5)
    finally:
        cosmo.close()


def test_corrfunc_rejects_bad_mu(gpu_ctx, setup):
    from coffe_gb300.api import CoffeGpuError

    k, pk, _, _, _ = setup
    gpu_ctx.background_init(0.31, 0.05, 9e-5, H, 10000)
    gpu_ctx.integrals_init(k, pk[None, :], LENS_TERMS, N=4096, precision="fp64", small_r=True)
    with pytest.raises(CoffeGpuError) as e:
        gpu_ctx.corrfunc([0], [1.0], [0, 1], [50.0], [0.5, 1.5])
    assert e.value.status == -1
