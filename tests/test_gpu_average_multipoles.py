"""GPU parity of the redshift-averaged multipoles (average_multipoles.c:69-156)
through the C ABI: FP64 against the oracle at 1e-10 and mixed at 1e-4
relative (floor 1e-3 of the multipole's largest |value|), den+rsd and with
lensing on reduced rules; the reference's golden averaged multipoles at its
rtol 5e-4; the Coffe mirror's bulk output in the reference's order."""
import numpy as np
import pytest

from conftest import H

pytestmark = pytest.mark.gpu

LENS_TERMS = [(0, 0), (0, 2), (0, 4), (1, 1), (1, 3), (2, 0)]
LS = (0, 2, 4)


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
    windows = [(0.6, 0.8, np.array([15.0, 60.0, 140.0]) / H),
               (1.2, 1.6, np.array([25.0, 200.0]) / H)]
    return k, pk, m, windows


def _rel(got, ref):
    floor = 1e-3 * np.abs(ref).max(axis=0, keepdims=True)
    return np.max(np.abs(got - ref) / np.maximum(np.abs(ref), floor))


@pytest.mark.parametrize("contrib,n_z", [(3, 16), (7, 8)])
def test_average_multipoles_match_oracle(gpu_ctx, setup, contrib, n_z):
    k, pk, m, windows = setup
    zmin = [w[0] for w in windows]
    zmax = [w[1] for w in windows]
    sep = np.concatenate([w[2] for w in windows])
    offs = np.cumsum([0] + [len(w[2]) for w in windows])
    ref = np.concatenate([np.stack([m.average_multipoles(contrib, a, b, s, l, n_z=n_z,
                                                         n_mu=16, n_x=32) for l in LS], axis=1)
                          for a, b, s in windows])
    for prec, tol in (("fp64", 1e-10), ("mixed", 1e-4)):
        gpu_ctx.background_init(0.31, 0.05, 9e-5, H, 10000)
        gpu_ctx.integrals_init(k, pk[None, :], LENS_TERMS, N=4096, precision=prec, small_r=True)
        gpu_ctx.set_lensing_rule(16, 32)
        got = gpu_ctx.average_multipoles([0, 0], zmin, zmax, offs, sep, LS, contrib, prec,
                                         n_z=n_z)
        e = _rel(got, ref)
        print(contrib, prec, "max rel error", e)
        assert e < tol, (contrib, prec, e)


def test_average_multipoles_golden_through_gpu(gpu_ctx, golden, class_pk):
    """The reference's golden den+rsd averaged multipoles (z in [0.9, 1.1],
    PkL_CLASS; test_coffe.py:305-326) at its rtol 5e-4, FP64."""
    k, pk = class_pk
    gpu_ctx.background_init(0.3, 0.05, 9e-5, H, 10000)
    gpu_ctx.integrals_init(k, pk[None, :], LENS_TERMS, N=8192, precision="fp64", small_r=True)
    sep = golden["avg_multipoles0"][:, 0] / H
    got = gpu_ctx.average_multipoles([0], [0.9], [1.1], [0, len(sep)], sep, LS, 3, n_z=16)
    for j, l in enumerate(LS):
        ref = golden[f"avg_multipoles{l}"][:, 1]
        assert np.allclose(got[:, j], ref, rtol=5e-4), (l, got[:, j] / ref - 1)


def test_coffe_mirror_average_multipoles_bulk(golden, class_pk):
    from coffe_gb300.api import Coffe

    k, pk = class_pk
    cosmo = Coffe(sep=np.array([10, 20, 40, 100, 150]) / H, l=[0, 2, 4], z_min=[0.9],
                  z_max=[1.1], has_density=True, has_rsd=True, integrals_fftlog_sampling=8192)
    try:
        cosmo.set_power_spectrum_linear(k, pk)
        res = cosmo.compute_average_multipoles_bulk()
        assert [(r.l, r.r) for r in res[:6]] == [(0, r) for r in cosmo.sep] + [(2, cosmo.sep[0])]
        for l in (0, 2, 4):
            vals = np.array([r.value for r in res if r.l == l])
            assert np.allclose(vals, golden[f"avg_multipoles{l}"][:, 1], rtol=5e-4), l
        one = cosmo.compute_average_multipole(z_min=0.9, z_max=1.1, r=float(cosmo.sep[3]), l=2)
        assert np.isclose(one, golden["avg_multipoles2"][3, 1], rtol=5e-4)
    finally:
        cosmo.close()


def test_average_multipoles_rejects_bad_window(gpu_ctx, setup):
    from coffe_gb300.api import CoffeGpuError

    k, pk, _, _ = setup
    gpu_ctx.background_init(0.31, 0.05, 9e-5, H, 10000)
    gpu_ctx.integrals_init(k, pk[None, :], LENS_TERMS, N=4096, precision="fp64", small_r=True)
    with pytest.raises(CoffeGpuError) as e:
        gpu_ctx.average_multipoles([0], [1.1], [0.9], [0, 1], [50.0])
    assert e.value.status == -1
