"""GPU parity of the 2D-FFTLog multipole covariance through the C ABI: the
double-Bessel integrals against the oracle's FFTLog (same algorithm, FP64,
1e-10 of each block's largest value), the assembled covariance against the
oracle's assembly of the oracle's integrals (1e-10 relative with the same
floor), and the golden covariance at the tolerance the FFTLog method itself
allows there (the golden file was made by direct quadrature)."""
import numpy as np
import pytest

from conftest import H

pytestmark = pytest.mark.gpu


def _blockrel(got, ref):
    scale = np.abs(ref).max(axis=(-1, -2), keepdims=True)
    return np.max(np.abs(got - ref) / scale)


@pytest.fixture(scope="module")
def cfg5(oracle):
    from coffe_gb300 import workloads

    bg = oracle.background_nodes(0.31, 0.05, 9e-5, H, 10000)
    chi = lambda z: np.interp(z, bg["z"], bg["chi"])
    return workloads.cfg5(chi), bg


@pytest.mark.parametrize("N", [1024, 2048])
def test_covariance_integrals_match_oracle(gpu_ctx, oracle, cfg5, N):
    c, _ = cfg5
    sep = c["sep"][::8]  # 16 separations across 20-300 Mpc/h
    jobs = [(1, 0, 0), (2, 0, 2), (1, 2, 4), (2, 4, 4)]
    got = gpu_ctx.covariance_integrals(c["k"], c["pk"], N, jobs, sep)
    for q, (p, l1, l2) in enumerate(jobs):
        ref = oracle.covariance_fftlog(c["k"], c["pk"], p, l1, l2, N, sep)
        e = _blockrel(got[q], ref)
        print(N, (p, l1, l2), "max abs error / block max", e)
        assert e < 1e-10, ((p, l1, l2), e)


def test_covariance_multipoles_match_oracle(gpu_ctx, oracle, cfg5):
    """cfg5 shapes with 24 separations (all five redshift bins, l = 0, 2, 4)."""
    c, bg = cfg5
    sep = c["sep"][::5][:24]
    N, ls = 1024, c["ls"]
    gpu_ctx.background_init(0.31, 0.05, 9e-5, H, 10000)
    got = gpu_ctx.covariance_multipoles(c["k"], c["pk"], N, c["z_mean"], c["deltaz"], c["fsky"],
                                        c["density"], c["density"], c["pixelsize"], ls, sep)
    nl, ns = len(ls), len(sep)
    ipk = np.zeros((nl, nl, ns, ns))
    ipk2 = np.zeros_like(ipk)
    for i, l1 in enumerate(ls):
        for j, l2 in enumerate(ls):
            if j < i:
                continue
            f = (2 * l1 + 1) * (2 * l2 + 1) / np.pi ** 2
            ipk[i, j] = oracle.covariance_fftlog(c["k"], c["pk"], 1, l1, l2, N, sep) * 2 * f
            ipk2[i, j] = oracle.covariance_fftlog(c["k"], c["pk"], 2, l1, l2, N, sep) * f
    for i in range(nl):
        for j in range(i):
            ipk[i, j] = ipk[j, i].T
            ipk2[i, j] = ipk2[j, i].T
    m = oracle.Model(bg, H, 0.31)
    ref = m.covariance_multipoles(3, c["z_mean"], c["deltaz"], c["fsky"], c["density"],
                                  c["pixelsize"], ls, sep, ipk, ipk2)
    # per (z, l1, l2) block, relative to the block's largest |value|
    g = np.moveaxis(got, 3, 2)
    r = np.moveaxis(ref, 3, 2)
    e = _blockrel(g, r)
    print("covariance max abs error / block max", e)
    assert e < 1e-10, e


def test_covariance_golden_through_gpu(gpu_ctx, golden):
    """The reference's golden covariance (direct quadrature) through the FFTLog
    path at N = 8192: the diagonal and near-diagonal elements, which carry the
    covariance, agree to 1e-2 of each block's largest value (the accuracy of
    the FFTLog method on the 159-point PkL_CLASS spectrum)."""
    k, pk = golden["pk_class"].T
    k, pk = k * H, pk / H ** 3
    sep = np.arange(50, 350, 50) / H
    gpu_ctx.background_init(0.3, 0.05, 9e-5, H, 10000)
    got = gpu_ctx.covariance_multipoles(k, pk, 8192, [1.0], [0.1], [0.2], [1e-3 * H ** 3],
                                        [1e-3 * H ** 3], [50 / H], (0, 2, 4), sep)
    for i, l1 in enumerate((0, 2, 4)):
        for j, l2 in enumerate((0, 2, 4)):
            d = golden[f"multipoles_covariance_{l1}{l2}"][:, 2].reshape(6, 6)
            e = np.abs(got[0, i, :, j, :] - d).max() / np.abs(d).max()
            print(l1, l2, "max abs error / block max", e)
            assert e < 1e-2, (l1, l2, e)


def test_covariance_rejects_bad_input(gpu_ctx, cfg5):
    from coffe_gb300.api import CoffeGpuError

    c, _ = cfg5
    with pytest.raises(CoffeGpuError):
        gpu_ctx.covariance_integrals(c["k"], c["pk"], 1000, [(1, 0, 0)], c["sep"][:4])
    with pytest.raises(CoffeGpuError):
        gpu_ctx.covariance_integrals(c["k"], c["pk"], 1024, [(1, 0, 0)], [1e9])


def test_average_covariance_multipoles_match_oracle(gpu_ctx, oracle, cfg5):
    """Covariance of the redshift-averaged multipoles: windows at
    (z_min + z_max)/2 with their effective volumes, against the oracle's
    assembly (QAG volume) of the oracle's FFTLog integrals, 1e-10 of each
    block's largest value."""
    c, bg = cfg5
    sep = c["sep"][::5][:16]
    N, ls = 1024, c["ls"]
    zmin, zmax = [0.5, 1.0, 0.3], [0.8, 1.5, 1.2]
    gpu_ctx.background_init(0.31, 0.05, 9e-5, H, 10000)
    got = gpu_ctx.average_covariance_multipoles(c["k"], c["pk"], N, zmin, zmax, 0.2, 1e-3 * H ** 3,
                                                1e-3 * H ** 3, 50 / H, ls, sep)
    nl, ns = len(ls), len(sep)
    ipk = np.zeros((nl, nl, ns, ns))
    ipk2 = np.zeros_like(ipk)
    for i, l1 in enumerate(ls):
        for j, l2 in enumerate(ls):
            if j < i:
                continue
            f = (2 * l1 + 1) * (2 * l2 + 1) / np.pi ** 2
            ipk[i, j] = oracle.covariance_fftlog(c["k"], c["pk"], 1, l1, l2, N, sep) * 2 * f
            ipk2[i, j] = oracle.covariance_fftlog(c["k"], c["pk"], 2, l1, l2, N, sep) * f
    for i in range(nl):
        for j in range(i):
            ipk[i, j] = ipk[j, i].T
            ipk2[i, j] = ipk2[j, i].T
    m = oracle.Model(bg, H, 0.31)
    ref = m.average_covariance_multipoles(3, zmin, zmax, 0.2, 1e-3 * H ** 3, 50 / H, ls, sep,
                                          ipk, ipk2)
    e = _blockrel(np.moveaxis(got, 3, 2), np.moveaxis(ref, 3, 2))
    print("average covariance max abs error / block max", e)
    assert e < 1e-10, e


def test_average_covariance_golden_through_gpu(gpu_ctx, golden):
    """The reference's golden averaged covariance (direct quadrature, z in
    [0.9, 1.1]) through the FFTLog path at N = 8192, to 1e-2 of each block's
    largest value, as the plain covariance."""
    k, pk = golden["pk_class"].T
    k, pk = k * H, pk / H ** 3
    sep = np.arange(50, 350, 50) / H
    gpu_ctx.background_init(0.3, 0.05, 9e-5, H, 10000)
    got = gpu_ctx.average_covariance_multipoles(k, pk, 8192, [0.9], [1.1], [0.2], [1e-3 * H ** 3],
                                                [1e-3 * H ** 3], [50 / H], (0, 2, 4), sep)
    for i, l1 in enumerate((0, 2, 4)):
        for j, l2 in enumerate((0, 2, 4)):
            d = golden[f"avg_multipoles_covariance_{l1}{l2}"][:, 2].reshape(6, 6)
            e = np.abs(got[0, i, :, j, :] - d).max() / np.abs(d).max()
            print(l1, l2, "max abs error / block max", e)
            assert e < 1e-2, (l1, l2, e)
    from coffe_gb300.api import CoffeGpuError

    with pytest.raises(CoffeGpuError):  # z_max <= z_min
        gpu_ctx.average_covariance_multipoles(k, pk, 1024, [1.1], [0.9], [0.2], [1e-3], [1e-3],
                                              [50 / H], (0,), sep)


def test_coffe_mirror_covariance_bulk(golden):
    """Coffe.compute_covariance_bulk / compute_average_covariance_bulk in the
    reference's order (z or window outer, then l1, r1, l2, r2) against the
    golden covariances at the tolerance of the Context tests above."""
    from coffe_gb300.api import Coffe

    k, pk = golden["pk_class"].T
    sep = np.arange(50, 350, 50) / H
    cosmo = Coffe(sep=sep, l=[0, 2, 4], z_mean=[1.0], deltaz=[0.1], z_min=[0.9], z_max=[1.1],
                  number_density1=[1e-3 * H ** 3], number_density2=[1e-3 * H ** 3],
                  pixelsize=[50 / H], fsky=[0.2], has_density=True, has_rsd=True)
    try:
        cosmo.set_power_spectrum_linear(k * H, pk / H ** 3)
        for name, res in (("multipoles_covariance", cosmo.compute_covariance_bulk()),
                          ("avg_multipoles_covariance", cosmo.compute_average_covariance_bulk())):
            assert len(res) == 9 * 36
            assert (res[0].l1, res[0].l2, res[0].r1, res[0].r2) == (0, 0, sep[0], sep[0])
            assert (res[1].r1, res[1].r2) == (sep[0], sep[1])
            assert (res[6].r1, res[6].l2) == (sep[0], 2)
            vals = np.array([r.value for r in res]).reshape(3, 6, 3, 6)
            for i, l1 in enumerate((0, 2, 4)):
                for j, l2 in enumerate((0, 2, 4)):
                    d = golden[f"{name}_{l1}{l2}"][:, 2].reshape(6, 6)
                    e = np.abs(vals[i, :, j, :] - d).max() / np.abs(d).max()
                    assert e < 1e-2, (name, l1, l2, e)
        cosmo.number_density2 = []
        with pytest.raises(ValueError):
            cosmo.compute_covariance_bulk()
    finally:
        cosmo.close()
