"""The covariance part of the CPU oracle: the 2D FFTLog of a diagonal kernel
against an independent dense numpy restatement of two_sph_bessel, the direct
double-Bessel integrals + assembly against the reference's golden covariance
(tests/test_coffe.py:382-417: rtol 5e-4), and the FFTLog integrals against
direct quadrature of the same integrand."""
import numpy as np
import pytest

from conftest import H


def _dense_two_sph_bessel(k, fk, l1, l2, nu1=1.01, nu2=1.01, width=0.25):
    """two_sph_bessel (twobessel.c:16-122, C branch) on a dense N x N kernel
    with numpy's real 2D FFTs (the FFTW r2c/c2r conventions) and scipy's
    lnGamma: an implementation independent of the oracle's."""
    from scipy.special import loggamma

    N = len(k)
    hN = N // 2
    dlnk = np.log(k[1] / k[0])
    r = 1.0 / k[::-1]
    eta_m = 2 * np.pi / dlnk / N * np.arange(hN + 1)

    def g(l, nu, eta):
        z = nu + 1j * eta
        return np.exp(z * np.log(2.0) + loggamma((l + z) / 2) - loggamma((3 + l - z) / 2))

    g1, g2 = g(l1, nu1, eta_m), g(l2, nu2, eta_m)
    Pb = fk / (k ** nu1)[:, None] / (k ** nu2)[None, :]
    out = np.fft.rfft2(Pb)
    # c_window_2d (utils.c:235-258)
    nc = int(hN * width)
    W = lambda t: t / nc - np.sin(2 * np.pi * t / nc) / (2 * np.pi)
    for j in range(nc + 1):
        out[:, hN - j] *= W(j)
    for i in range(nc + 1):
        out[hN - i, :] *= W(i)
        out[hN + 1 + i, :] *= W(i)
    kr = k[0] * r[0]
    col = (kr ** (-1j * eta_m)) * g2
    row = np.empty(N, dtype=complex)
    row[: hN + 1] = (kr ** (-1j * eta_m)) * g1
    row[hN + 1:] = np.conj((kr ** (-1j * eta_m[1:hN])) * g1[1:hN])[::-1]
    out = np.conj(out * col[None, :] * row[:, None])
    res = np.fft.irfft2(out, s=(N, N)) * N * N
    return r, res * np.pi / (16.0 * N * N * (r ** nu1)[:, None] * (r ** nu2)[None, :])


@pytest.mark.parametrize("l1,l2", [(0, 0), (0, 2), (2, 4), (4, 4)])
def test_twobessel_diagonal_matches_dense(oracle, l1, l2):
    N = 64
    k = 1e-3 * 10.0 ** (6.0 * np.arange(N) / N)
    rng = np.random.default_rng(1)
    diag = rng.uniform(0.5, 2.0, N) * k ** 1.5
    r, got = oracle.twobessel_diag(k, diag, l1, l2)
    r2, ref = _dense_two_sph_bessel(k, np.diag(diag), l1, l2)
    assert np.allclose(r, r2, rtol=1e-15)
    scale = np.abs(ref).max()
    assert np.abs(got - ref).max() < 1e-11 * scale, np.abs(got - ref).max() / scale


def _golden_setup(golden):
    k, pk = golden["pk_class"].T
    return k * H, pk / H ** 3, np.arange(50, 350, 50) / H, (0, 2, 4)


def _direct_integrals(oracle, k, pk, sep, ls):
    nl, ns = len(ls), len(sep)
    ipk = np.zeros((nl, nl, ns, ns))
    ipk2 = np.zeros_like(ipk)
    for i, l1 in enumerate(ls):
        for j, l2 in enumerate(ls):
            if j < i:
                continue
            for p, arr, den in ((1, ipk, 1.0), (2, ipk2, 2.0)):
                v = np.array([[oracle.covariance_integral(k, pk, p, sep[m], sep[n], l1, l2)
                               for m in range(ns)] for n in range(ns)])
                arr[i, j] = v * (2 * l1 + 1) * (2 * l2 + 1) / np.pi / den
    for i in range(nl):
        for j in range(i):
            ipk[i, j] = ipk[j, i].T
            ipk2[i, j] = ipk2[j, i].T
    return ipk, ipk2


def test_covariance_direct_matches_golden(golden, oracle, ref_bg):
    """covariance_integration_method 'standard' (the golden file's) plus the
    assembly of covariance.c:786-1059, at the test's settings
    (test_coffe.py:382-417): den + rsd, n = 1e-3 (h/Mpc)^3, z = 1, dz = 0.1,
    fsky = 0.2, pixel 50 Mpc/h, separations 50-300 Mpc/h."""
    k, pk, sep, ls = _golden_setup(golden)
    m = oracle.Model(ref_bg, H, 0.3)
    ipk, ipk2 = _direct_integrals(oracle, k, pk, sep, ls)
    cov = m.covariance_multipoles(3, [1.0], [0.1], [0.2], [1e-3 * H ** 3], [50 / H], ls, sep,
                                  ipk, ipk2)
    for i, l1 in enumerate(ls):
        for j, l2 in enumerate(ls):
            d = golden[f"multipoles_covariance_{l1}{l2}"]
            assert np.allclose(d[:, 0] / H, np.repeat(sep, len(sep)))
            assert np.allclose(cov[0, i, :, j, :].ravel(), d[:, 2], rtol=5e-4), (l1, l2)


@pytest.mark.parametrize("l1,l2", [(0, 0), (2, 2)])
def test_covariance_fftlog_close_to_direct(golden, oracle, l1, l2):
    """The 2D FFTLog integrals (covariance.c:357-470) at N = 2048 against direct
    quadrature of the same integrand (the power of the P(k) spline, as the
    FFTLog path samples it): the method's own discretisation error on the
    PkL_CLASS spectrum is 2% of the block's largest value at N = 2048 (8% at
    1024, 18% at 512), the accuracy the reference's FFTLog path has here."""
    k, pk, sep, _ = _golden_setup(golden)
    for p in (1, 2):
        f = oracle.covariance_fftlog(k, pk, p, l1, l2, 2048, sep)
        q = np.array([[oracle.covariance_integral(k, pk, p, sep[m], sep[n], l1, l2,
                                                  power_of_spline=True)
                       for m in range(len(sep))] for n in range(len(sep))]) * np.pi / 2
        assert np.abs(f - q).max() < 3e-2 * np.abs(q).max(), (p, np.abs(f - q).max() / np.abs(q).max())


def test_average_covariance_direct_matches_golden(golden, oracle, ref_bg):
    """Covariance of the redshift-averaged multipoles (covariance.c:811-840:
    the bin at (z_min + z_max) / 2 with the window's effective volume
    4 pi fsky / int dz / (conformal_H chi^2 (1 + z)) / (H0 h)^2) at the
    reference test's settings (test_coffe.py:433-470: z in [0.9, 1.1], the rest
    as test_covariance_direct_matches_golden), standard integration method."""
    k, pk, sep, ls = _golden_setup(golden)
    m = oracle.Model(ref_bg, H, 0.3)
    ipk, ipk2 = _direct_integrals(oracle, k, pk, sep, ls)
    cov = m.average_covariance_multipoles(3, [0.9], [1.1], [0.2], [1e-3 * H ** 3], [50 / H], ls,
                                          sep, ipk, ipk2)
    for i, l1 in enumerate(ls):
        for j, l2 in enumerate(ls):
            d = golden[f"avg_multipoles_covariance_{l1}{l2}"]
            assert np.allclose(d[:, 0] / H, np.repeat(sep, len(sep)))
            assert np.allclose(cov[0, i, :, j, :].ravel(), d[:, 2], rtol=5e-4), (
                l1, l2, cov[0, i, :, j, :].ravel() / d[:, 2] - 1)
