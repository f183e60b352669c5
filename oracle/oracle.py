"""ctypes bindings of the CPU oracle (test infrastructure only).

Wraps ``oracle/_build/libcoffe_oracle.so`` (built by ``make -C oracle``).  Every
function here restates the reference algorithm cited in ``coffe_oracle.h``.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

_HERE = Path(__file__).resolve().parent
_LIB_PATH = _HERE / "_build" / "libcoffe_oracle.so"
_lib = None

CONTRIB_DEN = 1
CONTRIB_RSD = 2
CONTRIB_LEN = 4
H0 = 1.0 / 2997.92458  # h/Mpc
N_SMALL_R = 42

_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_ip = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")


def build(force: bool = False) -> Path:
    """Compile the oracle with its Makefile (gcc + OpenMP)."""
    if force or not _LIB_PATH.exists() or any(
        (_HERE / f).stat().st_mtime > _LIB_PATH.stat().st_mtime
        for f in ("coffe_oracle.c", "coffe_oracle.h", "../coffe_gb300/csrc/gk61_table.h")
    ):
        subprocess.run(["make", "-C", str(_HERE)], check=True, capture_output=True)
    return _LIB_PATH


class _Cosmo(C.Structure):
    _fields_ = [
        ("Omega0_cdm", C.c_double),
        ("Omega0_baryon", C.c_double),
        ("Omega0_gamma", C.c_double),
        ("Omega0_de", C.c_double),
        ("h", C.c_double),
    ]


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(str(_LIB_PATH))
        L.or_spline_eval_array.argtypes = [C.c_int, _dp, _dp, C.c_size_t, _dp, _dp, C.c_size_t]
        L.or_spline_coeffs.argtypes = [C.c_int, _dp, _dp, C.c_size_t, _dp, _dp, _dp]
        L.or_lgamma_c.argtypes = [C.c_double, C.c_double, C.POINTER(C.c_double), C.POINTER(C.c_double)]
        L.or_sph_bessel.argtypes = [C.c_int, C.c_double]
        L.or_sph_bessel.restype = C.c_double
        L.or_legendre.argtypes = [C.c_int, C.c_double]
        L.or_legendre.restype = C.c_double
        L.or_fft.argtypes = [_dp, _dp, C.c_size_t, C.c_int]
        L.or_twofast_selectqnu.argtypes = [C.c_double, C.c_double]
        L.or_twofast_selectqnu.restype = C.c_double
        L.or_twofast_1bessel.argtypes = [_dp, _dp, C.c_size_t, _dp, _dp, C.c_size_t] + [C.c_double] * 6
        L.or_integral_table.argtypes = [_dp, _dp, C.c_size_t, C.c_int, C.c_int, C.c_size_t,
                                        C.c_double, C.c_double, C.c_int, _dp, _dp]
        L.or_integral_direct.argtypes = [_dp, _dp, C.c_size_t, C.c_int, C.c_int, C.c_double,
                                         C.c_double, C.c_double]
        L.or_integral_direct.restype = C.c_double
        L.or_divergent_i40.argtypes = [_dp, _dp, C.c_size_t, C.c_double, C.c_double, _dp,
                                       C.c_size_t, _dp, _dp, C.c_int]
        L.or_divergent_separations.argtypes = [_dp, C.c_size_t]
        L.or_divergent_separations.restype = C.c_size_t
        L.or_renormalization_grid.argtypes = [_dp, _dp, C.c_size_t, C.c_double, C.c_double, _dp,
                                              C.c_size_t, _dp, C.c_size_t, _dp, C.c_int]
        L.or_background_nodes.argtypes = [C.POINTER(_Cosmo), C.c_size_t] + [_dp] * 9
        L.or_gauss_legendre.argtypes = [C.c_size_t, _dp, _dp]
        L.or_model_new.restype = C.c_void_p
        L.or_model_free.argtypes = [C.c_void_p]
        L.or_model_set_background.argtypes = [C.c_void_p, _dp, _dp, _dp, _dp, _dp, _dp,
                                              C.c_size_t, C.c_double, C.c_double]
        L.or_model_set_bias.argtypes = [C.c_void_p, C.c_int, _dp, _dp, C.c_size_t]
        L.or_model_set_integral.argtypes = [C.c_void_p, C.c_int, C.c_int, _dp, _dp, C.c_size_t]
        L.or_xi_nonintegrated.argtypes = [C.c_void_p, C.c_int, C.c_double, C.c_double, C.c_double]
        L.or_xi_nonintegrated.restype = C.c_double
        L.or_multipole_nonintegrated.argtypes = [C.c_void_p, C.c_int, C.c_double, C.c_double,
                                                 C.c_int, C.c_double]
        L.or_multipole_nonintegrated.restype = C.c_double
        L.or_multipole_nonintegrated_gl.argtypes = [C.c_void_p, C.c_int, C.c_double, C.c_double,
                                                    C.c_int, C.c_size_t]
        L.or_multipole_nonintegrated_gl.restype = C.c_double
        L.or_multipoles_batch.argtypes = [C.c_void_p, C.c_int, _dp, _dp, _ip, C.c_size_t,
                                          C.c_double, _dp, C.c_int]
        L.or_last_qag_intervals.restype = C.c_int
        L.or_xi_single_integrated.argtypes = [C.c_void_p, C.c_int] + [C.c_double] * 4
        L.or_xi_single_integrated.restype = C.c_double
        L.or_xi_double_integrated.argtypes = [C.c_void_p, C.c_int] + [C.c_double] * 5
        L.or_xi_double_integrated.restype = C.c_double
        L.or_integral_table_half.argtypes = [_dp, _dp, C.c_size_t, C.c_int, C.c_int, C.c_size_t,
                                             C.c_double, C.c_double, _dp, _dp]
        L.or_flatsky_density_lensing.argtypes = [C.c_void_p, C.c_double, C.c_double, C.c_int]
        L.or_flatsky_density_lensing.restype = C.c_double
        L.or_flatsky_lensing_lensing.argtypes = [C.c_void_p, C.c_double, C.c_double, C.c_int,
                                                 C.c_double]
        L.or_flatsky_lensing_lensing.restype = C.c_double
        L.or_legendre_integral.argtypes = [C.c_int] * 4
        L.or_legendre_integral.restype = C.c_double
        L.or_twobessel_diag.argtypes = [_dp, _dp, C.c_size_t] + [C.c_double] * 5 + [_dp, _dp]
        L.or_covariance_fftlog.argtypes = [_dp, _dp, C.c_size_t, C.c_int, C.c_int, C.c_int,
                                           C.c_size_t, _dp, C.c_size_t, C.c_double, C.c_double,
                                           _dp]
        L.or_covariance_integral.argtypes = [_dp, _dp, C.c_size_t, C.c_int, C.c_double,
                                             C.c_double, C.c_int, C.c_int, C.c_double,
                                             C.c_double, C.c_double, C.c_int]
        L.or_covariance_integral.restype = C.c_double
        L.or_covariance_multipoles.argtypes = [C.c_void_p, C.c_int, C.c_size_t, _dp, _dp, _dp,
                                               _dp, _dp, _dp, C.c_size_t, _ip, C.c_size_t, _dp,
                                               _dp, _dp, _dp]
        L.or_covariance_multipoles_v.argtypes = [C.c_void_p, C.c_int, C.c_size_t, _dp, _dp, _dp,
                                                 _dp, _dp, C.c_size_t, _ip, C.c_size_t, _dp,
                                                 _dp, _dp, _dp]
        L.or_average_covariance_volume.argtypes = [C.c_void_p, C.c_double, C.c_double,
                                                   C.c_double]
        L.or_average_covariance_volume.restype = C.c_double
        L.or_average_multipoles_batch.argtypes = [C.c_void_p, C.c_int, _dp, _dp, _dp, _ip,
                                                  C.c_size_t, C.c_size_t, C.c_size_t,
                                                  C.c_size_t, _dp, C.c_int]
        L.or_average_multipoles_batch.restype = C.c_int
        L.or_corrfunc_batch.argtypes = [C.c_void_p, C.c_int, _dp, _dp, _dp, C.c_size_t,
                                        C.c_size_t, _dp, C.c_int]
        L.or_corrfunc_batch.restype = C.c_int
        L.or_multipoles_lensing_batch.argtypes = [C.c_void_p, C.c_int, _dp, _dp, C.c_size_t,
                                                  C.c_int, _ip, C.c_size_t, C.c_size_t, _dp,
                                                  C.c_int]
        _lib = L
    return _lib


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


# ----------------------------------------------------------------- primitives
def spline_eval(kind: str, x, y, xq):
    t = {"cspline": 0, "akima": 1, "linear": 2}[kind]
    x, y, xq = _f64(x), _f64(y), _f64(np.atleast_1d(xq))
    out = np.empty_like(xq)
    if lib().or_spline_eval_array(t, x, y, len(x), xq, out, len(xq)) != 0:
        raise ValueError("spline init failed")
    return out


def spline_coeffs(kind: str, x, y):
    t = {"cspline": 0, "akima": 1, "linear": 2}[kind]
    x, y = _f64(x), _f64(y)
    n = len(x)
    b, c, d = (np.zeros(n) for _ in range(3))
    if lib().or_spline_coeffs(t, x, y, n, b, c, d) != 0:
        raise ValueError("spline init failed")
    return b[:-1], c[:-1], d[:-1]


def lgamma_c(z: complex) -> complex:
    rr, ri = C.c_double(), C.c_double()
    lib().or_lgamma_c(z.real, z.imag, C.byref(rr), C.byref(ri))
    return complex(rr.value, ri.value)


def sph_bessel(l: int, x: float) -> float:
    return lib().or_sph_bessel(int(l), float(x))


def legendre(l: int, x: float) -> float:
    return lib().or_legendre(int(l), float(x))


def fft(x, sign=-1):
    x = np.asarray(x, dtype=np.complex128)
    re, im = _f64(x.real.copy()), _f64(x.imag.copy())
    lib().or_fft(re, im, len(x), int(sign))
    return re + 1j * im


def gauss_legendre(n: int):
    x, w = np.zeros(n), np.zeros(n)
    lib().or_gauss_legendre(n, x, w)
    return x, w


def selectqnu(l: float, nu: float) -> float:
    return lib().or_twofast_selectqnu(float(l), float(nu))


def twofast_1bessel(k, pk, N, l, nu, r0, k0, kmin, kmax):
    k, pk = _f64(k), _f64(pk)
    ox, oy = np.zeros(N), np.zeros(N)
    if lib().or_twofast_1bessel(ox, oy, N, k, pk, len(k), l, nu, r0, k0, kmin, kmax) != 0:
        raise ValueError("twofast_1bessel failed")
    return ox, oy


def integral_table(k, pk, n, l, N, kmin=None, kmax=None, with_small_r=True):
    """Full I_l^n table (N + 43 points) as coffe_integrals_renormalizable."""
    k, pk = _f64(k), _f64(pk)
    kmin = float(k[0] if kmin is None else kmin)
    kmax = float(k[-1] if kmax is None else kmax)
    ox, oy = np.zeros(N + N_SMALL_R + 1), np.zeros(N + N_SMALL_R + 1)
    if lib().or_integral_table(k, pk, len(k), n, l, N, kmin, kmax, int(with_small_r), ox, oy) != 0:
        raise ValueError("integral table failed")
    return ox, oy


def integral_direct(k, pk, n, l, r, kmin=None, kmax=None):
    k, pk = _f64(k), _f64(pk)
    kmin = float(k[0] if kmin is None else kmin)
    kmax = float(k[-1] if kmax is None else kmax)
    return lib().or_integral_direct(k, pk, len(k), n, l, float(r), kmin, kmax)


def divergent_separations():
    """The fixed separations (Mpc) of the divergent integral (integrals.c:76-103)."""
    n = lib().or_divergent_separations(np.zeros(1), 0)
    out = np.zeros(n)
    lib().or_divergent_separations(out, n)
    return out


def divergent_i40(k, pk, r, kmin=None, kmax=None, nthreads=0):
    """(r^4 I^4_0(r), r^4 x its r = 0 renormalisation integral), both / 2 pi^2, at
    separations r (integrals.c:773-845)."""
    k, pk, r = _f64(k), _f64(pk), _f64(np.atleast_1d(r))
    kmin = float(k[0] if kmin is None else kmin)
    kmax = float(k[-1] if kmax is None else kmax)
    res, res0 = np.zeros(len(r)), np.zeros(len(r))
    if lib().or_divergent_i40(k, pk, len(k), kmin, kmax, r, len(r), res, res0, nthreads) != 0:
        raise ValueError("divergent integral failed")
    return res, res0


def renormalization_grid(k, pk, chi1, chi2, kmin=None, kmax=None, nthreads=0):
    """out[b, a] = (1/2pi^2) int P j0(k chi1[a]) j0(k chi2[b]) / k^2 dk
    (integrals.c:424-444)."""
    k, pk = _f64(k), _f64(pk)
    c1, c2 = _f64(np.atleast_1d(chi1)), _f64(np.atleast_1d(chi2))
    kmin = float(k[0] if kmin is None else kmin)
    kmax = float(k[-1] if kmax is None else kmax)
    out = np.zeros((len(c2), len(c1)))
    if lib().or_renormalization_grid(k, pk, len(k), kmin, kmax, c1, len(c1), c2, len(c2), out,
                                     nthreads) != 0:
        raise ValueError("renormalisation grid failed")
    return out


def background_nodes(omega_m=0.3, omega_baryon=0.05, omega_gamma=9e-5, h=0.67, bins=10000):
    """Background node arrays on z_i = 15 i/(bins-1) (flat LCDM, w = -1)."""
    c = _Cosmo(omega_m - omega_baryon, omega_baryon, omega_gamma,
               1.0 - (omega_m + omega_gamma), h)
    names = ["z", "a", "Hz", "confH", "confHp", "D1", "f", "chi", "D1_unnormalised"]
    arrs = [np.zeros(bins) for _ in names]
    if lib().or_background_nodes(C.byref(c), bins, *arrs) != 0:
        raise ValueError("background failed")
    return dict(zip(names, arrs))


class Model:
    """Background + bias + integral splines: the inputs of the multipole integrands."""

    def __init__(self, bg: dict, h: float, omega_m: float):
        self._p = lib().or_model_new()
        z = _f64(bg["z"])
        lib().or_model_set_background(self._p, z, _f64(bg["chi"]), _f64(bg["D1"]),
                                      _f64(bg["f"]), _f64(bg["a"]), _f64(bg["confH"]),
                                      len(z), float(h), float(omega_m))
        self.h = h

    def __del__(self):
        if getattr(self, "_p", None):
            lib().or_model_free(self._p)
            self._p = None

    def set_bias(self, which: int, z, v):
        if lib().or_model_set_bias(self._p, which, _f64(z), _f64(v), len(z)) != 0:
            raise ValueError("bias spline failed")

    def set_integral(self, n: int, l: int, x, y):
        x, y = _f64(x), _f64(y)
        if lib().or_model_set_integral(self._p, n, l, x, y, len(x)) != 0:
            raise ValueError("integral spline failed")

    def xi(self, contrib, z_mean, mu, sep):
        return lib().or_xi_nonintegrated(self._p, contrib, z_mean, mu, sep)

    def multipole(self, contrib, z_mean, sep, l, epsrel=1e-5):
        return lib().or_multipole_nonintegrated(self._p, contrib, z_mean, sep, l, epsrel)

    def multipole_gl(self, contrib, z_mean, sep, l, n_mu):
        return lib().or_multipole_nonintegrated_gl(self._p, contrib, z_mean, sep, l, n_mu)

    def multipoles_batch(self, contrib, z_mean, sep, l, epsrel=1e-5, nthreads=0):
        z_mean, sep = _f64(z_mean), _f64(sep)
        l = np.ascontiguousarray(l, dtype=np.int32)
        out = np.zeros(len(sep))
        lib().or_multipoles_batch(self._p, contrib, z_mean, sep, l, len(sep), epsrel, out,
                                  int(nthreads))
        return out


    def set_integral_half(self, n_num: int, l_num: int, x, y):
        """a half-integer table I^{n_num/2}_{l_num/2}"""
        self.set_integral(10000 + n_num, 10000 + l_num, x, y)

    def flatsky_density_lensing(self, z_mean, sep, l):
        return lib().or_flatsky_density_lensing(self._p, z_mean, sep, l)

    def flatsky_lensing_lensing(self, z_mean, sep, l, epsrel=1e-5):
        return lib().or_flatsky_lensing_lensing(self._p, z_mean, sep, l, epsrel)

    def xi_single(self, contrib, z_mean, mu, sep, x):
        return lib().or_xi_single_integrated(self._p, contrib, z_mean, mu, sep, x)

    def xi_double(self, contrib, z_mean, mu, sep, x1, x2):
        return lib().or_xi_double_integrated(self._p, contrib, z_mean, mu, sep, x1, x2)

    def average_multipoles(self, contrib, z_min, z_max, sep, l, n_z=32, n_mu=64, n_x=128,
                           nthreads=0):
        """Redshift-averaged multipoles at (z_min, z_max, sep, l) points (broadcast):
        n_z Gauss-Legendre nodes in the redshift direction, the multipole per node
        (QAG in mu; with len the lensing rules n_mu x n_x)."""
        a, b, r, ll = np.broadcast_arrays(np.asarray(z_min, dtype=np.float64),
                                          np.asarray(z_max, dtype=np.float64),
                                          np.asarray(sep, dtype=np.float64), np.asarray(l))
        a, b, r = _f64(a.ravel()), _f64(b.ravel()), _f64(r.ravel())
        ll = np.ascontiguousarray(ll.ravel(), dtype=np.int32)
        out = np.zeros(len(r))
        lib().or_average_multipoles_batch(self._p, contrib, a, b, r, ll, len(r), int(n_z),
                                          int(n_mu), int(n_x), out, int(nthreads))
        return out

    def corrfunc(self, contrib, z_mean, mu, sep, n_x=256, nthreads=0):
        """Correlation function at (z_mean, mu, sep) points (broadcast): the
        nonintegrated den/rsd terms plus, with len, the lensing integrals at mu
        (split Gauss-Legendre lines of n_x nodes)."""
        z, m, r = np.broadcast_arrays(np.asarray(z_mean, dtype=np.float64),
                                      np.asarray(mu, dtype=np.float64),
                                      np.asarray(sep, dtype=np.float64))
        z, m, r = _f64(z.ravel()), _f64(m.ravel()), _f64(r.ravel())
        out = np.zeros(len(r))
        lib().or_corrfunc_batch(self._p, contrib, z, m, r, len(r), int(n_x), out, int(nthreads))
        return out

    def multipoles_lensing(self, contrib, z_mean, sep, ls, n_mu, n_x, nthreads=0):
        """Lensing multipoles (single + double integrated terms) with product
        Gauss-Legendre rules; returns (len(sep), len(ls))."""
        sep = _f64(np.atleast_1d(sep))
        z = _f64(np.broadcast_to(np.asarray(z_mean, dtype=np.float64), sep.shape))
        la = np.ascontiguousarray(ls, dtype=np.int32)
        out = np.zeros((len(sep), len(la)))
        if lib().or_multipoles_lensing_batch(self._p, contrib, z, sep, len(sep), len(la), la,
                                             int(n_mu), int(n_x), out, int(nthreads)) != 0:
            raise MemoryError("lensing multipoles failed")
        return out


    def covariance_multipoles(self, contrib, z_mean, deltaz, fsky, density, pixelsize, ls, sep,
                              ipk, ipk2, density2=None):
        """Multipole covariance (z, l1, r1, l2, r2) from the double-Bessel
        integrals ipk / ipk2 of shape (nl, nl, nsep(n), nsep(m))."""
        z = _f64(np.atleast_1d(z_mean))
        nz = len(z)
        arr = [_f64(np.broadcast_to(np.asarray(a, dtype=np.float64), z.shape))
               for a in (deltaz, fsky, density, density if density2 is None else density2,
                         pixelsize)]
        la = np.ascontiguousarray(ls, dtype=np.int32)
        sep = _f64(sep)
        nl, ns = len(la), len(sep)
        out = np.zeros(nz * nl * ns * nl * ns)
        lib().or_covariance_multipoles(self._p, contrib, nz, z, *arr, nl, la, ns, sep,
                                       _f64(ipk).ravel(), _f64(ipk2).ravel(), out)
        return out.reshape(nz, nl, ns, nl, ns)


    def average_covariance_multipoles(self, contrib, z_min, z_max, fsky, density, pixelsize, ls,
                                      sep, ipk, ipk2, density2=None):
        """Covariance of the redshift-averaged multipoles (window, l1, r1, l2, r2):
        the bins at (z_min + z_max) / 2 with the windows' effective volumes
        (covariance.c:811-840)."""
        a, b = _f64(np.atleast_1d(z_min)), _f64(np.atleast_1d(z_max))
        nz = len(a)
        arr = [_f64(np.broadcast_to(np.asarray(x, dtype=np.float64), a.shape))
               for x in (fsky, density, density if density2 is None else density2, pixelsize)]
        zb = _f64((a + b) / 2)
        V = _f64([lib().or_average_covariance_volume(self._p, a[i], b[i], arr[0][i])
                  for i in range(nz)])
        la = np.ascontiguousarray(ls, dtype=np.int32)
        sep = _f64(sep)
        nl, ns = len(la), len(sep)
        out = np.zeros(nz * nl * ns * nl * ns)
        lib().or_covariance_multipoles_v(self._p, contrib, nz, zb, V, arr[1], arr[2], arr[3], nl,
                                         la, ns, sep, _f64(ipk).ravel(), _f64(ipk2).ravel(), out)
        return out.reshape(nz, nl, ns, nl, ns)


def integral_table_half(k, pk, n_num, l_num, N, kmin=None, kmax=None):
    """FFTLog table of I^{n_num/2}_{l_num/2} (small-r entries NaN)."""
    k, pk = _f64(k), _f64(pk)
    kmin = float(k[0] if kmin is None else kmin)
    kmax = float(k[-1] if kmax is None else kmax)
    n_out = N + 43
    x, y = np.zeros(n_out), np.zeros(n_out)
    if lib().or_integral_table_half(k, pk, len(k), int(n_num), int(l_num), int(N), kmin, kmax,
                                    x, y) != 0:
        raise ValueError("half-integer table failed")
    return x, y


def legendre_integral(n, m, a, b) -> float:
    return lib().or_legendre_integral(n, m, a, b)


def twobessel_diag(k, diag, l1, l2, nu1=1.01, nu2=1.01, c_window_width=0.25):
    """2D FFTLog of a diagonal kernel; returns (r, out[a, b] at (r[a], r[b]))."""
    k, diag = _f64(k), _f64(diag)
    N = len(k)
    r = np.zeros(N)
    out = np.zeros((N, N))
    if lib().or_twobessel_diag(k, diag, N, l1, l2, nu1, nu2, c_window_width, r, out) != 0:
        raise ValueError("twobessel failed")
    return r, out


def covariance_fftlog(k, pk, power, l1, l2, N, sep, kmin=None, kmax=None):
    """covariance_integrate_fftlog: array [n, m] at (sep[m], sep[n])."""
    k, pk, sep = _f64(k), _f64(pk), _f64(sep)
    kmin = float(k[0] if kmin is None else kmin)
    kmax = float(k[-1] if kmax is None else kmax)
    out = np.zeros((len(sep), len(sep)))
    if lib().or_covariance_fftlog(k, pk, len(k), int(power), int(l1), int(l2), int(N), sep,
                                  len(sep), kmin, kmax, out) != 0:
        raise ValueError("covariance fftlog failed")
    return out


def covariance_integral(k, pk, power, r1, r2, l1, l2, kmin=None, kmax=None, epsrel=1e-5,
                        power_of_spline=False):
    """2/pi int k^2 P^power j_l1(k r1) j_l2(k r2) dk by QAG; P^power as the
    reference's direct method splines it (Akima of the node values P^power),
    or as the FFTLog path samples it (power of the Akima spline of P)."""
    k, pk = _f64(k), _f64(pk)
    kmin = float(k[0] if kmin is None else kmin)
    kmax = float(k[-1] if kmax is None else kmax)
    return lib().or_covariance_integral(k, pk, len(k), int(power), float(r1), float(r2), int(l1),
                                        int(l2), kmin, kmax, float(epsrel),
                                        int(bool(power_of_spline)))


def last_qag_intervals() -> int:
    return lib().or_last_qag_intervals()
