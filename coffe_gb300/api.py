"""Python host API over the C ABI: a context object and a ``Coffe`` class that
mirrors the reference's Python wrapper (python/coffe/coffe.pyx) for the
correlation-function hot path.

Units follow the reference: k in 1/Mpc, P(k) in Mpc^3, separations in Mpc.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from typing import Iterable, List, Sequence, Tuple

import numpy as np

from . import _lib
from ._lib import CoffeGpuError, Cosmology

# the default full-sky integrals of coffe_integrals_init (integrals.c:599-608)
DEFAULT_TERMS: Tuple[Tuple[int, int], ...] = (
    (0, 0), (0, 2), (0, 4), (1, 1), (1, 3), (2, 0), (2, 2), (3, 1),
)
DEN_RSD_TERMS: Tuple[Tuple[int, int], ...] = ((0, 0), (0, 2), (0, 4))
COFFE_H0 = 1.0 / 2997.92458  # h/Mpc (common.h:76)


def _dptr(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _iptr(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_int))


def _lptr(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_int64))


def _addr(a: np.ndarray) -> int:
    """Address of a numpy array's data (for the void * arguments)."""
    return a.__array_interface__["data"][0]


def _f64(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float64)


def _precision(p) -> int:
    if p in (0, "fp64", "double", "float64"):
        return _lib.FP64
    if p in (1, "mixed", "fp32"):
        return _lib.MIXED
    if p in (2, "fp64-fastalg"):
        return _lib.FP64_FASTALG
    raise ValueError(f"unknown precision {p!r} (use 'fp64' or 'mixed')")


class Context:
    """One ``coffe_gpu_ctx_t``: device buffers, a stream and the cached tables."""

    def __init__(self, device: int = 0):
        self._L = _lib.load()
        self._ctx = C.c_void_p()
        st = self._L.coffe_gpu_ctx_create(int(device), C.byref(self._ctx))
        if st != 0:
            raise CoffeGpuError(st, "coffe_gpu_ctx_create", "no usable CUDA device")
        self.device = device
        self.N = None
        self.terms: Tuple[Tuple[int, int], ...] = ()
        self.n_spectra = 0
        self.precision = None

    # -------------------------------------------------------------- plumbing
    def _check(self, st: int, what: str):
        if st != 0:
            detail = self._L.coffe_gpu_last_error(self._ctx)
            raise CoffeGpuError(st, what, detail.decode() if detail else "")

    def close(self):
        if getattr(self, "_ctx", None) and self._ctx.value:
            self._L.coffe_gpu_ctx_destroy(self._ctx)
            self._ctx = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    @property
    def handle(self) -> int:
        return self._ctx.value

    def synchronize(self):
        self._check(self._L.coffe_gpu_synchronize(self._ctx), "synchronize")

    def set_stream(self, stream_ptr: int | None):
        self._check(self._L.coffe_gpu_set_stream(self._ctx, C.c_void_p(stream_ptr or 0)),
                    "set_stream")

    def launch_count(self) -> int:
        return int(self._L.coffe_gpu_launch_count(self._ctx))

    def set_kernel_timing(self, enable: bool = True):
        """Per-kernel CUDA-event timing of this context's launches (see
        :meth:`kernel_times`)."""
        self._check(self._L.coffe_gpu_set_kernel_timing(self._ctx, int(bool(enable))),
                    "set_kernel_timing")

    def kernel_times(self, reset: bool = True) -> dict:
        """{kernel name: (launches, total ms)} recorded since the last reset."""
        cap = 64
        names = (C.c_char_p * cap)()
        launches = (C.c_longlong * cap)()
        ms = (C.c_double * cap)()
        n = self._L.coffe_gpu_kernel_times(self._ctx, names, launches, ms, cap, int(bool(reset)))
        if n < 0:
            self._check(n, "kernel_times")
        return {names[i].decode(): (int(launches[i]), float(ms[i])) for i in range(min(n, cap))}

    def debug_fail_alloc(self, nth: int):
        """Make the nth device allocation from now fail (ENOMEM); 0 disarms."""
        self._check(self._L.coffe_gpu_debug_fail_alloc(self._ctx, int(nth)), "debug_fail_alloc")

    def measure_peak(self, kind: str) -> float:
        """Measured FLOP/s of this device for ``kind`` in "fp64", "fp32" or
        "fp32x2" (packed pair FMA): the roofline denominators of the
        compute-bound kernels."""
        k = {"fp64": _lib.PEAK_FP64, "fp32": _lib.PEAK_FP32, "fp32x2": _lib.PEAK_FP32X2}[kind]
        v = C.c_double()
        self._check(self._L.coffe_gpu_measure_peak(self._ctx, k, C.byref(v)), "measure_peak")
        return float(v.value)

    # ------------------------------------------------------------- tuning
    def set_autotune(self, enable: bool = True):
        """Benchmark mode: the first table build and mixed multipole call of
        each shape time every candidate launch configuration and keep the
        fastest (calls under stream capture never time)."""
        self._check(self._L.coffe_gpu_set_autotune(self._ctx, int(bool(enable))), "set_autotune")

    def tuning(self) -> dict:
        """Configuration used by the most recent table build and mixed
        multipole call."""
        t = _lib.Tuning()
        self._check(self._L.coffe_gpu_get_tuning(self._ctx, C.byref(t)), "get_tuning")
        return {name: getattr(t, name) for name, _ in _lib.Tuning._fields_}

    def set_tuning(self, **cfg):
        """Default configuration (keys of :meth:`tuning`; missing keys keep their
        current value); forgets the configurations chosen by autotuning."""
        cur = self.tuning()
        unknown = set(cfg) - set(cur)
        if unknown:
            raise ValueError(f"unknown tuning keys {sorted(unknown)}")
        cur.update(cfg)
        t = _lib.Tuning(**{k: int(v) for k, v in cur.items()})
        self._check(self._L.coffe_gpu_set_tuning(self._ctx, C.byref(t)), "set_tuning")

    def last_retries(self) -> int:
        """(separation, l) outputs of the last multipoles call that needed the
        adaptive bisection after the first GK61 panel."""
        return int(self._L.coffe_gpu_multipoles_retries(self._ctx))

    # ------------------------------------------------------------ background
    def background_init(self, omega_m=0.3, omega_baryon=0.05, omega_gamma=9e-5, h=0.67,
                        bins=10000):
        c = Cosmology(omega_m - omega_baryon, omega_baryon, omega_gamma,
                      1.0 - (omega_m + omega_gamma), h, int(bins))
        self._check(self._L.coffe_gpu_background_init(self._ctx, C.byref(c)), "background_init")
        self.bins = int(bins)

    def background_set(self, z, chi, D1, f, a, conformal_Hz, omega_m, h):
        arrs = [_f64(x) for x in (z, chi, D1, f, a, conformal_Hz)]
        n = len(arrs[0])
        if any(len(x) != n for x in arrs):
            raise ValueError("background arrays must have equal lengths")
        self._check(self._L.coffe_gpu_background_set(self._ctx, *map(_dptr, arrs), n,
                                                     float(omega_m), float(h)), "background_set")
        self.bins = n

    def background(self, with_H: bool = True) -> dict:
        n = self.bins
        names = ["z", "chi", "D1", "f", "a", "Hz", "conformal_Hz", "conformal_Hz_prime"]
        arrs = {k: np.zeros(n) for k in names}
        ptrs = [_dptr(arrs[k]) for k in names]
        if not with_H:
            ptrs[5] = None
            ptrs[7] = None
        self._check(self._L.coffe_gpu_background_get(self._ctx, *ptrs), "background_get")
        return arrs

    def set_bias(self, which: int, z, value):
        z, v = _f64(z), _f64(value)
        self._check(self._L.coffe_gpu_set_bias(self._ctx, int(which), _dptr(z), _dptr(v), len(z)),
                    "set_bias")

    # ------------------------------------------------------------- integrals
    def integrals_init(self, k, pk, terms: Sequence[Tuple[int, int]] = DEFAULT_TERMS,
                       N: int = 4096, precision="fp64", small_r: bool = True,
                       tables_df: bool = False, sync: bool = True):
        """FFTLog tables of I_l^n for each spectrum row of ``pk`` (shape (S, nk)).
        ``tables_df`` (mixed precision): double-float inverse transforms too.
        ``sync=False``: return once ``pk`` has been copied to the device, with
        the tables still being made (COFFE_GPU_ASYNC); their device-side errors
        surface at the next call that checks (:meth:`multipoles`,
        :meth:`synchronize`)."""
        k = _f64(k)
        pk = _f64(np.atleast_2d(pk))
        if pk.shape[1] != len(k):
            raise ValueError("pk must have shape (n_spectra, len(k))")
        # a term is (n, l) or (n, l, half): half = 1 makes n, l numerators of n/2, l/2
        n = np.ascontiguousarray([t[0] for t in terms], dtype=np.int32)
        l = np.ascontiguousarray([t[1] for t in terms], dtype=np.int32)
        half = np.ascontiguousarray([t[2] if len(t) > 2 else 0 for t in terms], dtype=np.int32)
        prec = _precision(precision)
        flags = ((_lib.SMALL_R if small_r else 0) | (_lib.TABLES_DF if tables_df else 0)
                 | (0 if sync else _lib.ASYNC))
        self._check(self._L.coffe_gpu_integrals_init_ex(self._ctx, _addr(k), _addr(pk),
                                                        pk.shape[0], len(k), _addr(n), _addr(l),
                                                        _addr(half), len(terms), int(N), prec,
                                                        flags), "integrals_init")
        self.N = int(N)
        self.terms = tuple((int(t[0]), int(t[1])) + ((1,) if len(t) > 2 and t[2] else ())
                           for t in terms)
        self.n_spectra = pk.shape[0]
        self.precision = prec

    def set_flatsky(self, local_nonlocal: bool = False, nonlocal_: bool = False):
        """Flat-sky forms of density-lensing (local_nonlocal) and lensing-lensing
        (nonlocal_) in the multipoles, as the reference's flatsky flags."""
        self._check(self._L.coffe_gpu_set_flatsky(self._ctx, int(bool(local_nonlocal)),
                                                  int(bool(nonlocal_))), "set_flatsky")

    def table_len(self) -> int:
        return int(self._L.coffe_gpu_integral_table_len(self.N))

    def _term(self, n: int, l: int) -> int:
        try:
            return self.terms.index((n, l))
        except ValueError:
            raise ValueError(f"Cannot find integral with n = {n}, l = {l}") from None

    def integral_table(self, spectrum: int, n: int, l: int):
        m = self.table_len()
        x, y = np.zeros(m), np.zeros(m)
        self._check(self._L.coffe_gpu_integral_get(self._ctx, int(spectrum), self._term(n, l),
                                                   _dptr(x), _dptr(y)), "integral_get")
        return x, y

    def integral_eval(self, spectrum: int, n: int, l: int, r):
        r = _f64(np.atleast_1d(r))
        out = np.zeros(len(r))
        self._check(self._L.coffe_gpu_integral_eval(self._ctx, int(spectrum), self._term(n, l),
                                                    _dptr(r), len(r), _dptr(out)), "integral_eval")
        return out

    # ------------------------------------------------------------ multipoles
    def multipoles(self, req_spectrum, req_z_mean, req_offset, sep, ls=(0, 2, 4),
                   contrib=_lib.DEN | _lib.RSD, precision="fp64", epsrel=1e-5,
                   out=None) -> np.ndarray:
        """Batched multipoles; returns an array of shape (len(sep), len(ls)).
        ``out``: optional C-contiguous float64 array of that shape to fill; in
        page-locked host memory (e.g. a pinned torch tensor's ``.numpy()``) the
        den/rsd kernels write it directly, with no device copy and download."""
        rs = np.ascontiguousarray(req_spectrum, dtype=np.int32)
        rz = _f64(req_z_mean)
        ro = np.ascontiguousarray(req_offset, dtype=np.int64)
        sp = _f64(sep)
        la = np.ascontiguousarray(ls, dtype=np.int32)
        if len(ro) != len(rs) + 1 or len(rz) != len(rs):
            raise ValueError("req_offset needs len(req_spectrum) + 1 entries")
        if out is None:
            out = np.zeros((max(len(sp), 1), len(la)))
        elif (out.dtype != np.float64 or not out.flags["C_CONTIGUOUS"] or
              out.shape[0] < max(len(sp), 1) or out.shape[1] != len(la)):
            raise ValueError("out must be a C-contiguous float64 array of shape (len(sep), len(ls))")
        self._check(self._L.coffe_gpu_multipoles(self._ctx, int(contrib), _precision(precision),
                                                 float(epsrel), len(rs), _addr(rs), _addr(rz),
                                                 _addr(ro), _addr(sp), len(la), _addr(la),
                                                 _addr(out), 0), "multipoles")
        return out[: len(sp)]

    def average_multipoles(self, win_spectrum, z_min, z_max, win_offset, sep, ls=(0, 2, 4),
                           contrib=_lib.DEN | _lib.RSD, precision="fp64", epsrel=1e-5,
                           n_z: int = 32) -> np.ndarray:
        """Redshift-averaged multipoles of the batched windows; returns an array
        of shape (len(sep), len(ls)) (average_multipoles.c:69-156)."""
        ws = np.ascontiguousarray(win_spectrum, dtype=np.int32)
        a, b = _f64(z_min), _f64(z_max)
        wo = np.ascontiguousarray(win_offset, dtype=np.int64)
        sp = _f64(sep)
        la = np.ascontiguousarray(ls, dtype=np.int32)
        if len(wo) != len(ws) + 1 or len(a) != len(ws) or len(b) != len(ws):
            raise ValueError("win_offset needs len(win_spectrum) + 1 entries")
        out = np.zeros((max(len(sp), 1), len(la)))
        self._check(self._L.coffe_gpu_average_multipoles(
            self._ctx, int(contrib), _precision(precision), float(epsrel), len(ws), _iptr(ws),
            _dptr(a), _dptr(b), _lptr(wo), _dptr(sp), len(la), _iptr(la), int(n_z), _dptr(out), 0),
            "average_multipoles")
        return out[: len(sp)]

    # ------------------------------------------------ divergent I^4_0 (integrals.c:773-914)
    @staticmethod
    def _k_range(k, kmin, kmax):
        return (float(k[0]) if kmin is None else float(kmin),
                float(k[-1]) if kmax is None else float(kmax))

    def divergent_integral(self, k, pk, sep=None, kmin=None, kmax=None):
        """The divergent integral at separations ``sep`` (Mpc, default the fixed
        ones the reference splines it on): returns (sep, result, result0) with
        result = r^4 I^4_0(r) and result0 = r^4 times its r = 0 renormalisation
        integral, both over 2 pi^2 (integrals.c:797-826).  k in 1/Mpc, P in Mpc^3,
        integrated over [kmin, kmax] (default the k range)."""
        k, pk = _f64(k), _f64(pk)
        sp = divergent_separations() if sep is None else _f64(np.atleast_1d(sep))
        lo, hi = self._k_range(k, kmin, kmax)
        res, res0 = np.zeros(len(sp)), np.zeros(len(sp))
        self._check(self._L.coffe_gpu_divergent_integral(self._ctx, _dptr(k), _dptr(pk), len(k),
                                                         lo, hi, _dptr(sp), len(sp), _dptr(res),
                                                         _dptr(res0)), "divergent_integral")
        return sp, res, res0

    def renormalization_grid(self, k, pk, chi1, chi2=None, kmin=None, kmax=None) -> np.ndarray:
        """out[b, a] = (1/2 pi^2) int P j0(k chi1[a]) j0(k chi2[b]) / k^2 dk over
        [kmin, kmax] (integrals.c:424-444); chi2 defaults to chi1."""
        k, pk = _f64(k), _f64(pk)
        c1 = _f64(np.atleast_1d(chi1))
        c2 = c1 if chi2 is None else _f64(np.atleast_1d(chi2))
        lo, hi = self._k_range(k, kmin, kmax)
        out = np.zeros((len(c2), len(c1)))
        self._check(self._L.coffe_gpu_renormalization_grid(self._ctx, _dptr(k), _dptr(pk), len(k),
                                                           lo, hi, _dptr(c1), len(c1), _dptr(c2),
                                                           len(c2), _dptr(out)),
                    "renormalization_grid")
        return out

    def corrfunc(self, req_spectrum, req_z_mean, req_offset, sep, mu,
                 contrib=_lib.DEN | _lib.RSD, precision="fp64") -> np.ndarray:
        """Correlation function at every (separation, mu) of the batched requests;
        returns an array of shape (len(sep), len(mu)) (corrfunc.c:55-141)."""
        rs = np.ascontiguousarray(req_spectrum, dtype=np.int32)
        rz = _f64(req_z_mean)
        ro = np.ascontiguousarray(req_offset, dtype=np.int64)
        sp = _f64(sep)
        mu = _f64(np.atleast_1d(mu))
        if len(ro) != len(rs) + 1 or len(rz) != len(rs):
            raise ValueError("req_offset needs len(req_spectrum) + 1 entries")
        out = np.zeros((max(len(sp), 1), len(mu)))
        self._check(self._L.coffe_gpu_corrfunc(self._ctx, int(contrib), _precision(precision),
                                               len(rs), _iptr(rs), _dptr(rz), _lptr(ro),
                                               _dptr(sp), len(mu), _dptr(mu), _dptr(out), 0),
                    "corrfunc")
        return out[: len(sp)]

    def integrals_init_device(self, k, pk_dev, terms=DEN_RSD_TERMS, N: int = 4096,
                              precision="fp64", small_r: bool = False, sync: bool = True,
                              tables_df: bool = False):
        """Like :meth:`integrals_init` with P(k) already on the device (a CUDA
        float64 tensor of shape (S, nk)); ``sync=False`` only enqueues."""
        k = _f64(k)
        S, nk = int(pk_dev.shape[0]), int(pk_dev.shape[1])
        if nk != len(k):
            raise ValueError("pk must have shape (n_spectra, len(k))")
        n = np.ascontiguousarray([t[0] for t in terms], dtype=np.int32)
        l = np.ascontiguousarray([t[1] for t in terms], dtype=np.int32)
        flags = (_lib.PK_DEVICE | (_lib.SMALL_R if small_r else 0) | (0 if sync else _lib.ASYNC)
                 | (_lib.TABLES_DF if tables_df else 0))
        pk_ptr = C.cast(C.c_void_p(pk_dev.data_ptr()), C.POINTER(C.c_double))
        self._check(self._L.coffe_gpu_integrals_init(self._ctx, _dptr(k), pk_ptr, S, nk, _iptr(n),
                                                     _iptr(l), len(terms), int(N),
                                                     _precision(precision), flags),
                    "integrals_init")
        self.N = int(N)
        self.terms = tuple((int(a), int(b)) for a, b in terms)
        self.n_spectra = S
        self.precision = _precision(precision)

    def multipoles_scaled(self, req_spectrum, req_z_mean, req_offset, sep, n_sep: int, ls, out,
                          bias_scale=None, growth_scale=None, contrib=_lib.DEN | _lib.RSD):
        """Differentiable form of the den/rsd multipoles on CUDA tensors (first
        GK61 panel), with optional per-request bias / growth-rate scales."""
        P = lambda t, ty: None if t is None else C.cast(C.c_void_p(t.data_ptr()), C.POINTER(ty))
        la = np.ascontiguousarray(ls, dtype=np.int32)
        self._check(self._L.coffe_gpu_multipoles_scaled(
            self._ctx, int(contrib), int(req_spectrum.numel()), int(n_sep),
            P(req_spectrum, C.c_int), P(req_z_mean, C.c_double), P(req_offset, C.c_int64),
            P(sep, C.c_double), len(la), _iptr(la), P(bias_scale, C.c_double),
            P(growth_scale, C.c_double), P(out, C.c_double)), "multipoles_scaled")

    def multipoles_adjoint(self, req_spectrum, req_z_mean, req_offset, sep, n_sep: int, ls,
                           grad_out, grad_pk, grad_bias=None, grad_growth=None, bias_scale=None,
                           growth_scale=None, contrib=_lib.DEN | _lib.RSD):
        """Reverse-mode derivative of :meth:`multipoles_scaled` (CUDA tensors)."""
        P = lambda t, ty: None if t is None else C.cast(C.c_void_p(t.data_ptr()), C.POINTER(ty))
        la = np.ascontiguousarray(ls, dtype=np.int32)
        self._check(self._L.coffe_gpu_multipoles_adjoint(
            self._ctx, int(contrib), int(req_spectrum.numel()), int(n_sep),
            P(req_spectrum, C.c_int), P(req_z_mean, C.c_double), P(req_offset, C.c_int64),
            P(sep, C.c_double), len(la), _iptr(la), P(bias_scale, C.c_double),
            P(growth_scale, C.c_double), P(grad_out, C.c_double), P(grad_pk, C.c_double),
            P(grad_bias, C.c_double), P(grad_growth, C.c_double)), "multipoles_adjoint")

    def set_lensing_rule(self, n_mu: int = 128, n_x: int = 256):
        """Gauss-Legendre rule of the lensing terms: n_mu nodes in mu, n_x per x
        line (split in two panels at the line's integrand peak)."""
        self._check(self._L.coffe_gpu_set_lensing_rule(self._ctx, int(n_mu), int(n_x)),
                    "set_lensing_rule")

    def multipoles_async(self, req_spectrum, req_z_mean, req_offset, sep, n_sep: int, ls, out,
                         contrib=_lib.DEN | _lib.RSD, precision="fp64", epsrel=1e-5):
        """Enqueue-only multipoles on device tensors; ``ls`` is a host sequence.
        Errors surface at :meth:`synchronize`."""
        P = lambda t, ty: C.cast(C.c_void_p(t.data_ptr()), C.POINTER(ty))
        la = np.ascontiguousarray(ls, dtype=np.int32)
        self._check(self._L.coffe_gpu_multipoles_async(
            self._ctx, int(contrib), _precision(precision), float(epsrel),
            int(req_spectrum.numel()), int(n_sep), P(req_spectrum, C.c_int),
            P(req_z_mean, C.c_double), P(req_offset, C.c_int64), P(sep, C.c_double), len(la),
            _iptr(la), P(out, C.c_double)), "multipoles_async")

    def multipoles_noalloc(self, req_spectrum, req_z_mean, req_offset, sep, n_sep: int, ls, out,
                           contrib=_lib.DEN | _lib.RSD, precision="fp64", epsrel=1e-5):
        """:meth:`multipoles_async` without any device allocation by the library:
        scratch comes from a fixed array of the library (at most
        ``NOALLOC_MAX_OUTPUTS`` = n_sep * len(ls) outputs per call).  For callers
        whose device memory is all pooled up front, or who cannot have
        cudaMalloc/cudaFree stall the device mid-run.  Calls on one device share
        that array: serialise them (one stream).  The context's creation loads
        the array and the kernels, so the call itself allocates nothing."""
        P = lambda t, ty: C.cast(C.c_void_p(t.data_ptr()), C.POINTER(ty))
        la = np.ascontiguousarray(ls, dtype=np.int32)
        self._check(self._L.coffe_gpu_multipoles_noalloc(
            self._ctx, int(contrib), _precision(precision), float(epsrel),
            int(req_spectrum.numel()), int(n_sep), P(req_spectrum, C.c_int),
            P(req_z_mean, C.c_double), P(req_offset, C.c_int64), P(sep, C.c_double), len(la),
            _iptr(la), P(out, C.c_double)), "multipoles_noalloc")

    # ------------------------------------------------------------ covariance
    def covariance_integrals(self, k, pk, N, jobs, sep) -> np.ndarray:
        """2D-FFTLog double-Bessel integrals for jobs (power, l1, l2); returns
        (len(jobs), len(sep), len(sep)) with [q, n, m] at (r1 = sep[m], r2 = sep[n])."""
        k, pk, sep = _f64(k), _f64(pk), _f64(sep)
        p = np.ascontiguousarray([j[0] for j in jobs], dtype=np.int32)
        a = np.ascontiguousarray([j[1] for j in jobs], dtype=np.int32)
        b = np.ascontiguousarray([j[2] for j in jobs], dtype=np.int32)
        out = np.zeros((len(jobs), len(sep), len(sep)))
        self._check(self._L.coffe_gpu_covariance_integrals(
            self._ctx, _dptr(k), _dptr(pk), len(k), int(N), len(jobs), _iptr(p), _iptr(a),
            _iptr(b), _dptr(sep), len(sep), _dptr(out)), "covariance_integrals")
        return out

    def covariance_multipoles(self, k, pk, N, z_mean, deltaz, fsky, density1, density2,
                              pixelsize, ls, sep, contrib=_lib.DEN | _lib.RSD) -> np.ndarray:
        """Multipole covariance, shape (n_z, n_l, n_sep, n_l, n_sep) in the
        reference's (z, l1, r1, l2, r2) order."""
        k, pk, sep = _f64(k), _f64(pk), _f64(sep)
        z = _f64(np.atleast_1d(z_mean))
        per_z = [_f64(np.broadcast_to(np.asarray(v, dtype=np.float64), z.shape))
                 for v in (deltaz, fsky, density1, density2, pixelsize)]
        la = np.ascontiguousarray(ls, dtype=np.int32)
        out = np.zeros((len(z), len(la), len(sep), len(la), len(sep)))
        self._check(self._L.coffe_gpu_covariance_multipoles(
            self._ctx, int(contrib), _dptr(k), _dptr(pk), len(k), int(N), len(z), _dptr(z),
            *map(_dptr, per_z), len(la), _iptr(la), len(sep), _dptr(sep), _dptr(out)),
            "covariance_multipoles")
        return out

    def average_covariance_multipoles(self, k, pk, N, z_min, z_max, fsky, density1, density2,
                                      pixelsize, ls, sep, contrib=_lib.DEN | _lib.RSD) -> np.ndarray:
        """Covariance of the redshift-averaged multipoles, shape (n_win, n_l,
        n_sep, n_l, n_sep) in the reference's (window, l1, r1, l2, r2) order."""
        k, pk, sep = _f64(k), _f64(pk), _f64(sep)
        a = _f64(np.atleast_1d(z_min))
        per_w = [_f64(np.broadcast_to(np.asarray(v, dtype=np.float64), a.shape))
                 for v in (z_max, fsky, density1, density2, pixelsize)]
        la = np.ascontiguousarray(ls, dtype=np.int32)
        out = np.zeros((len(a), len(la), len(sep), len(la), len(sep)))
        self._check(self._L.coffe_gpu_average_covariance_multipoles(
            self._ctx, int(contrib), _dptr(k), _dptr(pk), len(k), int(N), len(a), _dptr(a),
            *map(_dptr, per_w), len(la), _iptr(la), len(sep), _dptr(sep), _dptr(out)),
            "average_covariance_multipoles")
        return out

    def multipoles_device(self, req_spectrum, req_z_mean, req_offset, sep, ls, out,
                          contrib=_lib.DEN | _lib.RSD, precision="fp64", epsrel=1e-5):
        """Same as :meth:`multipoles` with CUDA tensors (int32, float64, int64,
        float64, int32, float64 out of shape (len(sep), len(ls))); no copies."""
        self._check(self._L.coffe_gpu_multipoles(
            self._ctx, int(contrib), _precision(precision), float(epsrel), int(req_spectrum.numel()),
            req_spectrum.data_ptr(), req_z_mean.data_ptr(), req_offset.data_ptr(),
            sep.data_ptr(), int(ls.numel()), ls.data_ptr(), out.data_ptr(), 1),
            "multipoles")


# ---------------------------------------------------------------- Coffe mirror
@dataclass
class Multipoles:
    """One multipole value (python/coffe/representation.py's Multipoles record)."""

    z: float
    r: float
    l: int
    value: float

    def to_dict(self):
        return {"z": self.z, "r": self.r, "l": self.l, "value": self.value}


@dataclass
class AverageMultipoles:
    """One redshift-averaged multipole (python/coffe/representation.py's
    AverageMultipoles record)."""

    z_min: float
    z_max: float
    r: float
    l: int
    value: float

    def to_dict(self):
        return {"z_min": self.z_min, "z_max": self.z_max, "r": self.r, "l": self.l,
                "value": self.value}


@dataclass
class Corrfunc:
    """One correlation-function value (python/coffe/representation.py's Corrfunc record)."""

    z: float
    r: float
    mu: float
    value: float

    def to_dict(self):
        return {"z": self.z, "r": self.r, "mu": self.mu, "value": self.value}


@dataclass
class Covariance:
    """One covariance value (python/coffe/representation.py's Covariance record)."""

    z: float
    r1: float
    r2: float
    l1: int
    l2: int
    value: float


@dataclass
class AverageCovariance:
    """One covariance value of the averaged multipoles (representation.py's
    AverageCovariance record)."""

    z_min: float
    z_max: float
    r1: float
    r2: float
    l1: int
    l2: int
    value: float


def divergent_separations() -> np.ndarray:
    """The fixed separations (Mpc) on which the reference splines the divergent
    integral I^4_0 (integrals.c:76-103)."""
    L = _lib.load()
    n = L.coffe_gpu_divergent_separations(None, 0)
    out = np.zeros(n)
    L.coffe_gpu_divergent_separations(_dptr(out), n)
    return out


def _check_parameter(name, value, kind, lo, hi):
    """Range/type check with the reference's semantics (coffe.pyx:86-110)."""
    if not isinstance(value, kind) or isinstance(value, bool) and kind is not bool:
        raise TypeError(f"Expected {kind}, got {type(value)} for {name}")
    if not (lo <= value <= hi):
        raise ValueError(f"Value {value} of {name} outside of interval [{lo}, {hi}]")


class Coffe:
    """Mirror of ``coffe.Coffe`` (coffe.pyx:237-3585) for the hot path: the
    FFTLog integrals, density/RSD multipoles, with lazy initialisation and
    caching like the reference (background -> power spectrum -> integrals ->
    multipoles), computed on the GPU through the C ABI.
    """

    def __init__(self, *, omega_m=0.3, omega_baryon=0.05, omega_gamma=9e-5, h=0.67,
                 sep=None, l=(0, 2, 4), mu=(0.5,), z_mean=(1.0,), z_min=(0.9,),
                 z_max=(1.1,), has_density=True,
                 has_rsd=False, has_lensing=False,
                 integrals_fftlog_sampling=4096, background_bins=10000,
                 integration_1d_prec=1e-5, precision="fp64", deltaz=(0.2,),
                 number_density1=(), number_density2=(), pixelsize=(10.0,), fsky=(1.0,),
                 covariance_fftlog_sampling=8192, device=0):
        self._ctx = Context(device)
        self.omega_m = float(omega_m)
        self.omega_baryon = float(omega_baryon)
        self.omega_gamma = float(omega_gamma)
        self.h = float(h)
        # default separations of coffe_parse_default_parameters (parser.c:836-838)
        self.sep = np.linspace(5, 305, 100, endpoint=False) if sep is None else np.asarray(sep, float)
        self.l = list(l)
        # default mu of coffe_parse_default_parameters (parser.c:980-982)
        self.mu = [float(m) for m in mu]
        self.z_mean = list(z_mean)
        # redshift windows of the averaged multipoles (parser.c defaults 0.9, 1.1)
        self.z_min = [float(z) for z in z_min]
        self.z_max = [float(z) for z in z_max]
        self.has_density = bool(has_density)
        self.has_rsd = bool(has_rsd)
        self.has_lensing = bool(has_lensing)
        self.integrals_fftlog_sampling = int(integrals_fftlog_sampling)
        self.background_bins = int(background_bins)
        self.integration_1d_prec = float(integration_1d_prec)
        self.precision = precision
        # covariance parameters, one value per z_mean (or per averaging window):
        # half-width deltaz, number densities (1/Mpc^3), pixel size (Mpc), sky
        # fraction (parser.c:934-939 defaults for pixelsize and fsky)
        self.deltaz = [float(v) for v in deltaz]
        self.number_density1 = [float(v) for v in number_density1]
        self.number_density2 = [float(v) for v in number_density2]
        self.pixelsize = [float(v) for v in pixelsize]
        self.fsky = [float(v) for v in fsky]
        self.covariance_fftlog_sampling = int(covariance_fftlog_sampling)
        self._k = None
        self._pk = None
        self._bg_ready = False
        self._int_ready = False
        self._bias = {}

    # ------------------------------------------------------------ parameters
    def set_power_spectrum_linear(self, k: Iterable[float], pk: Iterable[float], z: float = 0):
        """k in 1/Mpc, P(k) in Mpc^3 (coffe.pyx:2929-2996); kmin/kmax = k[0], k[-1]."""
        k = np.asarray(k, dtype=float)
        pk = np.asarray(pk, dtype=float)
        if not np.allclose(k, np.sort(k)):
            raise ValueError("The input k array must be sorted")
        if len(k) != len(pk):
            raise ValueError("The input arrays have mismatching lengths")
        self._k, self._pk = k, pk
        self._int_ready = False

    def set_galaxy_bias1(self, z, value):
        self._set_bias(0, z, value)

    def set_galaxy_bias2(self, z, value):
        self._set_bias(1, z, value)

    def _set_bias(self, which, z, value):
        z = np.asarray(z, float)
        if np.any(z < 0) or np.any(z > 15):
            raise ValueError("bias redshifts must be in [0, 15]")
        self._bias[which] = (z, np.asarray(value, float))
        if self._bg_ready:
            self._ctx.set_bias(which, *self._bias[which])

    # ------------------------------------------------------------------ init
    def _background_init(self):
        self._ctx.background_init(self.omega_m, self.omega_baryon, self.omega_gamma, self.h,
                                  self.background_bins)
        for which, (z, v) in self._bias.items():
            self._ctx.set_bias(which, z, v)
        self._bg_ready = True

    def _integrals_init(self):
        if self._k is None:
            raise ValueError("no power spectrum: call set_power_spectrum_linear first")
        self._ctx.integrals_init(self._k, self._pk[None, :], DEFAULT_TERMS,
                                 N=self.integrals_fftlog_sampling, precision=self.precision,
                                 small_r=True)
        self._int_ready = True

    def _ensure(self):
        if not self._bg_ready:
            self._background_init()
        if not self._int_ready:
            self._integrals_init()

    @property
    def _contrib(self) -> int:
        c = ((_lib.DEN if self.has_density else 0) | (_lib.RSD if self.has_rsd else 0) |
             (_lib.LEN if self.has_lensing else 0))
        if c == 0:
            raise ValueError("no contributions selected (has_density / has_rsd / has_lensing)")
        return c

    # --------------------------------------------------------------- outputs
    def integral(self, *, r: float, n: int, l: int) -> float:
        """I_l^n(r) (times r^(n-l) when n > l), coffe.pyx:1657-1713."""
        _check_parameter("r", r, (int, float), 0, 25000)
        _check_parameter("n", n, int, -2, 4)
        _check_parameter("l", l, int, 0, 4)
        self._ensure()
        return float(self._ctx.integral_eval(0, n, l, [float(r)])[0])

    def compute_multipole(self, *, z: float, r: float, l: int) -> float:
        """One multipole at (z_mean, r, l) (coffe.pyx:3232-3300)."""
        _check_parameter("z", z, (int, float), 0, 15)
        _check_parameter("r", r, (int, float), 0, 1500)
        _check_parameter("l", l, int, 0, 10)
        self._ensure()
        out = self._ctx.multipoles([0], [float(z)], [0, 1], [float(r)], [l], self._contrib,
                                   self.precision, self.integration_1d_prec)
        return float(out[0, 0])

    def compute_multipoles_bulk(self) -> List[Multipoles]:
        """All (z_mean, l, sep) points in the reference's order: z outer, l,
        then separation (multipoles.c:76-86)."""
        self._ensure()
        nz, ns = len(self.z_mean), len(self.sep)
        offs = np.arange(nz + 1, dtype=np.int64) * ns
        sep = np.tile(self.sep, nz)
        vals = self._ctx.multipoles(np.zeros(nz, np.int32), self.z_mean, offs, sep, self.l,
                                    self._contrib, self.precision, self.integration_1d_prec)
        res = []
        for iz, zm in enumerate(self.z_mean):
            for il, ll in enumerate(self.l):
                for js, r in enumerate(self.sep):
                    res.append(Multipoles(z=zm, r=float(r), l=ll, value=float(vals[iz * ns + js, il])))
        return res

    def compute_average_multipole(self, *, z_min: float, z_max: float, r: float, l: int) -> float:
        """One redshift-averaged multipole (coffe.pyx's compute_average_multipoles_bulk
        for a single point)."""
        _check_parameter("z_min", z_min, (int, float), 0, 15)
        _check_parameter("z_max", z_max, (int, float), 0, 15)
        _check_parameter("r", r, (int, float), 0, 1500)
        _check_parameter("l", l, int, 0, 10)
        self._ensure()
        out = self._ctx.average_multipoles([0], [float(z_min)], [float(z_max)], [0, 1],
                                           [float(r)], [l], self._contrib, self.precision,
                                           self.integration_1d_prec)
        return float(out[0, 0])

    def compute_average_multipoles_bulk(self) -> List[AverageMultipoles]:
        """All (window, l, sep) points in the reference's order: window outer, l,
        then separation (average_multipoles.c:96-106)."""
        if len(self.z_min) != len(self.z_max):
            raise ValueError("z_min and z_max must have the same length")
        self._ensure()
        nw, ns = len(self.z_min), len(self.sep)
        offs = np.arange(nw + 1, dtype=np.int64) * ns
        sep = np.tile(self.sep, nw)
        vals = self._ctx.average_multipoles(np.zeros(nw, np.int32), self.z_min, self.z_max, offs,
                                            sep, self.l, self._contrib, self.precision,
                                            self.integration_1d_prec)
        res = []
        for iw in range(nw):
            for il, ll in enumerate(self.l):
                for js, r in enumerate(self.sep):
                    res.append(AverageMultipoles(z_min=self.z_min[iw], z_max=self.z_max[iw],
                                                 r=float(r), l=ll,
                                                 value=float(vals[iw * ns + js, il])))
        return res

    def compute_corrfunc(self, *, z: float, r: float, mu: float) -> float:
        """The correlation function at (z_mean, r, mu) (coffe.pyx:3159-3240)."""
        _check_parameter("z", z, (int, float), 0, 15)
        _check_parameter("r", r, (int, float), 0, 1500)
        _check_parameter("mu", mu, (int, float), -1, 1)
        self._ensure()
        out = self._ctx.corrfunc([0], [float(z)], [0, 1], [float(r)], [float(mu)], self._contrib,
                                 self.precision)
        return float(out[0, 0])

    def compute_corrfunc_bulk(self) -> List[Corrfunc]:
        """All (z_mean, mu, sep) points in the reference's order: z outer, mu,
        then separation (corrfunc.c:78-86)."""
        self._ensure()
        nz, ns = len(self.z_mean), len(self.sep)
        offs = np.arange(nz + 1, dtype=np.int64) * ns
        sep = np.tile(self.sep, nz)
        vals = self._ctx.corrfunc(np.zeros(nz, np.int32), self.z_mean, offs, sep, self.mu,
                                  self._contrib, self.precision)
        res = []
        for iz, zm in enumerate(self.z_mean):
            for im, m in enumerate(self.mu):
                for js, r in enumerate(self.sep):
                    res.append(Corrfunc(z=zm, r=float(r), mu=m, value=float(vals[iz * ns + js, im])))
        return res

    def _covariance_contrib(self) -> int:
        c = (_lib.DEN if self.has_density else 0) | (_lib.RSD if self.has_rsd else 0)
        if c == 0:
            raise ValueError("the covariance needs has_density and/or has_rsd")
        return c

    def compute_covariance_bulk(self) -> List["Covariance"]:
        """Covariance of the multipoles for every z_mean, in the reference's
        order: z outer, then l1, r1, l2, r2 (coffe.pyx:3428-3480,
        covariance.c:1046-1059); the FFTLog method with covariance_fftlog_sampling
        points."""
        nz = len(self.z_mean)
        if not all(len(v) == nz for v in (self.deltaz, self.number_density1,
                                          self.number_density2, self.pixelsize, self.fsky)):
            raise ValueError("Mismatching lengths for covariance parameters (`z_mean`, `deltaz`, "
                             "`number_density1`, `number_density2`, `pixelsize`, `fsky`)")
        if self._k is None:
            raise ValueError("set_power_spectrum_linear first")
        if not self._bg_ready:
            self._background_init()
        cov = self._ctx.covariance_multipoles(
            self._k, self._pk, self.covariance_fftlog_sampling, self.z_mean, self.deltaz,
            self.fsky, self.number_density1, self.number_density2, self.pixelsize, self.l,
            self.sep, self._covariance_contrib())
        return [Covariance(z=float(zm), r1=float(r1), r2=float(r2), l1=l1, l2=l2,
                           value=float(cov[iz, i, a, j, b]))
                for iz, zm in enumerate(self.z_mean)
                for i, l1 in enumerate(self.l) for a, r1 in enumerate(self.sep)
                for j, l2 in enumerate(self.l) for b, r2 in enumerate(self.sep)]

    def compute_average_covariance_bulk(self) -> List["AverageCovariance"]:
        """Covariance of the redshift-averaged multipoles for every window
        (z_min, z_max), in the reference's order (coffe.pyx:3482-3537)."""
        nw = len(self.z_min)
        if not all(len(v) == nw for v in (self.z_max, self.number_density1,
                                          self.number_density2, self.pixelsize, self.fsky)):
            raise ValueError("Mismatching lengths for average covariance parameters (`z_min`, "
                             "`z_max`, `number_density1`, `number_density2`, `pixelsize`, `fsky`)")
        if self._k is None:
            raise ValueError("set_power_spectrum_linear first")
        if not self._bg_ready:
            self._background_init()
        cov = self._ctx.average_covariance_multipoles(
            self._k, self._pk, self.covariance_fftlog_sampling, self.z_min, self.z_max,
            self.fsky, self.number_density1, self.number_density2, self.pixelsize, self.l,
            self.sep, self._covariance_contrib())
        return [AverageCovariance(z_min=float(a_), z_max=float(b_), r1=float(r1), r2=float(r2),
                                  l1=l1, l2=l2, value=float(cov[iw, i, a, j, b]))
                for iw, (a_, b_) in enumerate(zip(self.z_min, self.z_max))
                for i, l1 in enumerate(self.l) for a, r1 in enumerate(self.sep)
                for j, l2 in enumerate(self.l) for b, r2 in enumerate(self.sep)]

    def close(self):
        self._ctx.close()
