"""Seeded synthetic inputs for the five benchmark configurations.

No dataset is involved: the linear power spectrum is the BBKS (Bardeen et al.
1986) transfer-function form P(k) = A k^n_s T(k/Gamma)^2 normalised to sigma8
with a top-hat window of radius 8 Mpc/h, integrated on the same grid.  All
functions return k in 1/Mpc and P(k) in Mpc^3 (the reference's internal units:
k[1/Mpc] = h k[h/Mpc], P[Mpc^3] = P[(Mpc/h)^3] / h^3); separations in Mpc.
"""
from __future__ import annotations

from dataclasses import dataclass
from typing import List

import numpy as np

CFG3_SEED = 20261203


def bbks_pk(kh, n_s=0.965, gamma=0.21, sigma8=0.81, bao=False):
    """BBKS P(k) on k in h/Mpc (returned in (Mpc/h)^3), sigma8-normalised.

    With ``bao`` the spectrum is multiplied by 1 + 0.05 sin(105 k) exp(-(k/0.2)^2)."""
    kh = np.asarray(kh, dtype=np.float64)
    q = kh / gamma
    T = np.log1p(2.34 * q) / (2.34 * q) * (
        1 + 3.89 * q + (16.1 * q) ** 2 + (5.46 * q) ** 3 + (6.71 * q) ** 4) ** -0.25
    P = kh ** n_s * T ** 2
    x = kh * 8.0
    W = 3 * (np.sin(x) - x * np.cos(x)) / x ** 3
    lnk = np.log(kh)
    s2 = np.trapezoid(kh ** 3 * P * W ** 2, lnk) / (2 * np.pi ** 2)
    P = P * sigma8 ** 2 / s2
    if bao:
        P = P * (1 + 0.05 * np.sin(105 * kh) * np.exp(-(kh / 0.2) ** 2))
    return P


def k_grid_h(n=4096, kmin=1e-5, kmax=1e2):
    return np.logspace(np.log10(kmin), np.log10(kmax), n)


def to_internal(kh, pk_h, h):
    """(h/Mpc, (Mpc/h)^3) -> (1/Mpc, Mpc^3)."""
    return np.asarray(kh) * h, np.asarray(pk_h) / h ** 3


@dataclass
class Cosmo:
    omega_m: float = 0.31
    omega_baryon: float = 0.05
    omega_gamma: float = 9e-5
    h: float = 0.67


def cfg1():
    """Plain den+RSD multipoles l = 0,2,4 at z = 1, 100 separations 10-200 Mpc/h."""
    c = Cosmo()
    kh = k_grid_h(4096)
    k, pk = to_internal(kh, bbks_pk(kh), c.h)
    sep = np.linspace(10, 200, 100) / c.h
    return dict(cosmo=c, k=k, pk=pk, z_mean=1.0, sep=sep, ls=(0, 2, 4))


def cfg2():
    """All I_l^n for l = 0..4, n = -1..4 of the BAO-modulated spectrum on 2^14 points."""
    c = Cosmo()
    kh = k_grid_h(16384)
    k, pk = to_internal(kh, bbks_pk(kh, bao=True), c.h)
    terms = [(n, l) for l in range(5) for n in range(-1, 5)]
    r_out = np.logspace(0, 4, 16384) / c.h
    return dict(cosmo=c, k=k, pk=pk, terms=terms, N=16384, r_out=r_out)


LENS_TERMS = ((0, 0), (0, 2), (0, 4), (1, 1), (1, 3), (2, 0))


def cfg4():
    """den+RSD+lensing multipoles l = 0,2,4,6 at z = 1.5 (delta z 0.2), 200
    separations 20-300 Mpc/h, lensing by Gauss-Legendre 128 mu x 256 chi."""
    c = Cosmo()
    kh = k_grid_h(4096)
    k, pk = to_internal(kh, bbks_pk(kh), c.h)
    sep = np.linspace(20, 300, 200) / c.h
    return dict(cosmo=c, k=k, pk=pk, z_mean=1.5, deltaz=0.2, sep=sep, ls=(0, 2, 4, 6),
                terms=LENS_TERMS, rule=(128, 256))


def cfg5(chi_of_z=None):
    """Flat-sky Gaussian covariance of the l = 0,2,4 multipoles: 5 redshift bins
    (z = 0.5..2.0, delta z 0.1), each of volume 1 (Gpc/h)^3, n = 1e-3 (h/Mpc)^3,
    128 x 128 separations 20-300 Mpc/h, 2D FFTLog on 2^11 x 2^11 points.
    chi_of_z (Mpc) fixes fsky from the volume; without it fsky is None."""
    c = Cosmo()
    kh = k_grid_h(4096)
    k, pk = to_internal(kh, bbks_pk(kh), c.h)
    z = np.linspace(0.5, 2.0, 5)
    dz = np.full(5, 0.1)
    sep = np.linspace(20, 300, 128) / c.h
    fsky = None
    if chi_of_z is not None:
        vol = 1e9 / c.h ** 3  # (Gpc/h)^3 in Mpc^3
        shell = 4 * np.pi * (chi_of_z(z + dz) ** 3 - chi_of_z(z - dz) ** 3) / 3
        fsky = vol / shell
    return dict(cosmo=c, k=k, pk=pk, z_mean=z, deltaz=dz, fsky=fsky,
                density=np.full(5, 1e-3 * c.h ** 3), pixelsize=np.full(5, sep[1] - sep[0]),
                sep=sep, ls=(0, 2, 4), N=2048)


@dataclass
class Batch:
    k: np.ndarray
    pk: np.ndarray  # (S, nk)
    req_spectrum: np.ndarray
    req_z_mean: np.ndarray
    req_offset: np.ndarray
    sep: np.ndarray
    ls: tuple
    cosmo: Cosmo

    @property
    def n_evals(self) -> int:
        return len(self.sep) * len(self.ls)


def cfg3(n_spectra=512, n_z=6, seed=CFG3_SEED, nk=4096, rmin=5.0, rmax=250.0, count=(20, 400)):
    """512 seeded spectra x 6 z_mean x l = 0,2,4 with uneven separation lists."""
    c = Cosmo()
    rng = np.random.default_rng(seed)
    kh = k_grid_h(nk)
    s8 = rng.uniform(0.7, 0.9, n_spectra)
    ns = rng.uniform(0.93, 1.0, n_spectra)
    gm = rng.uniform(0.15, 0.3, n_spectra)
    pk = np.stack([bbks_pk(kh, ns[i], gm[i], s8[i]) for i in range(n_spectra)])
    k, pk = to_internal(kh, pk, c.h)
    zs = np.linspace(0.5, 2.0, n_z)
    req_s, req_z, offs, seps = [], [], [0], []
    for s in range(n_spectra):
        for z in zs:
            m = int(rng.integers(count[0], count[1] + 1))
            r = np.sort(rng.uniform(rmin, rmax, m)) / c.h
            req_s.append(s)
            req_z.append(z)
            seps.append(r)
            offs.append(offs[-1] + m)
    return Batch(k=k, pk=pk, req_spectrum=np.asarray(req_s, np.int32),
                 req_z_mean=np.asarray(req_z), req_offset=np.asarray(offs, np.int64),
                 sep=np.concatenate(seps), ls=(0, 2, 4), cosmo=c)


def subset(b: Batch, n_spectra: int) -> Batch:
    """The first n_spectra spectra of a batch with their requests."""
    keep = b.req_spectrum < n_spectra
    nreq = int(keep.sum())
    end = int(b.req_offset[nreq])
    return Batch(k=b.k, pk=b.pk[:n_spectra], req_spectrum=b.req_spectrum[:nreq],
                 req_z_mean=b.req_z_mean[:nreq], req_offset=b.req_offset[: nreq + 1],
                 sep=b.sep[:end], ls=b.ls, cosmo=b.cosmo)
