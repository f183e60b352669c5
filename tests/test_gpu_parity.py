"""GPU parity: the CUDA path through the C ABI against the CPU oracle on the same
seeded inputs, and against the reference's golden vectors.

Tolerances (stated per test):
  * FP64 path: 1e-10 relative (the benchmark spec), with a floor of 1e-3 of the largest
    |value| of the same multipole / 1e-8 of the local table envelope so that
    zero crossings do not turn rounding into infinite relative error;
  * mixed path: 1e-4 relative with the same floors; multipoles that vanish
    in the flat-sky limit (odd l, l >= 6, density-only l >= 2) to a few FP32
    ulps of the monopole (see _mixed_err);
  * golden vectors: the reference's own tolerances (integrals rtol 1e-4,
    multipoles rtol 5e-4, np.isclose semantics).
"""
import numpy as np
import pytest

from conftest import COFFE_H0, H

pytestmark = pytest.mark.gpu

TERMS8 = [(0, 0), (0, 2), (0, 4), (1, 1), (1, 3), (2, 0), (2, 2), (3, 1)]


def rel_floor(got, ref, floor):
    return np.max(np.abs(got - ref) / np.maximum(np.abs(ref), floor))


def local_envelope(y, half=64):
    a = np.nan_to_num(np.abs(y), nan=0.0)
    out = np.empty_like(a)
    for i in range(len(a)):
        out[i] = a[max(0, i - half): i + half + 1].max()
    return out


def table_err(gy, oy, mask, floor=1e-8):
    env = local_envelope(oy)
    return np.max((np.abs(gy - oy) / np.maximum(np.abs(oy), floor * env))[mask])


@pytest.fixture(scope="module")
def w():
    from coffe_gb300 import workloads

    return workloads


@pytest.fixture(scope="module")
def cfg1(w):
    return w.cfg1()


@pytest.fixture(scope="module")
def bg031(oracle):
    return oracle.background_nodes(0.31, 0.05, 9e-5, H, 10000)


def oracle_model(oracle, bg, k, pk, N, omega_m=0.31, small_r=False):
    m = oracle.Model(bg, H, omega_m)
    for n, l in [(0, 0), (0, 2), (0, 4)]:
        x, y = oracle.integral_table(k, pk, n, l, N, with_small_r=small_r)
        m.set_integral(n, l, x, y)
    return m


# ----------------------------------------------------------------- background
def test_background_init_matches_oracle(gpu_ctx, bg031):
    gpu_ctx.background_init(0.31, 0.05, 9e-5, H, 10000)
    g = gpu_ctx.background()
    pairs = {"z": "z", "chi": "chi", "D1": "D1", "f": "f", "a": "a", "Hz": "Hz",
             "conformal_Hz": "confH", "conformal_Hz_prime": "confHp"}
    for gk, ok in pairs.items():
        err = rel_floor(g[gk], bg031[ok], 1e-300)
        assert err < 1e-12, (gk, err)


def test_background_set_roundtrip(gpu_ctx, bg031):
    gpu_ctx.background_set(bg031["z"], bg031["chi"], bg031["D1"], bg031["f"], bg031["a"],
                           bg031["confH"], 0.31, H)
    g = gpu_ctx.background(with_H=False)
    assert np.array_equal(g["chi"], bg031["chi"]) and np.array_equal(g["f"], bg031["f"])


# ------------------------------------------------------------------ integrals
def test_integral_tables_fp64_match_oracle(gpu_ctx, oracle, cfg1):
    k, pk = cfg1["k"], cfg1["pk"]
    N = 4096
    gpu_ctx.integrals_init(k, pk[None, :], TERMS8, N=N, precision="fp64", small_r=True)
    for n, l in TERMS8:
        gx, gy = gpu_ctx.integral_table(0, n, l)
        ox, oy = oracle.integral_table(k, pk, n, l, N, with_small_r=True)
        assert rel_floor(gx, ox, 1e-300) < 1e-14
        fft = np.zeros(len(ox), bool)
        fft[43:] = True
        mask = fft & (ox >= 1.0) & (ox <= 1e4)
        e_fft = table_err(gy, oy, mask)
        e_small = rel_floor(gy[:43], oy[:43], 1e-8 * np.abs(oy[:43]).max())
        assert e_fft < 1e-10, ((n, l), e_fft)
        assert e_small < 1e-9, ((n, l), e_small)


@pytest.mark.parametrize("N", [4096, 2048, 8192])
@pytest.mark.parametrize("tables_df", [False, True])
def test_integral_tables_mixed_close_to_oracle(gpu_ctx, oracle, cfg1, tables_df, N):
    """Mixed-precision tables of I_0^0, I_2^0, I_4^0 over the multipoles' range.
    FP32 inverse transforms (default): 1e-5 relative with a floor of 1e-3 of the
    range's largest |I| (their rounding is ~1e-7 of the outputs' scale, so the
    error stays near that fraction of the scale, also at zero crossings).
    Double-float inverse transforms: 1e-5 relative with a floor of 1e-6 of the
    local envelope (the float spline-curvature correction of the resampled
    P(k) adds ~1e-6 near zero crossings).  N = 2048 and 8192 run the forward
    transform's two packed N/4-point halves with a radix-2 first stage (odd
    log2(N/4)), N = 4096 without."""
    k, pk = cfg1["k"], cfg1["pk"]
    gpu_ctx.integrals_init(k, pk[None, :], [(0, 0), (0, 2), (0, 4)], N=N, precision="mixed",
                           small_r=False, tables_df=tables_df)
    for n, l in [(0, 0), (0, 2), (0, 4)]:
        gx, gy = gpu_ctx.integral_table(0, n, l)
        ox, oy = oracle.integral_table(k, pk, n, l, N, with_small_r=False)
        mask = (ox >= 5 / H) & (ox <= 300 / H)
        mask[:43] = False
        assert np.isnan(gy[:43]).all()  # not requested
        if tables_df:
            e = table_err(gy, oy, mask, floor=1e-6)
        else:
            e = rel_floor(gy[mask], oy[mask], 1e-3 * np.abs(oy[mask]).max())
        print((n, l), "tables_df" if tables_df else "fp32 inverse", e)
        assert e < 1e-5, ((n, l), e)


@pytest.mark.parametrize("fused", [1, 0])
def test_integral_tables_mixed_irregular_grid(oracle, cfg1, fused):
    """A k grid that is not geometric (log-spacing varying by +-15% along the
    grid): the natural spline's band is applied as full rows instead of the
    factorised form, in the fused table kernel (fused = 1) and in
    cspline_band_kernel (fused = 0).  Tables of I_0^0, I_2^0, I_4^0 against the
    oracle on the same grid, with the tolerance of the geometric case."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from coffe_gb300.api import Context

    k0, pk0 = cfg1["k"], cfg1["pk"]
    u = np.linspace(0.0, 1.0, len(k0))
    lk = np.log(k0[0]) + np.log(k0[-1] / k0[0]) * (u + 0.15 * np.sin(10 * np.pi * u) / (10 * np.pi))
    k = np.exp(lk)
    k[0], k[-1] = k0[0], k0[-1]
    pk = np.exp(np.interp(lk, np.log(k0), np.log(pk0)))
    dl = np.diff(np.log(k))
    assert np.all(dl > 0) and dl.max() / dl.min() > 1.3
    N = 4096
    ctx = Context(0)
    try:
        ctx.set_tuning(fft_fused=fused)
        ctx.integrals_init(k, pk[None, :], [(0, 0), (0, 2), (0, 4)], N=N, precision="mixed",
                           small_r=False)
        assert ctx.tuning()["fft_fused"] == fused
        for n, l in [(0, 0), (0, 2), (0, 4)]:
            gx, gy = ctx.integral_table(0, n, l)
            ox, oy = oracle.integral_table(k, pk, n, l, N, with_small_r=False)
            mask = (ox >= 5 / H) & (ox <= 300 / H)
            mask[:43] = False
            e = rel_floor(gy[mask], oy[mask], 1e-3 * np.abs(oy[mask]).max())
            print("irregular grid, fused", fused, (n, l), e)
            assert e < 1e-5, ((n, l), e)
    finally:
        ctx.close()


def test_all_bessel_integrals_2e14_fp64(gpu_ctx, oracle, w):
    """l = 0..4, n = -1..4 on 2^14 points, including the pairs whose Gamma-ratio
    reflection overflows at high frequency (kept as the reference computes them)."""
    c = w.cfg2()
    k, pk, N = c["k"], c["pk"], c["N"]
    gpu_ctx.integrals_init(k, pk[None, :], c["terms"], N=N, precision="fp64", small_r=False)
    worst = 0.0
    for n, l in c["terms"]:
        gx, gy = gpu_ctx.integral_table(0, n, l)
        ox, oy = oracle.integral_table(k, pk, n, l, N, with_small_r=False)
        mask = (ox >= 1.0) & (ox <= 1e4)
        mask[:43] = False
        # The Gamma-ratio coefficients at t ~ 3000 carry ~1e-12 relative rounding
        # in the reference itself (checked against 40-digit log-Gamma), and the
        # inverse FFT sums 8192 such modes; values far below the table's scale
        # are therefore compared with an absolute floor of 1e-10 of the largest
        # |I| over r in [1, 1e4] Mpc, everything else to 1e-10 relative.
        scale = np.abs(oy[mask]).max()
        e = np.max(np.abs(gy[mask] - oy[mask]) / np.maximum(np.abs(oy[mask]), scale))
        e_rel = table_err(gy, oy, mask, floor=1e-6)
        worst = max(worst, e)
        print((n, l), "abs/scale", e, "rel (floor 1e-6 local)", e_rel)
        assert e < 1e-10, ((n, l), e)
    print("worst FP64 table error (2^14, 30 terms):", worst)


def _cfg2_errors(got, ref):
    """Errors of one config-2 table on r in [1, 1e4] Mpc/h: (max abs error /
    the table's scale, the relative error with a floor of 1e-3 of the scale --
    the convention of the multipole metric --, and the relative error with a
    floor of only 1e-6 of the local envelope).  The last is reported, not
    asserted: the n = -1 tables fall by many decades over the range, and where
    they are far below their scale even the FP64 FFTLog's rounding (1e-15 of
    the scale) is a large fraction of the value."""
    scale = np.abs(ref).max()
    d = np.abs(got - ref)
    a = np.abs(ref)
    env = np.array([a[max(0, i - 64): i + 65].max() for i in range(len(a))])
    return (d.max() / scale, np.max(d / np.maximum(a, 1e-3 * scale)),
            np.max(d / np.maximum(a, 1e-6 * env)))


# config-2 mixed tolerances on r in [1, 1e4] Mpc/h: (abs error / the table's
# scale, relative error with a floor of 1e-3 of the scale).  FP32 inverse
# transforms (default): measured up to 6.8e-6 and 1.8e-5 (the n = -1 tables
# cross zero inside the range; a float transform leaves them ~2e-7 of their
# scale); double-float inverse transforms: 5.8e-8 and 9.4e-7.
CFG2_MIXED_TOL = {False: (1e-5, 1e-4), True: (2e-7, 1e-5)}


@pytest.mark.parametrize("tables_df", [False, True])
def test_all_bessel_integrals_2e14_mixed(gpu_ctx, oracle, w, tables_df):
    """Config 2 in mixed precision (double-float forward transform on the FP32
    pipes, FP32 or double-float inverse transforms, FP64 Gamma-ratio
    coefficients, tables stored as float): every one of the 30 (n, l) tables at
    2^14 points against the FP64 oracle on r in [1, 1e4] Mpc/h
    (CFG2_MIXED_TOL)."""
    c = w.cfg2()
    k, pk, N = c["k"], c["pk"], c["N"]
    gpu_ctx.integrals_init(k, pk[None, :], c["terms"], N=N, precision="mixed", small_r=False,
                           tables_df=tables_df)
    tol = CFG2_MIXED_TOL[tables_df]
    worst = np.zeros(3)
    for n, l in c["terms"]:
        gx, gy = gpu_ctx.integral_table(0, n, l)
        ox, oy = oracle.integral_table(k, pk, n, l, N, with_small_r=False)
        mask = (ox >= 1.0 / H) & (ox <= 1e4 / H)
        mask[:43] = False
        e = _cfg2_errors(gy[mask], oy[mask])
        worst = np.maximum(worst, e)
        print((n, l), "abs/scale %.3g  rel (floor 1e-3 scale) %.3g  rel (floor 1e-6 local) %.3g"
              % e)
        assert e[0] < tol[0], ((n, l), e)
        assert e[1] < tol[1], ((n, l), e)
    print("worst mixed table errors (2^14, 30 terms, tables_df=%s): abs/scale %.3g, rel %.3g, "
          "local %.3g" % ((tables_df,) + tuple(worst)))


@pytest.mark.parametrize("precision", ["fp64", "mixed", "mixed-df"])
def test_cfg2_resampled_on_log_r(gpu_ctx, oracle, w, precision):
    """Config 2's output grid: every table resampled by its Akima spline
    (coffe_gpu_integral_eval, the lookup of coffe_interp_spline) at 2^14
    log-spaced r in [1, 1e4] Mpc/h, against the same spline of the oracle's table.
    FP64: 1e-10 of the table's scale and 1e-10 relative with a floor of 1e-3 of
    the scale; mixed: CFG2_MIXED_TOL."""
    c = w.cfg2()
    k, pk, N, r = c["k"], c["pk"], c["N"], c["r_out"]
    df = precision == "mixed-df"
    gpu_ctx.integrals_init(k, pk[None, :], c["terms"], N=N, precision=precision[:5],
                           small_r=False, tables_df=df)
    tol_scale, tol_rel = (1e-10, 1e-10) if precision == "fp64" else CFG2_MIXED_TOL[df]
    for n, l in c["terms"]:
        got = gpu_ctx.integral_eval(0, n, l, r)
        ox, oy = oracle.integral_table(k, pk, n, l, N, with_small_r=False)
        ref = oracle.spline_eval("akima", ox[43:], oy[43:], r)
        e = _cfg2_errors(got, ref)
        print(precision, (n, l), "abs/scale %.3g  rel (floor 1e-3 scale) %.3g  local %.3g" % e)
        assert e[0] < tol_scale, ((n, l), e)
        assert e[1] < tol_rel, ((n, l), e)


def test_integrals_golden_through_gpu(gpu_ctx, golden, class_pk):
    k, pk = class_pk
    gpu_ctx.integrals_init(k, pk[None, :], TERMS8, N=16384, precision="fp64", small_r=True)
    for i, (n, l) in enumerate(TERMS8):
        d = golden[f"integral{i}"]
        r = d[:, 0] / (COFFE_H0 * H)
        val = gpu_ctx.integral_eval(0, n, l, r)
        if n > l:
            val = val * (COFFE_H0 * H) ** (n - l)
        assert np.isclose(d[:, 1], val, rtol=1e-4).all(), (n, l)


# ----------------------------------------------------------------- multipoles
def _run_batch(ctx, b, precision):
    return ctx.multipoles(b.req_spectrum, b.req_z_mean, b.req_offset, b.sep, b.ls,
                          precision=precision)


def _oracle_batch(oracle, bg, b, N):
    out = np.zeros((len(b.sep), len(b.ls)))
    for s in range(b.pk.shape[0]):
        m = oracle_model(oracle, bg, b.k, b.pk[s], N)
        for q in np.where(b.req_spectrum == s)[0]:
            lo, hi = b.req_offset[q], b.req_offset[q + 1]
            for j, l in enumerate(b.ls):
                z = np.full(hi - lo, b.req_z_mean[q])
                out[lo:hi, j] = m.multipoles_batch(3, z, b.sep[lo:hi], np.full(hi - lo, l))
    return out


def _per_l_floor(ref, b, frac):
    """floor = frac * max |ref| over the request's separations, per l"""
    fl = np.zeros_like(ref)
    for q in range(len(b.req_spectrum)):
        lo, hi = b.req_offset[q], b.req_offset[q + 1]
        if hi > lo:
            fl[lo:hi] = frac * np.abs(ref[lo:hi]).max(axis=0)
    return np.maximum(fl, 1e-300)


@pytest.fixture(scope="module")
def small_batch(w):
    return w.subset(w.cfg3(n_spectra=6), 6)


@pytest.fixture(scope="module")
def small_batch_ref(oracle, bg031, small_batch):
    return _oracle_batch(oracle, bg031, small_batch, 4096)


def test_multipoles_cfg1_fp64(gpu_ctx, oracle, bg031, cfg1):
    k, pk = cfg1["k"], cfg1["pk"]
    gpu_ctx.background_init(0.31, 0.05, 9e-5, H, 10000)
    gpu_ctx.integrals_init(k, pk[None, :], [(0, 0), (0, 2), (0, 4)], N=4096, precision="fp64",
                           small_r=False)
    sep = cfg1["sep"]
    got = gpu_ctx.multipoles([0], [1.0], [0, len(sep)], sep, (0, 2, 4), precision="fp64")
    m = oracle_model(oracle, bg031, k, pk, 4096)
    for j, l in enumerate((0, 2, 4)):
        ref = m.multipoles_batch(3, np.ones(len(sep)), sep, np.full(len(sep), l))
        e = rel_floor(got[:, j], ref, 1e-3 * np.abs(ref).max())
        assert e < 1e-10, (l, e)


def test_multipoles_batch_fp64(gpu_ctx, small_batch, small_batch_ref):
    b = small_batch
    gpu_ctx.background_init(0.31, 0.05, 9e-5, H, 10000)
    gpu_ctx.integrals_init(b.k, b.pk, [(0, 0), (0, 2), (0, 4)], N=4096, precision="fp64",
                           small_r=False)
    got = _run_batch(gpu_ctx, b, "fp64")
    e = np.max(np.abs(got - small_batch_ref) /
               np.maximum(np.abs(small_batch_ref), _per_l_floor(small_batch_ref, b, 1e-3)))
    print("fp64 max rel error:", e)
    assert e < 1e-10, e


@pytest.mark.parametrize("poly", [1, 0])
def test_multipoles_batch_mixed(gpu_ctx, small_batch, small_batch_ref, poly):
    b = small_batch
    gpu_ctx.set_tuning(lane_poly=poly)
    gpu_ctx.background_init(0.31, 0.05, 9e-5, H, 10000)
    gpu_ctx.integrals_init(b.k, b.pk, [(0, 0), (0, 2), (0, 4)], N=4096, precision="mixed",
                           small_r=False)
    got = _run_batch(gpu_ctx, b, "mixed")
    gpu_ctx.set_tuning(lane_poly=1)
    e = np.max(np.abs(got - small_batch_ref) /
               np.maximum(np.abs(small_batch_ref), _per_l_floor(small_batch_ref, b, 1e-3)))
    print("mixed max rel error (polynomial integrand %d):" % poly, e)
    assert e < 1e-4, e


@pytest.mark.parametrize("poly", [1, 0])
def test_multipoles_batch_fp64_fastalg(gpu_ctx, small_batch, small_batch_ref, poly):
    """COFFE_GPU_FP64_FASTALG (the mixed path's algorithm in FP64, the
    precision-only baseline of the mixed path) against the oracle: its
    approximations are the degree-5 background polynomial along each request's
    line of sight, ~(X/L)^6 ~ 1e-8 relative, and (polynomial integrand) the
    truncated 1/D series, < 1e-12; asserted at 1e-6 with the per-request floor
    of the other batch tests."""
    b = small_batch
    gpu_ctx.set_tuning(lane_poly=poly)
    gpu_ctx.background_init(0.31, 0.05, 9e-5, H, 10000)
    gpu_ctx.integrals_init(b.k, b.pk, [(0, 0), (0, 2), (0, 4)], N=4096, precision="fp64",
                           small_r=False)
    got = _run_batch(gpu_ctx, b, "fp64-fastalg")
    gpu_ctx.set_tuning(lane_poly=1)
    e = np.max(np.abs(got - small_batch_ref) /
               np.maximum(np.abs(small_batch_ref), _per_l_floor(small_batch_ref, b, 1e-3)))
    print("fp64-fastalg max rel error (polynomial integrand %d):" % poly, e)
    assert e < 1e-6, e


FP32_RES = 4 * 2.0 ** -23  # a few FP32 ulps


def _rel_fp64(got, ref, ls):
    """FP64 error: 1e-10 relative with a floor of 1e-3 of the largest |value|
    of the multipole; for odd l (rounding noise when the tracers are equal)
    and l >= 6, of the largest |value| of the whole output."""
    floor = 1e-3 * np.abs(ref).max(axis=0, keepdims=True)
    small = np.array([(l % 2 == 1) or l >= 6 for l in ls])[None, :]
    floor = np.where(small, 1e-3 * np.abs(ref).max(), floor)
    return np.max(np.abs(got - ref) / np.maximum(np.abs(ref), floor))


def _mixed_err(got, ref, ls, mono, contrib=3):
    """Mixed-path error, as a fraction of its bound (pass: < 1).
    Multipoles of the size of the monopole: 1e-4 relative with a floor of 1e-3
    of the multipole's largest |value|.  Multipoles that vanish in the
    flat-sky limit -- odd l (zero for equal tracers), l >= 6, and every l >= 2
    of the density term alone (a wide-angle effect of order (r / chi)^2, ~1e-6
    of the monopole at 10 Mpc/h) -- are known only to the FP32 resolution of
    the integrand: |error| <= 4 * 2^-23 of the monopole's largest |value|."""
    small = np.array([(l % 2 == 1) or l >= 6 or (contrib == 1 and l >= 2) for l in ls])
    floor = 1e-3 * np.abs(ref).max(axis=0, keepdims=True)
    rel = np.abs(got - ref) / np.maximum(np.abs(ref), floor) / 1e-4
    absm = np.abs(got - ref) / (FP32_RES * np.abs(mono).max())
    return max(rel[:, ~small].max(initial=0.0), absm[:, small].max(initial=0.0))


@pytest.mark.parametrize("contrib", [1, 2, 3])
@pytest.mark.parametrize("ls", [(0,), (2, 4), (0, 2, 4, 6), (0, 1, 2, 3)])
def test_multipoles_mixed_variants(gpu_ctx, oracle, bg031, cfg1, contrib, ls):
    """Mixed path against the oracle for each contribution mask and several
    multipole lists: even lists of up to four run the unit-bias kernel, the
    odd list the general one."""
    k, pk = cfg1["k"], cfg1["pk"]
    gpu_ctx.background_init(0.31, 0.05, 9e-5, H, 10000)
    gpu_ctx.integrals_init(k, pk[None, :], [(0, 0), (0, 2), (0, 4)], N=4096, precision="mixed",
                           small_r=False)
    sep = cfg1["sep"][::7]
    z = 0.8
    got = gpu_ctx.multipoles([0], [z], [0, len(sep)], sep, ls, contrib=contrib, precision="mixed")
    m = oracle_model(oracle, bg031, k, pk, 4096)
    ref = np.stack([m.multipoles_batch(contrib, np.full(len(sep), z), sep, np.full(len(sep), l))
                    for l in ls], axis=1)
    mono = m.multipoles_batch(contrib, np.full(len(sep), z), sep, np.zeros(len(sep)))
    e = _mixed_err(got, ref, ls, mono, contrib)
    print(contrib, ls, "mixed error / bound", e)
    assert e < 1, e


@pytest.mark.parametrize("equal", [False, True])
def test_multipoles_with_galaxy_bias(oracle, bg031, cfg1, equal):
    """z-dependent galaxy biases of both tracers (different ones give odd
    multipoles), FP64 at 1e-10 and mixed at 1e-4 against the oracle."""
    k, pk = cfg1["k"], cfg1["pk"]
    zb = np.linspace(0.0, 3.0, 31)
    b1 = 1.2 + 0.3 * zb
    b2 = b1 if equal else 1.6 + 0.1 * zb ** 2
    m = oracle_model(oracle, bg031, k, pk, 4096)
    m.set_bias(0, zb, b1)
    m.set_bias(1, zb, b2)
    sep = cfg1["sep"][::9]
    ls = (0, 1, 2, 3, 4)
    z = 1.1
    ref = np.stack([m.multipoles_batch(3, np.full(len(sep), z), sep, np.full(len(sep), l))
                    for l in ls], axis=1)
    from coffe_gb300.api import Context

    ctx = Context(0)  # biases stay set for the context's lifetime
    try:
        ctx.background_init(0.31, 0.05, 9e-5, H, 10000)
        ctx.set_bias(0, zb, b1)
        ctx.set_bias(1, zb, b2)
        for prec in ("fp64", "mixed"):
            ctx.integrals_init(k, pk[None, :], [(0, 0), (0, 2), (0, 4)], N=4096,
                               precision=prec, small_r=False)
            got = ctx.multipoles([0], [z], [0, len(sep)], sep, ls, precision=prec)
            if prec == "fp64":
                e = _rel_fp64(got, ref, ls)
                print("equal" if equal else "different", "fp64 max rel error", e)
                assert e < 1e-10, e
            else:
                e = _mixed_err(got, ref, ls, ref[:, 0])
                print("equal" if equal else "different", "mixed error / bound", e)
                assert e < 1, e
    finally:
        ctx.close()


def test_multipoles_golden_through_gpu(gpu_ctx, golden, class_pk, ref_bg):
    k, pk = class_pk
    gpu_ctx.background_init(0.3, 0.05, 9e-5, H, 10000)
    gpu_ctx.integrals_init(k, pk[None, :], [(0, 0), (0, 2), (0, 4)], N=16384, precision="fp64",
                           small_r=True)
    for name, mask in [("den", 1), ("rsd", 2), ("std", 3)]:
        d0 = golden[f"{name}_multipoles0"]
        sep = d0[:, 0] / H
        got = gpu_ctx.multipoles([0], [1.0], [0, len(sep)], sep, (0, 2, 4), contrib=mask)
        for j, l in enumerate((0, 2, 4)):
            d = golden[f"{name}_multipoles{l}"]
            assert np.allclose(got[:, j], d[:, 1], rtol=5e-4), (name, l)


def test_multipoles_sub_mpc_uses_small_r_table(gpu_ctx, oracle, bg031, cfg1):
    k, pk = cfg1["k"], cfg1["pk"]
    gpu_ctx.background_init(0.31, 0.05, 9e-5, H, 10000)
    gpu_ctx.integrals_init(k, pk[None, :], [(0, 0), (0, 2), (0, 4)], N=4096, precision="fp64",
                           small_r=True)
    sep = np.array([0.05, 0.3, 0.95, 1.004, 2.0])
    got = gpu_ctx.multipoles([0], [1.2], [0, len(sep)], sep, (0, 2, 4))
    m = oracle_model(oracle, bg031, k, pk, 4096, small_r=True)
    for j, l in enumerate((0, 2, 4)):
        ref = m.multipoles_batch(3, np.full(len(sep), 1.2), sep, np.full(len(sep), l))
        assert rel_floor(got[:, j], ref, 1e-3 * np.abs(ref).max()) < 1e-10, l


def test_ragged_and_empty_requests(gpu_ctx, oracle, bg031, cfg1):
    k, pk = cfg1["k"], cfg1["pk"]
    gpu_ctx.background_init(0.31, 0.05, 9e-5, H, 10000)
    gpu_ctx.integrals_init(k, np.stack([pk, 1.3 * pk]), [(0, 0), (0, 2), (0, 4)], N=4096,
                           precision="fp64", small_r=False)
    # request 0 empty, request 1 one separation, request 2 three, request 3 empty
    offs = [0, 0, 1, 4, 4]
    sep = np.array([50.0, 10.0, 60.0, 150.0])
    got = gpu_ctx.multipoles([0, 1, 0, 1], [1.0, 0.7, 1.5, 2.0], offs, sep, (2, 0))
    m0 = oracle_model(oracle, bg031, k, pk, 4096)
    m1 = oracle_model(oracle, bg031, k, 1.3 * pk, 4096)
    ref = np.array([[m1.multipole(3, 0.7, 50.0, 2), m1.multipole(3, 0.7, 50.0, 0)]] +
                   [[m0.multipole(3, 1.5, r, 2), m0.multipole(3, 1.5, r, 0)] for r in sep[1:]])
    assert rel_floor(got, ref, 1e-300) < 1e-10


# ----------------------------------------------------------------- API mirror
def test_coffe_mirror_against_golden(golden, class_pk):
    from coffe_gb300.api import Coffe

    k, pk = class_pk
    c = Coffe(omega_m=0.3, sep=golden["std_multipoles0"][:, 0] / H, l=[0, 2, 4], z_mean=[1.0],
              has_density=True, has_rsd=True, integrals_fftlog_sampling=16384)
    c.set_power_spectrum_linear(k, pk)
    res = c.compute_multipoles_bulk()
    assert [(r.z, r.l) for r in res[:6]] == [(1.0, 0)] * 5 + [(1.0, 2)]
    for l in (0, 2, 4):
        vals = np.array([r.value for r in res if r.l == l])
        assert np.allclose(vals, golden[f"std_multipoles{l}"][:, 1], rtol=5e-4)
    d = golden["integral1"]
    r = float(d[10, 0] / (COFFE_H0 * H))
    assert np.isclose(c.integral(r=r, n=0, l=2), d[10, 1], rtol=1e-4)
    v = c.compute_multipole(z=1.0, r=float(golden["std_multipoles2"][2, 0] / H), l=2)
    assert np.isclose(v, golden["std_multipoles2"][2, 1], rtol=5e-4)
    with pytest.raises(ValueError):
        c.integral(r=-1.0, n=0, l=0)
    with pytest.raises(ValueError):
        c.integral(r=1.0, n=0, l=7)
    c.close()


# --------------------------------------------------------------- error paths
def test_error_statuses(w, cfg1):
    from coffe_gb300._lib import CoffeGpuError
    from coffe_gb300.api import Context

    k, pk = cfg1["k"], cfg1["pk"]
    with Context(0) as ctx:
        with pytest.raises(CoffeGpuError) as e:  # multipoles before anything
            ctx.multipoles([0], [1.0], [0, 1], [10.0])
        assert e.value.status == -5
        with pytest.raises(CoffeGpuError) as e:  # N not a power of two
            ctx.integrals_init(k, pk[None, :], [(0, 0)], N=1000)
        assert e.value.status == -1
        with pytest.raises(CoffeGpuError) as e:  # k not increasing
            ctx.integrals_init(k[::-1].copy(), pk[None, :], [(0, 0)], N=1024)
        assert e.value.status == -1
        bad = pk.copy()
        bad[100] = np.nan
        with pytest.raises(CoffeGpuError) as e:  # NaN P(k): the reference would exit
            ctx.integrals_init(k, bad[None, :], [(0, 0)], N=1024)
        assert e.value.status == -4
        ctx.background_init(0.31, 0.05, 9e-5, H, 2000)
        ctx.integrals_init(k, pk[None, :], [(0, 0), (0, 2), (0, 4)], N=1024)
        with pytest.raises(CoffeGpuError) as e:  # spectrum index out of range
            ctx.multipoles([3], [1.0], [0, 1], [10.0])
        assert e.value.status == -1
        with pytest.raises(CoffeGpuError) as e:  # precision mismatch with the tables
            ctx.multipoles([0], [1.0], [0, 1], [10.0], precision="mixed")
        assert e.value.status == -1
        with pytest.raises(CoffeGpuError) as e:  # non-positive separation
            ctx.multipoles([0], [1.0], [0, 3], [10.0, -5.0, 20.0])
        assert e.value.status == -1 and "positive" in str(e.value)
        ok = ctx.multipoles([0], [1.0], [0, 2], [10.0, 20.0])  # the context stays usable
        assert np.isfinite(ok).all()
        assert ctx.launch_count() > 0
