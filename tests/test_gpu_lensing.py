"""GPU parity of the lensing terms (single-integrated den/rsd x lensing and the
double-integrated lensing-lensing term) through the C ABI, against the CPU
oracle with the same split Gauss-Legendre rule, and against the reference's
golden multipoles.

Tolerances: FP64 1e-10 relative, mixed 1e-4 relative, both with a floor of
1e-3 of the largest |value| of the same multipole over the separations;
golden values at the oracle's own golden-test tolerances.
"""
import numpy as np
import pytest

from conftest import H

pytestmark = pytest.mark.gpu

LENS_TERMS = [(0, 0), (0, 2), (0, 4), (1, 1), (1, 3), (2, 0)]
DEN, RSD, LEN = 1, 2, 4


def _rel(got, ref):
    floor = 1e-3 * np.abs(ref).max(axis=0, keepdims=True)
    return np.max(np.abs(got - ref) / np.maximum(np.abs(ref), floor))


def _rel_mixed(got, ref, ls):
    """Mixed-path error: per-multipole floor for l <= 4; for l = 6 the floor is
    1e-3 of the largest |value| of the whole output, because the den+RSD part of
    the l = 6 multipole is ~1e-6 of the monopole (zero in the flat-sky limit)
    and below what an FP32 integrand resolves."""
    floor = 1e-3 * np.abs(ref).max(axis=0, keepdims=True)
    floor = np.where(np.asarray(ls)[None, :] >= 6, 1e-3 * np.abs(ref).max(), floor)
    return np.max(np.abs(got - ref) / np.maximum(np.abs(ref), floor))


@pytest.fixture(scope="module")
def lens_tables(oracle):
    from coffe_gb300 import workloads

    c = workloads.cfg1()
    k, pk = c["k"], c["pk"]
    bg = oracle.background_nodes(0.31, 0.05, 9e-5, H, 10000)
    tabs = [(n, l) + oracle.integral_table(k, pk, n, l, 4096, with_small_r=True)
            for n, l in LENS_TERMS]
    return k, pk, bg, tabs


def _model(oracle, bg, tabs):
    m = oracle.Model(bg, H, 0.31)
    for n, l, x, y in tabs:
        m.set_integral(n, l, x, y)
    return m


@pytest.fixture(scope="module")
def lens_setup(oracle, lens_tables):
    k, pk, bg, tabs = lens_tables
    return k, pk, _model(oracle, bg, tabs)


def _gpu(ctx, k, pk, precision, sep, z, ls, contrib, rule):
    ctx.background_init(0.31, 0.05, 9e-5, H, 10000)
    ctx.integrals_init(k, pk[None, :], LENS_TERMS, N=4096, precision=precision, small_r=True)
    ctx.set_lensing_rule(*rule)
    return ctx.multipoles([0], [z], [0, len(sep)], sep, ls, contrib=contrib, precision=precision)


@pytest.mark.parametrize("contrib", [LEN, DEN | LEN, RSD | LEN, DEN | RSD | LEN])
def test_lensing_fp64_matches_oracle(gpu_ctx, lens_setup, contrib):
    k, pk, m = lens_setup
    sep = np.array([20.0, 55.0, 120.0, 300.0]) / H
    ls = (0, 2, 4, 6)
    rule = (16, 32)
    got = _gpu(gpu_ctx, k, pk, "fp64", sep, 1.5, ls, contrib, rule)
    ref = m.multipoles_lensing(contrib, 1.5, sep, ls, *rule)
    if contrib & (DEN | RSD):
        for j, l in enumerate(ls):
            ref[:, j] += [m.multipole(contrib & 3, 1.5, r, l) for r in sep]
    e = _rel(got, ref)
    print("contrib", contrib, "fp64 max rel error", e)
    assert e < 1e-10, e


@pytest.mark.parametrize("contrib", [LEN, DEN | RSD | LEN])
def test_lensing_fp64_fastalg_matches_oracle(gpu_ctx, lens_setup, contrib):
    """The mixed path's lensing algorithm in FP64 (degree-9 D1/a polynomials along
    the lines of sight, the plane integrand over the five combined records): the
    matched-algorithm baseline of the mixed path, within the polynomials' ~1e-8
    of the oracle's spline lookups."""
    k, pk, m = lens_setup
    sep = np.array([20.0, 55.0, 120.0, 300.0]) / H
    ls = (0, 2, 4, 6)
    rule = (16, 32)
    gpu_ctx.background_init(0.31, 0.05, 9e-5, H, 10000)
    gpu_ctx.integrals_init(k, pk[None, :], LENS_TERMS, N=4096, precision="fp64", small_r=True)
    gpu_ctx.set_lensing_rule(*rule)
    got = gpu_ctx.multipoles([0], [1.5], [0, len(sep)], sep, ls, contrib=contrib,
                             precision="fp64-fastalg")
    ref = m.multipoles_lensing(contrib, 1.5, sep, ls, *rule)
    if contrib & (DEN | RSD):
        for j, l in enumerate(ls):
            ref[:, j] += [m.multipole(contrib & 3, 1.5, r, l) for r in sep]
    # with den+RSD the l = 6 floor of the mixed tests: the degree-5 background
    # polynomials of the den/RSD part (~1e-8 of the monopole) are not resolved
    # against that multipole's own (wide-angle) scale
    e = _rel_mixed(got, ref, ls) if contrib & (DEN | RSD) else _rel(got, ref)
    print("contrib", contrib, "fp64-fastalg max rel error", e)
    assert e < 1e-6, e
    par = gpu_ctx.multipoles([0], [1.5], [0, len(sep)], sep, ls, contrib=contrib,
                             precision="fp64")
    assert not np.array_equal(got, par)  # the other algorithm ran


def test_lensing_mixed_close_to_oracle(gpu_ctx, lens_setup):
    k, pk, m = lens_setup
    sep = np.array([20.0, 55.0, 120.0, 300.0]) / H
    ls = (0, 2, 4, 6)
    rule = (16, 32)
    got = _gpu(gpu_ctx, k, pk, "mixed", sep, 1.5, ls, DEN | RSD | LEN, rule)
    ref = m.multipoles_lensing(DEN | RSD | LEN, 1.5, sep, ls, *rule)
    for j, l in enumerate(ls):
        ref[:, j] += [m.multipole(3, 1.5, r, l) for r in sep]
    e = _rel_mixed(got, ref, ls)
    print("mixed max rel error", e)
    assert e < 1e-4, e
    # the lensing-lensing part alone (FP32 integrand, compensated sums)
    got = _gpu(gpu_ctx, k, pk, "mixed", sep, 1.5, ls, LEN, rule)
    ref = m.multipoles_lensing(LEN, 1.5, sep, ls, *rule)
    e = _rel(got, ref)
    print("mixed len-len max rel error", e)
    assert e < 1e-4, e


@pytest.mark.parametrize("case", ["equal", "different_s", "different_b", "odd_l"])
def test_lensing_tracer_symmetry(oracle, lens_tables, case):
    """The lensing terms are even in mu when both tracers share their biases,
    and each even multipole then sums the rule's mu > 0 half twice (GPU and
    oracle alike), whatever else the list holds; with different magnification
    (or, for density-lensing, galaxy) biases every multipole sums every node.
    FP64 at 1e-10 against the oracle in each case; with odd multipoles in the
    list the even ones equal those of an even-only list bit for bit.  For equal tracers the mirrored sum differs from the
    sum over every node of the same rule only by the rule's own error (the
    plane rule at -mu is the one at mu with x1 and x2 exchanged): on this
    16 x 32 rule 2.3e-3 of the largest l = 4 value, while both are 4.5e-2 away
    from a 128 x 256 rule; the check allows 5e-3."""
    from coffe_gb300.api import Context

    k, pk, bg, tabs = lens_tables
    m = _model(oracle, bg, tabs)  # a model of its own: its biases stay set
    zb = np.linspace(0.0, 5.0, 41)
    s1 = s2 = 0.2 + 0.05 * zb
    b1 = b2 = 1.0 + 0.3 * zb
    if case == "different_s":
        s2 = 0.1 + 0.08 * zb
    if case == "different_b":
        b2 = 1.4 + 0.1 * zb
    ls = (0, 1, 2, 3) if case == "odd_l" else (0, 2, 4)
    sep = np.array([25.0, 90.0, 240.0]) / H
    rule = (16, 32)
    ctx = Context(0)
    try:
        ctx.background_init(0.31, 0.05, 9e-5, H, 10000)
        for which, v in enumerate((b1, b2, s1, s2)):
            m.set_bias(which, zb, v)
            ctx.set_bias(which, zb, v)
        ctx.integrals_init(k, pk[None, :], LENS_TERMS, N=4096, precision="fp64", small_r=True)
        ctx.set_lensing_rule(*rule)
        got = ctx.multipoles([0], [1.2], [0, len(sep)], sep, ls, contrib=DEN | RSD | LEN)
        lens = m.multipoles_lensing(DEN | RSD | LEN, 1.2, sep, ls, *rule)
        nonint = np.array([[m.multipole(3, 1.2, r, l) for l in ls] for r in sep])
        ref = lens + nonint
        even = np.array([l % 2 == 0 for l in ls])
        e = _rel(got[:, even], ref[:, even])
        # odd multipoles of equal tracers vanish: rounding noise of both sides,
        # compared on the scale of the whole output
        e_odd = np.max(np.abs(got[:, ~even] - ref[:, ~even]), initial=0) / np.abs(ref).max()
        print(case, "fp64 max rel error", e, "odd", e_odd)
        assert e < 1e-10 and e_odd < 1e-10, (case, e, e_odd)
        if case == "odd_l":  # the even multipoles do not depend on the list
            # (the nonintegrated part's own rule does: 31 mirrored GK61 nodes for
            # even-only lists, all 61 otherwise, so the totals agree to rounding)
            only_even = ctx.multipoles([0], [1.2], [0, len(sep)], sep, (0, 2),
                                       contrib=DEN | RSD | LEN)
            assert np.allclose(got[:, [0, 2]], only_even, rtol=1e-12, atol=0)
            lens_odd = ctx.multipoles([0], [1.2], [0, len(sep)], sep, ls, contrib=LEN)
            lens_even = ctx.multipoles([0], [1.2], [0, len(sep)], sep, (0, 2), contrib=LEN)
            assert np.array_equal(lens_odd[:, [0, 2]], lens_even)
            assert np.array_equal(lens[:, [0, 2]],
                                  m.multipoles_lensing(DEN | RSD | LEN, 1.2, sep, (0, 2), *rule))
        if case == "equal":
            m.set_bias(3, zb, s2 * (1 + 1e-15))  # other samples: no longer the same tracer
            full = m.multipoles_lensing(DEN | RSD | LEN, 1.2, sep, ls, *rule)
            d = np.abs(full - lens) / np.abs(full).max(axis=0, keepdims=True)
            print("mirrored vs full rule", d.max())
            assert d.max() < 5e-3
    finally:
        ctx.close()


@pytest.mark.parametrize("z,rule", [(1.5, (16, 32)), (0.4, (32, 64))])
def test_lensing_single_integrated_mixed(gpu_ctx, lens_setup, z, rule):
    """The single-integrated den/rsd x lensing term alone on the mixed path
    (FP32 integrand): total minus nonintegrated minus lensing-lensing, against
    the oracle's single term, at 5e-5 of the term's largest |value| per l."""
    k, pk, m = lens_setup
    sep = np.array([15.0, 60.0, 150.0, 350.0]) / H
    ls = (0, 2, 4, 6)
    for contrib in (DEN | LEN, RSD | LEN, DEN | RSD | LEN):
        ref = (m.multipoles_lensing(contrib, z, sep, ls, *rule) -
               m.multipoles_lensing(LEN, z, sep, ls, *rule))
        got = (_gpu(gpu_ctx, k, pk, "mixed", sep, z, ls, contrib, rule) -
               _gpu(gpu_ctx, k, pk, "mixed", sep, z, ls, contrib & 3, rule) -
               _gpu(gpu_ctx, k, pk, "mixed", sep, z, ls, LEN, rule))
        e = np.max(np.abs(got - ref) / np.abs(ref).max(axis=0, keepdims=True))
        print(contrib, z, "single-integrated mixed error", e)
        assert e < 5e-5, (contrib, z, e)


def test_lensing_full_rule_matches_oracle(gpu_ctx, lens_setup):
    """The 128 mu x 256 x rule at two separations (8.4M len-len nodes each)."""
    k, pk, m = lens_setup
    sep = np.array([30.0, 200.0]) / H
    ls = (0, 2, 4, 6)
    for prec, tol in (("fp64", 1e-10), ("mixed", 1e-4)):
        got = _gpu(gpu_ctx, k, pk, prec, sep, 1.5, ls, LEN | DEN | RSD, (128, 256))
        ref = m.multipoles_lensing(LEN | DEN | RSD, 1.5, sep, ls, 128, 256)
        for j, l in enumerate(ls):
            ref[:, j] += [m.multipole(3, 1.5, r, l) for r in sep]
        e = _rel(got, ref) if prec == "fp64" else _rel_mixed(got, ref, ls)
        print(prec, "128x256 max rel error", e)
        assert e < tol, (prec, e)


def test_lensing_golden_through_gpu(gpu_ctx, golden, class_pk):
    """The reference's len and std_len golden multipoles (z = 1, PkL_CLASS),
    with the tolerances of the oracle's golden tests."""
    k, pk = class_pk
    gpu_ctx.background_init(0.3, 0.05, 9e-5, H, 10000)
    gpu_ctx.integrals_init(k, pk[None, :], LENS_TERMS, N=8192, precision="fp64", small_r=True)
    gpu_ctx.set_lensing_rule(128, 256)
    sep = golden["len_multipoles0"][:, 0] / H
    got = gpu_ctx.multipoles([0], [1.0], [0, len(sep)], sep, (0, 2, 4), contrib=LEN)
    far = sep * H >= 100
    for j, l in enumerate((0, 2, 4)):
        ref = golden[f"len_multipoles{l}"][:, 1]
        assert np.allclose(got[far, j], ref[far], rtol=2e-3), (l, got[:, j] / ref - 1)
    got = gpu_ctx.multipoles([0], [1.0], [0, len(sep)], sep, (0, 2, 4), contrib=DEN | RSD | LEN)
    for j, l in enumerate((0, 2, 4)):
        ref = golden[f"std_len_multipoles{l}"][:, 1]
        tol = 5e-4 if l < 4 else 2e-3
        assert np.allclose(got[:, j], ref, rtol=tol), (l, got[:, j] / ref - 1)


def test_lensing_needs_small_r_and_terms(gpu_ctx, lens_setup):
    from coffe_gb300.api import CoffeGpuError

    k, pk, _ = lens_setup
    gpu_ctx.background_init(0.31, 0.05, 9e-5, H, 10000)
    gpu_ctx.integrals_init(k, pk[None, :], LENS_TERMS, N=4096, precision="fp64", small_r=False)
    with pytest.raises(CoffeGpuError) as ei:
        gpu_ctx.multipoles([0], [1.0], [0, 1], [50.0], (0,), contrib=LEN)
    assert ei.value.status == -5
    gpu_ctx.integrals_init(k, pk[None, :], [(0, 0), (0, 2), (0, 4)], N=4096, precision="fp64")
    with pytest.raises(CoffeGpuError) as ei:
        gpu_ctx.multipoles([0], [1.0], [0, 1], [50.0], (0,), contrib=LEN)
    assert ei.value.status == -5


# ------------------------------------------------------------------- flat sky
FLAT_TERMS = [(0, 0), (0, 2), (0, 4), (1, 0), (1, 2), (1, 4), (3, 1, 1), (5, 3, 1), (7, 5, 1)]
ONLY_CROSS = 8


@pytest.fixture(scope="module")
def flat_setup(oracle):
    from coffe_gb300 import workloads

    c = workloads.cfg1()
    k, pk = c["k"], c["pk"]
    bg = oracle.background_nodes(0.31, 0.05, 9e-5, H, 10000)
    m = oracle.Model(bg, H, 0.31)
    for t in FLAT_TERMS:
        if len(t) == 3:
            x, y = oracle.integral_table_half(k, pk, t[0], t[1], 4096)
            m.set_integral_half(t[0], t[1], x, y)
        else:
            x, y = oracle.integral_table(k, pk, t[0], t[1], 4096, with_small_r=True)
            m.set_integral(t[0], t[1], x, y)
    return k, pk, m


@pytest.mark.parametrize("prec,tol", [("fp64", 1e-10), ("mixed", 1e-4)])
def test_flatsky_lensing_matches_oracle(gpu_ctx, flat_setup, prec, tol):
    """den + flat-sky density-lensing + flat-sky lensing-lensing (l = 0, 2, 4)."""
    k, pk, m = flat_setup
    sep = np.array([20.0, 55.0, 120.0, 300.0]) / H
    ls = (0, 2, 4)
    gpu_ctx.background_init(0.31, 0.05, 9e-5, H, 10000)
    gpu_ctx.integrals_init(k, pk[None, :], FLAT_TERMS, N=4096, precision=prec, small_r=True)
    gpu_ctx.set_flatsky(True, True)
    try:
        got = gpu_ctx.multipoles([0], [1.5], [0, len(sep)], sep, ls, contrib=DEN | LEN,
                                 precision=prec)
    finally:
        gpu_ctx.set_flatsky(False, False)
    ref = np.array([[m.multipole(DEN, 1.5, r, l) + m.flatsky_density_lensing(1.5, r, l) +
                     m.flatsky_lensing_lensing(1.5, r, l) for l in ls] for r in sep])
    e = _rel(got, ref)
    print(prec, "flat-sky max rel error", e)
    assert e < tol, e


def test_flatsky_golden_through_gpu(gpu_ctx, golden, class_pk):
    """The reference's flat-sky golden multipoles (test_coffe.py:328-380): lensing-
    lensing alone, and density-lensing with only cross-correlations."""
    k, pk = class_pk
    gpu_ctx.background_init(0.3, 0.05, 9e-5, H, 10000)
    gpu_ctx.integrals_init(k, pk[None, :], FLAT_TERMS, N=8192, precision="fp64", small_r=True)
    sep = golden["flatsky_lensing_lensing_multipoles0"][:, 0] / H
    try:
        gpu_ctx.set_flatsky(False, True)
        ll = gpu_ctx.multipoles([0], [1.0], [0, len(sep)], sep, (0, 2, 4), contrib=LEN)
        gpu_ctx.set_flatsky(True, True)
        dl = gpu_ctx.multipoles([0], [1.0], [0, len(sep)], sep, (0, 2, 4),
                                contrib=DEN | LEN | ONLY_CROSS)
    finally:
        gpu_ctx.set_flatsky(False, False)
    for j, l in enumerate((0, 2, 4)):
        assert np.allclose(ll[:, j], golden[f"flatsky_lensing_lensing_multipoles{l}"][:, 1],
                           rtol=5e-4), (l, ll[:, j])
        assert np.allclose(dl[:, j], golden[f"flatsky_density_lensing_multipoles{l}"][:, 1],
                           rtol=5e-4), (l, dl[:, j])
