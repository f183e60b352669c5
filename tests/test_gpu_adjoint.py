"""Derivatives of the den/RSD multipoles (adjoint kernels through the C ABI and
the torch.autograd surface) against central finite differences with relative
step 1e-4, at 1e-6 relative agreement; and the differentiable value against
the adaptive forward path."""
import numpy as np
import pytest

from conftest import H

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def setup():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from coffe_gb300 import workloads
    from coffe_gb300.api import Context

    c = workloads.cfg1()
    ctx = Context(0)
    ctx.background_init(0.31, 0.05, 9e-5, H, 10000)
    dev = torch.device("cuda:0")
    sep = c["sep"]
    req = (torch.tensor([0], dtype=torch.int32, device=dev),
           torch.tensor([1.0], dtype=torch.float64, device=dev),
           torch.tensor([0, len(sep)], dtype=torch.int64, device=dev),
           torch.tensor(sep, dtype=torch.float64, device=dev))
    pk = torch.tensor(c["pk"][None, :], dtype=torch.float64, device=dev)
    yield torch, ctx, c, req, pk
    ctx.close()


def _value(torch, ctx, c, req, pk, beta=1.0, alpha=1.0, ls=(0, 2, 4)):
    rs, rz, ro, sep = req
    ctx.integrals_init_device(c["k"], pk, N=4096, precision="fp64")
    out = torch.empty((sep.numel(), len(ls)), dtype=torch.float64, device="cuda:0")
    b = torch.full((rs.numel(),), beta, dtype=torch.float64, device="cuda:0")
    f = torch.full((rs.numel(),), alpha, dtype=torch.float64, device="cuda:0")
    ctx.multipoles_scaled(rs, rz, ro, sep, sep.numel(), ls, out, bias_scale=b, growth_scale=f)
    return out.cpu().numpy()


def _adjoint(torch, ctx, c, req, pk, G, ls=(0, 2, 4)):
    rs, rz, ro, sep = req
    ctx.integrals_init_device(c["k"], pk, N=4096, precision="fp64")
    g_pk = torch.empty_like(pk)
    g_b = torch.empty(rs.numel(), dtype=torch.float64, device="cuda:0")
    g_f = torch.empty_like(g_b)
    Gt = torch.tensor(G, dtype=torch.float64, device="cuda:0")
    ctx.multipoles_adjoint(rs, rz, ro, sep, sep.numel(), ls, Gt, g_pk, g_b, g_f)
    return g_pk.cpu().numpy(), g_b.cpu().numpy(), g_f.cpu().numpy()


def test_scaled_value_matches_forward(setup):
    torch, ctx, c, req, pk = setup
    v = _value(torch, ctx, c, req, pk)
    ctx.integrals_init(c["k"], c["pk"][None, :], [(0, 0), (0, 2), (0, 4)], N=4096,
                       precision="fp64", small_r=False)
    ref = ctx.multipoles([0], [1.0], [0, len(c["sep"])], c["sep"], (0, 2, 4), precision="fp64")
    floor = 1e-3 * np.abs(ref).max(axis=0)
    e = np.max(np.abs(v - ref) / np.maximum(np.abs(ref), floor))
    print("first-panel value vs adaptive forward", e, "retries", ctx.last_retries())
    assert e < 1e-10, e


def _smooth_direction(rng, k):
    """A random smooth relative perturbation of P(k): three sinusoids in ln k.
    Rough per-node noise is avoided on purpose: the tables inherit it, and the
    Akima slope weights |m_{i+1} - m_i| of the table lookup are not
    differentiable where two secants cross, which a +-1e-4 step over noise
    crosses often (the adjoint is the exact one-sided derivative there)."""
    lnk = np.log(k)
    return sum(np.sin(rng.uniform(0.1, 2.0) * lnk + rng.uniform(0, 2 * np.pi)) for _ in range(3))


def test_pk_gradient_matches_finite_differences(setup):
    torch, ctx, c, req, pk = setup
    rng = np.random.default_rng(7)
    G = rng.normal(size=(len(c["sep"]), 3))
    g_pk, _, _ = _adjoint(torch, ctx, c, req, pk, G)
    P = c["pk"]
    # Euler: the tables are linear in P and Akima interpolation is homogeneous
    # of degree one, so <dL/dP, P> = L exactly
    L = np.sum(G * _value(torch, ctx, c, req, pk))
    assert abs(np.sum(g_pk[0] * P) - L) <= 1e-12 * np.abs(G * _value(torch, ctx, c, req, pk)).sum()
    eps = 1e-4
    for trial in range(4):
        v = _smooth_direction(rng, c["k"])
        Lp = np.sum(G * _value(torch, ctx, c, req, torch.tensor((P * (1 + eps * v))[None, :], device="cuda:0")))
        Lm = np.sum(G * _value(torch, ctx, c, req, torch.tensor((P * (1 - eps * v))[None, :], device="cuda:0")))
        fd = (Lp - Lm) / (2 * eps)
        ad = np.sum(g_pk[0] * P * v)
        print("direction", trial, "fd", fd, "adjoint", ad)
        assert abs(fd - ad) <= 1e-6 * abs(fd), (fd, ad)
    # single k nodes below 0.1 h/Mpc where the multipoles are most sensitive (a
    # bump at higher k makes the tables oscillate on the scale of their own
    # knot spacing, where the Akima weights switch within the step)
    sens = np.abs(g_pk[0] * P) * (c["k"] < 0.1 * H)
    for i in np.argsort(sens)[-4:]:
        d = np.zeros_like(P)
        d[i] = P[i] * eps
        Lp = np.sum(G * _value(torch, ctx, c, req, torch.tensor((P + d)[None, :], device="cuda:0")))
        Lm = np.sum(G * _value(torch, ctx, c, req, torch.tensor((P - d)[None, :], device="cuda:0")))
        fd = (Lp - Lm) / (2 * eps)
        ad = g_pk[0, i] * P[i]
        print("k index", i, "fd", fd, "adjoint", ad)
        assert abs(fd - ad) <= 1e-6 * abs(fd), (i, fd, ad)


def test_bias_and_growth_gradients_match_finite_differences(setup):
    torch, ctx, c, req, pk = setup
    rng = np.random.default_rng(8)
    G = rng.normal(size=(len(c["sep"]), 3))
    _, g_b, g_f = _adjoint(torch, ctx, c, req, pk, G)
    eps = 1e-4
    fd_b = (np.sum(G * _value(torch, ctx, c, req, pk, beta=1 + eps)) -
            np.sum(G * _value(torch, ctx, c, req, pk, beta=1 - eps))) / (2 * eps)
    fd_f = (np.sum(G * _value(torch, ctx, c, req, pk, alpha=1 + eps)) -
            np.sum(G * _value(torch, ctx, c, req, pk, alpha=1 - eps))) / (2 * eps)
    print("bias", fd_b, g_b[0], "growth", fd_f, g_f[0])
    assert abs(fd_b - g_b[0]) <= 1e-6 * abs(fd_b)
    assert abs(fd_f - g_f[0]) <= 1e-6 * abs(fd_f)


def test_autograd_function(setup):
    torch, ctx, c, req, pk = setup
    from coffe_gb300.autograd import multipoles

    rs, rz, ro, sep = req
    p = pk.clone().requires_grad_(True)
    b = torch.ones(1, dtype=torch.float64, device="cuda:0", requires_grad=True)
    f = torch.ones(1, dtype=torch.float64, device="cuda:0", requires_grad=True)
    mp = multipoles(ctx, c["k"], p, rs, rz, ro, sep, (0, 2, 4), b, f)
    rng = np.random.default_rng(9)
    G = rng.normal(size=tuple(mp.shape))
    (mp * torch.tensor(G, device="cuda:0")).sum().backward()
    g_pk, g_b, g_f = _adjoint(torch, ctx, c, req, pk, G)
    assert np.allclose(p.grad.cpu().numpy(), g_pk, rtol=1e-12, atol=0)
    assert np.allclose(b.grad.cpu().numpy(), g_b, rtol=1e-12)
    assert np.allclose(f.grad.cpu().numpy(), g_f, rtol=1e-12)


def test_batched_gradients_per_spectrum(setup):
    """Two spectra x six redshifts: each spectrum's gradient only sees its own
    requests (directional finite differences per spectrum)."""
    torch, ctx, _, _, _ = setup
    from coffe_gb300 import workloads

    b = workloads.subset(workloads.cfg3(n_spectra=2), 2)
    dev = "cuda:0"
    req = (torch.tensor(b.req_spectrum, device=dev), torch.tensor(b.req_z_mean, device=dev),
           torch.tensor(b.req_offset, device=dev), torch.tensor(b.sep, device=dev))
    c = {"k": b.k, "sep": b.sep}
    pk = torch.tensor(b.pk, device=dev)
    rng = np.random.default_rng(10)
    G = rng.normal(size=(len(b.sep), 3))
    g_pk, g_b, g_f = _adjoint(torch, ctx, c, req, pk, G)
    eps = 1e-4
    for s in range(2):
        v = np.zeros_like(b.pk)
        v[s] = _smooth_direction(rng, b.k)
        Lp = np.sum(G * _value(torch, ctx, c, req, torch.tensor(b.pk * (1 + eps * v), device=dev)))
        Lm = np.sum(G * _value(torch, ctx, c, req, torch.tensor(b.pk * (1 - eps * v), device=dev)))
        fd = (Lp - Lm) / (2 * eps)
        ad = np.sum(g_pk * b.pk * v)
        print("spectrum", s, fd, ad)
        assert abs(fd - ad) <= 1e-6 * abs(fd)
    assert g_b.shape == (len(b.req_spectrum),) and np.all(np.isfinite(g_b)) and np.all(np.isfinite(g_f))


def test_rejected_first_panels_are_counted_and_raise(setup):
    """At a separation where the monopole crosses zero, QUADPACK rejects the
    first panel (its tolerance, 1e-5 of a vanishing value, is below the
    round-off floor): the differentiable forward counts that output as the
    adaptive forward does, and the autograd surface refuses to differentiate a
    value that is not the adaptive one unless told to."""
    torch, ctx, c, req, pk = setup
    from coffe_gb300.autograd import FirstPanelRejected, multipoles

    ctx.integrals_init(c["k"], c["pk"][None, :], [(0, 0), (0, 2), (0, 4)], N=4096,
                       precision="fp64", small_r=False)

    def mono(r):
        return ctx.multipoles([0], [1.0], [0, len(r)], r, (0,), precision="fp64")[:, 0]

    r = np.linspace(60, 140, 161) / H
    v = mono(r)
    i = np.where(np.sign(v[:-1]) != np.sign(v[1:]))[0][0]
    a, b = r[i], r[i + 1]
    fa = v[i]
    for _ in range(60):  # bisection to the double-precision zero crossing
        m = 0.5 * (a + b)
        fm = mono(np.array([m]))[0]
        if np.sign(fm) == np.sign(fa):
            a, fa = m, fm
        else:
            b = m
    seps = np.array([a, 100 / H, b])
    ctx.multipoles([0], [1.0], [0, 3], seps, (0, 2, 4), precision="fp64")
    n_adaptive = ctx.last_retries()
    assert n_adaptive >= 1
    dev = "cuda:0"
    rq = (torch.tensor([0], dtype=torch.int32, device=dev),
          torch.tensor([1.0], dtype=torch.float64, device=dev),
          torch.tensor([0, 3], dtype=torch.int64, device=dev),
          torch.tensor(seps, dtype=torch.float64, device=dev))
    out = torch.empty((3, 3), dtype=torch.float64, device=dev)
    ctx.integrals_init_device(c["k"], pk, N=4096, precision="fp64")
    ctx.multipoles_scaled(*rq, 3, (0, 2, 4), out)
    assert ctx.last_retries() == n_adaptive
    p = pk.clone().requires_grad_(True)
    with pytest.raises(FirstPanelRejected):
        multipoles(ctx, c["k"], p, *rq, (0, 2, 4))
    mp = multipoles(ctx, c["k"], p, *rq, (0, 2, 4), allow_rejected=True)
    mp.sum().backward()
    assert torch.isfinite(p.grad).all()


# ------------------------------------------------------------------ lensing
LENS_TERMS = ((0, 0), (0, 2), (0, 4), (1, 1), (1, 3), (2, 0))
DEN, RSD, LEN = 1, 2, 4


@pytest.fixture(scope="module")
def lens_setup(setup):
    torch, ctx, c, req, pk = setup
    dev = torch.device("cuda:0")
    sep = np.array([20.0, 55.0, 120.0, 300.0]) / H
    lreq = (torch.tensor([0], dtype=torch.int32, device=dev),
            torch.tensor([1.5], dtype=torch.float64, device=dev),
            torch.tensor([0, len(sep)], dtype=torch.int64, device=dev),
            torch.tensor(sep, dtype=torch.float64, device=dev))
    return torch, ctx, c, lreq, pk


def _lens_value(torch, ctx, c, req, pk, contrib, beta=1.0, alpha=1.0, ls=(0, 2, 4)):
    rs, rz, ro, sep = req
    ctx.set_lensing_rule(16, 32)
    ctx.integrals_init_device(c["k"], pk, LENS_TERMS, N=4096, precision="fp64", small_r=True)
    out = torch.empty((sep.numel(), len(ls)), dtype=torch.float64, device="cuda:0")
    b = torch.full((rs.numel(),), beta, dtype=torch.float64, device="cuda:0")
    f = torch.full((rs.numel(),), alpha, dtype=torch.float64, device="cuda:0")
    ctx.multipoles_scaled(rs, rz, ro, sep, sep.numel(), ls, out, bias_scale=b, growth_scale=f,
                          contrib=contrib)
    return out.cpu().numpy()


def _lens_adjoint(torch, ctx, c, req, pk, G, contrib, ls=(0, 2, 4)):
    rs, rz, ro, sep = req
    ctx.set_lensing_rule(16, 32)
    ctx.integrals_init_device(c["k"], pk, LENS_TERMS, N=4096, precision="fp64", small_r=True)
    g_pk = torch.empty_like(pk)
    g_b = torch.empty(rs.numel(), dtype=torch.float64, device="cuda:0")
    g_f = torch.empty_like(g_b)
    Gt = torch.tensor(G, dtype=torch.float64, device="cuda:0")
    ctx.multipoles_adjoint(rs, rz, ro, sep, sep.numel(), ls, Gt, g_pk, g_b, g_f, contrib=contrib)
    return g_pk.cpu().numpy(), g_b.cpu().numpy(), g_f.cpu().numpy()


@pytest.mark.parametrize("contrib", [LEN, DEN | RSD | LEN])
def test_lensing_scaled_value_matches_forward(lens_setup, contrib):
    """The differentiable lensing multipoles are the forward call's (same rule,
    mu symmetry and weights; den/RSD on their first panel)."""
    torch, ctx, c, req, pk = lens_setup
    v = _lens_value(torch, ctx, c, req, pk, contrib)
    sep = req[3].cpu().numpy()
    ref = ctx.multipoles([0], [1.5], [0, len(sep)], sep, (0, 2, 4), contrib=contrib,
                         precision="fp64")
    floor = 1e-3 * np.abs(ref).max(axis=0)
    e = np.max(np.abs(v - ref) / np.maximum(np.abs(ref), floor))
    print("contrib", contrib, "differentiable value vs forward", e)
    assert e < 1e-10, e


@pytest.mark.parametrize("contrib", [LEN, DEN | RSD | LEN])
def test_lensing_pk_gradient_matches_finite_differences(lens_setup, contrib):
    """d(multipoles)/dP(k) through the lensing integrands, the Akima records
    of the six tables, the FFTLog transforms and the sub-Mpc QAG entries."""
    torch, ctx, c, req, pk = lens_setup
    rng = np.random.default_rng(11)
    G = rng.normal(size=(req[3].numel(), 3))
    g_pk, _, _ = _lens_adjoint(torch, ctx, c, req, pk, G, contrib)
    assert np.all(np.isfinite(g_pk))
    P = c["pk"]
    val = _lens_value(torch, ctx, c, req, pk, contrib)
    L = np.sum(G * val)
    euler = np.sum(g_pk[0] * P)
    print("Euler <dL/dP, P>", euler, "L", L)
    assert abs(euler - L) <= 1e-11 * np.abs(G * val).sum(), (euler, L)
    eps = 1e-4
    for trial in range(3):
        v = _smooth_direction(rng, c["k"])
        Lp = np.sum(G * _lens_value(torch, ctx, c, req,
                                    torch.tensor((P * (1 + eps * v))[None, :], device="cuda:0"),
                                    contrib))
        Lm = np.sum(G * _lens_value(torch, ctx, c, req,
                                    torch.tensor((P * (1 - eps * v))[None, :], device="cuda:0"),
                                    contrib))
        fd = (Lp - Lm) / (2 * eps)
        ad = np.sum(g_pk[0] * P * v)
        print("direction", trial, "fd", fd, "adjoint", ad)
        assert abs(fd - ad) <= 1e-6 * abs(fd), (fd, ad)


def test_lensing_bias_and_growth_gradients(lens_setup):
    """The den-lensing part scales with the bias scale, the RSD-lensing part
    with the growth scale, the lensing-lensing part with neither."""
    torch, ctx, c, req, pk = lens_setup
    rng = np.random.default_rng(12)
    G = rng.normal(size=(req[3].numel(), 3))
    contrib = DEN | RSD | LEN
    _, g_b, g_f = _lens_adjoint(torch, ctx, c, req, pk, G, contrib)
    eps = 1e-4
    fd_b = (np.sum(G * _lens_value(torch, ctx, c, req, pk, contrib, beta=1 + eps)) -
            np.sum(G * _lens_value(torch, ctx, c, req, pk, contrib, beta=1 - eps))) / (2 * eps)
    fd_f = (np.sum(G * _lens_value(torch, ctx, c, req, pk, contrib, alpha=1 + eps)) -
            np.sum(G * _lens_value(torch, ctx, c, req, pk, contrib, alpha=1 - eps))) / (2 * eps)
    print("bias", fd_b, g_b[0], "growth", fd_f, g_f[0])
    assert abs(fd_b - g_b[0]) <= 1e-7 * abs(fd_b)
    assert abs(fd_f - g_f[0]) <= 1e-7 * abs(fd_f)


def test_autograd_function_with_lensing(lens_setup):
    torch, ctx, c, req, pk = lens_setup
    from coffe_gb300.autograd import multipoles

    rs, rz, ro, sep = req
    ctx.set_lensing_rule(16, 32)
    p = pk.clone().requires_grad_(True)
    b = torch.ones(1, dtype=torch.float64, device="cuda:0", requires_grad=True)
    f = torch.ones(1, dtype=torch.float64, device="cuda:0", requires_grad=True)
    mp = multipoles(ctx, c["k"], p, rs, rz, ro, sep, (0, 2, 4), b, f, contrib=DEN | RSD | LEN)
    assert np.allclose(mp.detach().cpu().numpy(),
                       _lens_value(torch, ctx, c, req, pk, DEN | RSD | LEN), rtol=1e-14, atol=0)
    rng = np.random.default_rng(13)
    G = rng.normal(size=tuple(mp.shape))
    (mp * torch.tensor(G, device="cuda:0")).sum().backward()
    g_pk, g_b, g_f = _lens_adjoint(torch, ctx, c, req, pk, G, DEN | RSD | LEN)
    assert np.allclose(p.grad.cpu().numpy(), g_pk, rtol=1e-10, atol=1e-12 * np.abs(g_pk).max())
    assert np.allclose(b.grad.cpu().numpy(), g_b, rtol=1e-10)
    assert np.allclose(f.grad.cpu().numpy(), g_f, rtol=1e-10)
