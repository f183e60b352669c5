"""PyTorch autograd surface of the den/RSD (+ lensing) multipoles: derivatives
with respect to the input power spectra and to per-request galaxy-bias and
growth-rate scales, computed by the library's adjoint kernels (no counterpart
in the reference, which has no derivatives).

    mp = multipoles(ctx, k, pk, req_spectrum, req_z_mean, req_offset, sep, ls,
                    bias_scale, growth_scale)
    mp.backward(g)   # pk.grad, bias_scale.grad, growth_scale.grad

``pk`` is a CUDA float64 tensor (n_spectra, nk) on the k grid ``k`` (1/Mpc);
the request tensors follow :meth:`Context.multipoles_async`.  The value is the
first-GK61-panel multipole (coffe_gpu_multipoles_scaled), equal to the
adaptive result wherever the first panel meets the tolerance.  Where QUADPACK
would reject a first panel (and refine it adaptively), the differentiable
value is not the adaptive one: the forward raises :class:`FirstPanelRejected`
unless ``allow_rejected=True`` (the value and gradient then stay the first
panel's for those outputs).  With ``contrib`` including lensing (4), the
full-sky lensing terms on the context's Gauss-Legendre rule
(:meth:`Context.set_lensing_rule`) are added and differentiated too (the
tables then include the six lensing integrals and their sub-Mpc entries).
"""
from __future__ import annotations

import torch

from . import _lib
from .api import DEN_RSD_TERMS, Context

LENS_TERMS = ((0, 0), (0, 2), (0, 4), (1, 1), (1, 3), (2, 0))


class FirstPanelRejected(RuntimeError):
    """Some outputs' first GK61 panel misses the quadrature tolerance: the
    adaptive multipole differs from the differentiable (first-panel) value."""


class _Spec:
    def __init__(self, engine: Context, k, req, ls, contrib, N, allow_rejected=False):
        self.engine, self.k, self.req, self.ls, self.contrib, self.N = engine, k, req, ls, contrib, N
        self.allow_rejected = allow_rejected

    def tables(self, pk):
        """FP64 tables of this spectrum batch for the call's contributions."""
        lens = bool(self.contrib & _lib.LEN)
        self.engine.integrals_init_device(self.k, pk.detach().contiguous(),
                                          LENS_TERMS if lens else DEN_RSD_TERMS, N=self.N,
                                          precision="fp64", small_r=lens, sync=True)


class MultipolesFunction(torch.autograd.Function):
    """(pk, bias_scale, growth_scale) -> multipoles (n_sep, n_l)."""

    @staticmethod
    def forward(fctx, pk, bias_scale, growth_scale, spec: _Spec):
        e = spec.engine
        rs, rz, ro, sep = spec.req
        torch.cuda.synchronize()
        spec.tables(pk)
        out = torch.empty((sep.numel(), len(spec.ls)), dtype=torch.float64, device=pk.device)
        e.multipoles_scaled(rs, rz, ro, sep, sep.numel(), spec.ls, out,
                            bias_scale=bias_scale.detach().contiguous(),
                            growth_scale=growth_scale.detach().contiguous(),
                            contrib=spec.contrib)
        rejected = e.last_retries()
        if rejected > 0 and not spec.allow_rejected:
            raise FirstPanelRejected(
                f"{rejected} outputs' first GK61 panel misses the 1e-5 tolerance: their adaptive "
                "multipole differs from the differentiable first-panel value (pass "
                "allow_rejected=True to differentiate the first panel anyway)")
        fctx.spec = spec
        fctx.save_for_backward(pk, bias_scale, growth_scale)
        return out

    @staticmethod
    def backward(fctx, grad_out):
        pk, bias_scale, growth_scale = fctx.saved_tensors
        spec = fctx.spec
        e = spec.engine
        rs, rz, ro, sep = spec.req
        torch.cuda.synchronize()
        # the tables of this forward's spectra (another forward may have run since)
        spec.tables(pk)
        g_pk = torch.empty_like(pk, dtype=torch.float64)
        g_b = torch.empty_like(bias_scale, dtype=torch.float64)
        g_f = torch.empty_like(growth_scale, dtype=torch.float64)
        e.multipoles_adjoint(rs, rz, ro, sep, sep.numel(), spec.ls,
                             grad_out.detach().to(torch.float64).contiguous(), g_pk, g_b, g_f,
                             bias_scale=bias_scale.detach().contiguous(),
                             growth_scale=growth_scale.detach().contiguous(),
                             contrib=spec.contrib)
        return g_pk, g_b, g_f, None


def multipoles(engine: Context, k, pk, req_spectrum, req_z_mean, req_offset, sep, ls=(0, 2, 4),
               bias_scale=None, growth_scale=None, contrib=_lib.DEN | _lib.RSD, N: int = 4096,
               allow_rejected: bool = False):
    """Differentiable batched den/RSD (+ lensing) multipoles, shape (len(sep), len(ls))."""
    n_req = req_spectrum.numel()
    dev = pk.device
    if bias_scale is None:
        bias_scale = torch.ones(n_req, dtype=torch.float64, device=dev)
    if growth_scale is None:
        growth_scale = torch.ones(n_req, dtype=torch.float64, device=dev)
    spec = _Spec(engine, k, (req_spectrum, req_z_mean, req_offset, sep), tuple(ls), contrib, N,
                 allow_rejected)
    return MultipolesFunction.apply(pk, bias_scale, growth_scale, spec)
