"""A batched step (FFTLog tables + multipoles on device buffers) captured as a
CUDA graph replays to the direct launch's output bit for bit, also when steps
of the other precision (and another multipole list) ran directly between the
capture and the replay."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TERMS = ((0, 0), (0, 2), (0, 4))


def test_graph_replay_matches_direct_launch():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from coffe_gb300 import workloads
    from coffe_gb300.api import Context

    b = workloads.subset(workloads.cfg3(n_spectra=16), 16)
    c = b.cosmo
    dev = torch.device("cuda:0")
    stream = torch.cuda.Stream(device=dev)
    ctx = Context(0)
    try:
        with torch.cuda.stream(stream):
            ctx.set_stream(stream.cuda_stream)
            ctx.background_init(c.omega_m, c.omega_baryon, c.omega_gamma, c.h, 10000)
            pk = torch.from_numpy(b.pk).to(dev)
            rs = torch.from_numpy(b.req_spectrum).to(dev)
            rz = torch.from_numpy(b.req_z_mean).to(dev)
            ro = torch.from_numpy(b.req_offset).to(dev)
            sep = torch.from_numpy(b.sep).to(dev)
            n = len(b.sep)
            outs = {p: torch.empty((n, 3), dtype=torch.float64, device=dev)
                    for p in ("mixed", "fp64")}

            def step(prec, ls=(0, 2, 4), out=None):
                ctx.integrals_init_device(b.k, pk, TERMS, N=4096, precision=prec, sync=False)
                ctx.multipoles_async(rs, rz, ro, sep, n, ls,
                                     outs[prec] if out is None else out, precision=prec)

            for prec in ("mixed", "fp64"):
                ctx.integrals_init_device(b.k, pk, TERMS, N=4096, precision=prec, sync=True)
                step(prec)
            ctx.synchronize()
            graphs = {}
            for prec in ("mixed", "fp64"):
                step(prec)
                ctx.synchronize()
                g = torch.cuda.CUDAGraph()
                with torch.cuda.graph(g, stream=stream):
                    step(prec)
                graphs[prec] = g
            # direct launches of the other precision and of another l list
            # between the capture and the replays
            extra = torch.empty((n, 2), dtype=torch.float64, device=dev)
            step("fp64", ls=(0, 2), out=extra)
            step("mixed", ls=(0, 2), out=extra)
            replayed = {}
            for prec in ("mixed", "fp64"):
                outs[prec].fill_(np.nan)
                graphs[prec].replay()
                ctx.synchronize()
                replayed[prec] = outs[prec].clone()
            for prec in ("mixed", "fp64"):
                outs[prec].fill_(np.nan)
                step(prec)
                ctx.synchronize()
                assert torch.equal(replayed[prec], outs[prec]), prec
            assert torch.isfinite(outs["mixed"]).all()
    finally:
        ctx.set_stream(None)
        ctx.close()
