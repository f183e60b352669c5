"""Launch-shape tuning: every configuration of the table stage and of the
mixed multipole kernel gives the default configuration's results (bit for bit
except the FFT radix, which changes the double-float rounding, and the node-loop
unrolling, which may contract a multiply-add differently), and benchmark mode
picks a configuration per shape and reuses it."""
import numpy as np
import pytest

from conftest import H

pytestmark = pytest.mark.gpu

TERMS = [(0, 0), (0, 2), (0, 4)]


@pytest.fixture(scope="module")
def setup():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from coffe_gb300 import workloads
    from coffe_gb300.api import Context

    b = workloads.subset(workloads.cfg3(n_spectra=4), 4)
    ctx = Context(0)
    ctx.background_init(0.31, 0.05, 9e-5, H, 10000)
    yield ctx, b
    ctx.close()


DEFAULT = dict(fft_threads=512, fft_radix=4, fft_swizzle=0, spline_group=8, lane_threads=256,
               lane_unroll=1, fft_threads_fwd=512, lane_pack=1, fft_fused=0, lane_poly=0)


def _tables(ctx, b, precision, **cfg):
    ctx.set_tuning(**{**DEFAULT, **cfg})
    ctx.integrals_init(b.k, b.pk, TERMS, N=4096, precision=precision, small_r=False)
    return np.stack([ctx.integral_table(s, n, l)[1] for s in range(b.pk.shape[0])
                     for n, l in TERMS])


def _multipoles(ctx, b):
    return ctx.multipoles(b.req_spectrum, b.req_z_mean, b.req_offset, b.sep, b.ls,
                          precision="mixed")


def test_table_configurations_agree(setup):
    ctx, b = setup
    ref = _tables(ctx, b, "mixed")
    fin = np.isfinite(ref)
    scale = np.abs(np.where(fin, ref, 0)).max(axis=1, keepdims=True)
    for ft in (128, 256, 512):
        for rad in (2, 4):
            for sw in (0, 1):
                for grp in (2, 4, 8):
                    got = _tables(ctx, b, "mixed", fft_threads=ft, fft_radix=rad,
                                  fft_swizzle=sw, spline_group=grp,
                                  fft_threads_fwd=(256 if grp == 4 else 512))
                    assert np.array_equal(np.isfinite(got), fin)
                    if rad == DEFAULT["fft_radix"]:
                        assert np.array_equal(got[fin], ref[fin]), (ft, rad, sw, grp)
                    else:
                        # float tables from double-float transforms rounded differently
                        e = np.max(np.abs(got - ref)[fin] / np.broadcast_to(scale, ref.shape)[fin])
                        assert e < 1e-7, (ft, rad, sw, grp, e)
    ref64 = _tables(ctx, b, "fp64")
    for ft in (128, 256):
        got = _tables(ctx, b, "fp64", fft_threads=ft, fft_threads_fwd=ft)
        assert np.array_equal(got, ref64, equal_nan=True), ft


def test_fused_table_stage_matches_three_kernels(setup):
    """The one-kernel-per-spectrum mixed table stage runs the same arithmetic as
    the three separate kernels: the tables agree to float rounding."""
    ctx, b = setup
    sep = _tables(ctx, b, "mixed", fft_fused=0)
    fused = _tables(ctx, b, "mixed", fft_fused=1)
    assert ctx.tuning()["fft_fused"] == 1
    fin = np.isfinite(sep)
    assert np.array_equal(fin, np.isfinite(fused))
    scale = np.nanmax(np.abs(sep), axis=1, keepdims=True)
    e = np.max(np.abs(fused - sep)[fin] / np.broadcast_to(scale, sep.shape)[fin])
    print("fused vs three kernels, max |difference| / table scale:", e)
    assert e < 1e-7, e


def test_fused_bulk_copy_rows_match_plain_loads():
    """The fused kernel copies each P(k) row into shared memory with one bulk
    asynchronous copy from the 16-byte boundary at or below the row, and reads
    a row whose rounded end would pass the P(k) array with plain loads.  With
    an odd k-grid length (4095 knots) and three spectra the batch has an
    aligned row, a row 8 bytes past a boundary and a last row read with plain
    loads; a call with one spectrum always takes the plain loads.  The tables
    are bit for bit those of one spectrum per call, for host and device P(k)."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from coffe_gb300 import workloads
    from coffe_gb300.api import Context

    b = workloads.subset(workloads.cfg3(n_spectra=4), 4)
    ctx = Context(0)
    try:
        ctx.background_init(0.31, 0.05, 9e-5, H, 10000)
        ctx.set_tuning(**{**DEFAULT, "fft_fused": 1, "fft_swizzle": 1})
        for k, pk in ((b.k[:-1], b.pk[:3, :-1]), (b.k, b.pk[:3])):
            k, pk = np.ascontiguousarray(k), np.ascontiguousarray(pk)

            def tables(n_spec):
                return np.stack([ctx.integral_table(s, n, l)[1] for s in range(n_spec)
                                 for n, l in TERMS])

            ctx.integrals_init(k, pk, TERMS, N=4096, precision="mixed", small_r=False)
            assert ctx.tuning()["fft_fused"] == 1
            batch = tables(3)
            assert np.isfinite(batch[:, 43:]).all()
            one = []
            for s in range(3):
                ctx.integrals_init(k, pk[s:s + 1], TERMS, N=4096, precision="mixed",
                                   small_r=False)
                one.append(tables(1))
            assert np.array_equal(batch, np.concatenate(one), equal_nan=True), len(k)
            ctx.integrals_init_device(k, torch.from_numpy(pk).cuda(), TERMS, N=4096,
                                      precision="mixed")
            assert np.array_equal(tables(3), batch, equal_nan=True), len(k)
    finally:
        ctx.close()


def test_lane_configurations_agree(setup):
    ctx, b = setup
    _tables(ctx, b, "mixed")
    ref = _multipoles(ctx, b)
    floor = 1e-3 * np.abs(ref).max(axis=0, keepdims=True)
    first = {}
    for po, pk in ((0, 1), (0, 2), (1, 1)):
        for un in (1, 2):
            for lt in (64, 128, 256):
                ctx.set_tuning(**{**DEFAULT, "lane_threads": lt, "lane_unroll": un,
                                  "lane_pack": pk, "lane_poly": po})
                got = _multipoles(ctx, b)
                cfg = ctx.tuning()
                assert (cfg["lane_threads"], cfg["lane_unroll"], cfg["lane_pack"],
                        cfg["lane_poly"]) == (lt, un, pk, po)
                # the block size never changes a result; the unrolled node loop,
                # the packed pair kernel and the polynomial integrand (its
                # coefficients and moment sums in float) may round differently
                first.setdefault((po, pk, un), got)
                assert np.array_equal(got, first[(po, pk, un)]), (lt, un, pk, po)
                e = np.max(np.abs(got - ref) / np.maximum(np.abs(ref), floor))
                print("poly" if po else "node", "pack", pk, "unroll", un, "threads", lt,
                      "vs node kernel", e)
                assert e < (2e-5 if po else 1e-6), (lt, un, pk, po, e)
    assert np.array_equal(first[(0, 1, 1)], ref)


def test_autotune_chooses_and_reuses(setup):
    ctx, b = setup
    _tables(ctx, b, "mixed")
    ref = _multipoles(ctx, b)
    ctx.set_tuning(**DEFAULT)  # forgets earlier choices
    ctx.set_autotune(True)
    try:
        l0 = ctx.launch_count()
        ctx.integrals_init(b.k, b.pk, TERMS, N=4096, precision="mixed", small_r=False)
        got = _multipoles(ctx, b)
        tuned = ctx.launch_count() - l0
        cfg = ctx.tuning()
        l0 = ctx.launch_count()
        ctx.integrals_init(b.k, b.pk, TERMS, N=4096, precision="mixed", small_r=False)
        again = _multipoles(ctx, b)
        plain = ctx.launch_count() - l0
    finally:
        ctx.set_autotune(False)
    print("chosen", cfg, "launches while tuning", tuned, "after", plain)
    assert cfg["fft_threads"] in (128, 256, 512) and cfg["fft_radix"] in (2, 4)
    assert cfg["spline_group"] in (2, 4, 8) and cfg["lane_threads"] in (64, 128, 256)
    assert cfg["lane_unroll"] in (1, 2) and cfg["lane_pack"] in (1, 2)
    assert tuned > 10 * plain  # candidates were timed once, then reused
    assert ctx.tuning() == cfg
    assert np.array_equal(again, got)
    floor = 1e-3 * np.abs(ref).max(axis=0, keepdims=True)
    assert np.max(np.abs(got - ref) / np.maximum(np.abs(ref), floor)) < 1e-5


def test_set_tuning_rejects_bad_values(setup):
    from coffe_gb300.api import CoffeGpuError

    ctx, _ = setup
    for bad in (dict(fft_threads=384), dict(fft_radix=8), dict(fft_swizzle=2),
                dict(spline_group=3), dict(lane_threads=32), dict(lane_unroll=4),
                dict(fft_threads_fwd=100), dict(lane_pack=3), dict(fft_fused=2),
                dict(lane_poly=2)):
        with pytest.raises(CoffeGpuError):
            ctx.set_tuning(**{**DEFAULT, **bad})
    with pytest.raises(ValueError):
        ctx.set_tuning(warp_size=32)
    ctx.set_tuning(**DEFAULT)


def test_pipelined_host_upload_matches_device_input():
    """Host P(k) on the fused table path is uploaded in two parts that overlap
    the tables of the first wave of spectra; the tables equal those made from a
    device copy of the same spectra in one launch, bit for bit."""
    torch = pytest.importorskip("torch")
    from coffe_gb300 import workloads
    from coffe_gb300.api import Context

    b = workloads.cfg3(n_spectra=512)  # more spectra than the device holds blocks of
    ctx = Context(0)
    try:
        ctx.background_init(0.31, 0.05, 9e-5, 0.67, 10000)
        ctx.set_tuning(**{**DEFAULT, "fft_fused": 1, "fft_swizzle": 1})
        pin = torch.from_numpy(np.ascontiguousarray(b.pk)).pin_memory()
        ctx.integrals_init(b.k, pin.numpy(), TERMS, N=4096, precision="mixed", small_r=False)
        host = np.stack([ctx.integral_table(s, n, l)[1] for s in (0, 303, 304, 305, 511)
                         for n, l in TERMS])
        ctx.integrals_init_device(b.k, pin.cuda(), TERMS, N=4096, precision="mixed")
        dev = np.stack([ctx.integral_table(s, n, l)[1] for s in (0, 303, 304, 305, 511)
                        for n, l in TERMS])
        assert np.array_equal(host, dev, equal_nan=True)
    finally:
        ctx.close()


def test_async_tables_then_host_multipoles_match_sync():
    """integrals_init(sync=False) returns once P(k) is on the device; the
    host-array multipole call that follows uploads its requests while the
    tables are still being made: the results equal the synchronous sequence's."""
    torch = pytest.importorskip("torch")
    from coffe_gb300 import workloads
    from coffe_gb300.api import Context

    b = workloads.subset(workloads.cfg3(n_spectra=512), 512)
    ctx = Context(0)
    try:
        ctx.background_init(0.31, 0.05, 9e-5, 0.67, 10000)
        pin = lambda a: torch.from_numpy(np.ascontiguousarray(a)).pin_memory().numpy()
        h_pk, h_sep = pin(b.pk), pin(b.sep)
        out = []
        for sync in (True, False, False):
            ctx.integrals_init(b.k, h_pk, TERMS, N=4096, precision="mixed", small_r=False,
                               sync=sync)
            out.append(ctx.multipoles(b.req_spectrum, b.req_z_mean, b.req_offset, h_sep, b.ls,
                                      precision="mixed").copy())
        assert np.array_equal(out[0], out[1]) and np.array_equal(out[0], out[2])
    finally:
        ctx.close()
