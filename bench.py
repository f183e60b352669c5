#!/usr/bin/env python
"""Benchmark of the batched multipole path (FFTLog I_l^n tables + den/RSD
multipole quadrature) on GB300.

Workload (one "step"): 512 seeded BBKS spectra (sigma8 ~ U[0.7,0.9],
n_s ~ U[0.93,1.0], Gamma ~ U[0.15,0.3]) x 6 mean redshifts in [0.5, 2] x
l = 0, 2, 4, each (spectrum, z) request carrying 20-400 separations uniform in
[5, 250] Mpc/h: FFTLog tables of I_0^0, I_2^0, I_4^0 on N = 4096 points for
every spectrum, then every multipole by GK61 QAG.  Metric: multipole
evaluations per second (one evaluation = one (spectrum, z, l, r) output).

Arms:
  default           : the GPU path (mixed precision headline; FP64 path beside it)
  --impl reference  : the reference algorithm on the host cores (the CPU oracle,
                      a C restatement: the reference itself cannot be built here),
                      on a bounded sample of the same workload.

Prints one JSON line (rank 0).  Multi-GPU (torchrun): independent replicas,
one batch per rank ("weak" scaling), times max-reduced over ranks.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

METRIC = "multipole evals/s at <=1e-4 rel err vs FP64: batched mixed vs plain FP64 on 1 GB300"
UNIT = "evals/s"
TERMS = ((0, 0), (0, 2), (0, 4))
N_FFT = 4096
# FLOP of one multipole-quadrature node of the mixed kernel (mp_fast_kernel<3,3>,
# counted from multipoles.cu, FMA = 2): chi1/chi2 4, D1 and f D1 at both ends
# from the per-request degree-5 polynomials 18,
# D, 1/D, s, c 6, density 2, RSD polynomial 16, density-RSD 16, Kronrod
# (Kahan) / Gauss / |f| sums 27, second-pass resasc sums 12
FLOP_PER_NODE = 101
# per (request, separation): chi(z_mean) 8, three Akima table lookups 141,
# per-pair constants 14, QUADPACK acceptance test of three multipoles 57
FLOP_PER_PAIR_EXTRA = 220
# nodes evaluated per (request, separation): the integrand is even in mu for the
# benchmark's equal tracers and even multipoles, so the kernel evaluates the 31
# GK61 nodes with mu >= 0 (the other 30 are their mirror images)
NODES = 31
# FLOP of one (request, separation) of the polynomial-integrand kernel
# (mp_poly_kernel<3,3>, counted from multipoles.cu, FMA = 2): the integrand's
# coefficients in mu^2 662 (density 51, 1/D series and c 21, c^2 66, RSD
# quadratics 24, R(c) 84, F1 F2 45, F1 F2 R 78, A 45, B 39, the K1 term 13, Q 32,
# (1 + c)(1 - w) 7, g 73, g Q 84), the Kronrod and Gauss moment sums 111, the 31
# nodes x 34 (Horner 16, QUADPACK's |f| and |f - mean| sums 18) and the per-pair
# lookups and acceptance test 220
FLOP_PER_PAIR_POLY = 662 + 111 + 31 * 34 + 220
# bytes of the fused table kernel per spectrum (algorithmic): the FP64 spectrum
# in (8 B per knot) and the float tables out (4 B x (N + 43) per term)
TABLE_BYTES_PER_SPECTRUM = 8 * 4096 + 4 * (4096 + 43) * 3
# its DRAM traffic per launch from the ncu capture of the full batch
# (dram__bytes_read.sum + dram__bytes_write.sum: the spectra are read, the
# tables stay in L2 during the kernel)
TABLE_DRAM_BYTES_PER_LAUNCH = 17.168384e6
# the FP64 instantiation of the same kernel (COFFE_GPU_FP64_FASTALG) has no
# Kahan compensation: 3 fewer operations per multipole and node
FLOP_PER_NODE_FP64_FASTALG = FLOP_PER_NODE - 9
# the FP64 parity kernel (mp_lane_kernel<3, double>): the reference algebra per
# node with the background from spline records (z(chi) cursors, f/D1 records)
FLOP_PER_NODE_LANE = 170
PRECISIONS = ("mixed", "fp64", "fp64-fastalg")
# FFTLog table stage, per transform of N = 4096 real points (FMA = 2):
#   FFT 2.5 N log2 N, kernel multiply 6 (N/2 + 1), prefactor N (inverse);
#   resampling ~10 N and the real-FFT post-pass ~10 N/2 (forward)
FFT_FLOP = 2.5 * N_FFT * 12
INV_FLOP = FFT_FLOP + 6 * (N_FFT // 2 + 1) + N_FFT
FWD_FLOP = FFT_FLOP + 10 * N_FFT + 5 * N_FFT
# HBM bytes per transform: the inverse reads the half spectrum (N/2+1 complex
# float on the mixed path, double on the FP64 path) and writes the table
# (float / double)
INV_BYTES = {"mixed": 8 * (N_FFT // 2 + 1) + 4 * N_FFT, "fp64": 16 * (N_FFT // 2 + 1) + 8 * N_FFT}


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=500)
    p.add_argument("--warmup", type=int, default=5)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--n-spectra", type=int, default=512)
    p.add_argument("--fp64-steps", type=int, default=0, help="0: max(3, steps // 50)")
    p.add_argument("--cpu-spectra", type=int, default=48, help="CPU baseline sample size")
    p.add_argument("--no-cpu", action="store_true")
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--no-graph", action="store_true",
                   help="launch the step's kernels directly instead of replaying a CUDA graph")
    p.add_argument("--no-extras", action="store_true",
                   help="skip the lensing / covariance / gradient workload timings")
    p.add_argument("--no-clocks", action="store_true")
    p.add_argument("--no-autotune", action="store_true",
                   help="keep the default launch configuration instead of timing candidates")
    p.add_argument("--launch-config", default=None,
                   help="fixed launch configuration instead of autotuning, e.g. "
                        "fft_threads=512,fft_radix=4,fft_swizzle=1,spline_group=8,"
                        "lane_threads=128,lane_unroll=2,fft_threads_fwd=256 (profiling runs)")
    p.add_argument("--kernel-only",
                   choices=["mixed", "fp64", "tables-mixed", "tables-fp64", "lensing-mixed"],
                   default=None,
                   help="profiling aid: run only the multipole kernel (mixed/fp64), only the "
                        "FFTLog tables (tables-*) or only the config-4 lensing multipoles "
                        "(lensing-mixed, --lensing-seps separations) `steps` times")
    p.add_argument("--lensing-seps", type=int, default=200,
                   help="separations of the lensing-mixed profiling run (config 4 has 200)")
    return p.parse_args()


# ------------------------------------------------------------------- clocks
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int, enabled: bool = True):
        self.device = device
        self.enabled = enabled
        self.proc = None

    def __enter__(self):
        if not self.enabled:
            return self
        self.tmp = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=self.tmp, stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        time.sleep(0.25)
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            time.sleep(0.15)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.enabled or self.proc is None:
            return None
        self.tmp.flush()
        rows = []
        with open(self.tmp.name) as fh:
            for line in fh:
                parts = [x.strip() for x in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        os.unlink(self.tmp.name)
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons, "samples": len(rows)}


# ------------------------------------------------------------- CPU baseline
def cpu_eval(batch, n_spectra, nthreads):
    """The oracle (FP64 C restatement, OpenMP) on the first n_spectra spectra."""
    import oracle as orc
    from coffe_gb300 import workloads

    b = workloads.subset(batch, n_spectra)
    c = b.cosmo
    bg = orc.background_nodes(c.omega_m, c.omega_baryon, c.omega_gamma, c.h, 10000)
    t0 = time.perf_counter()
    out = np.zeros((len(b.sep), len(b.ls)))
    for s in range(n_spectra):
        m = orc.Model(bg, c.h, c.omega_m)
        for n, l in TERMS:
            m.set_integral(n, l, *orc.integral_table(b.k, b.pk[s], n, l, N_FFT, with_small_r=False))
        qs = np.where(b.req_spectrum == s)[0]
        lo, hi = int(b.req_offset[qs[0]]), int(b.req_offset[qs[-1] + 1])
        zz = np.repeat(b.req_z_mean[qs], np.diff(b.req_offset[qs[0]: qs[-1] + 2]))
        for j, l in enumerate(b.ls):
            out[lo:hi, j] = m.multipoles_batch(3, zz, b.sep[lo:hi], np.full(hi - lo, l),
                                               nthreads=nthreads)
    dt = time.perf_counter() - t0
    return b.n_evals, dt, out


def reduce_over_ranks(torch, values, world, device):
    """Each timing's maximum over the ranks: the slowest replica sets the job's time."""
    t = torch.tensor(values, dtype=torch.float64, device=device)
    if world > 1:
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return t.tolist()


def job_throughput(evals_per_rank, steps, world, seconds):
    """Whole-job evaluations per second: every rank evaluates its own batch
    (independent replicas, no exchange), all within `seconds`."""
    return evals_per_rank * steps * world / seconds


def reference_arm(args, rank, world):
    from coffe_gb300 import workloads

    if rank != 0:
        return
    nthreads = os.cpu_count() or 1
    batch = workloads.cfg3(n_spectra=max(args.n_spectra, 1))
    # size each step's sample so that the whole run takes about 90 s of CPU time
    t1 = None
    for _ in range(max(args.warmup, 1)):
        t0 = time.perf_counter()
        cpu_eval(batch, 1, nthreads)
        t1 = time.perf_counter() - t0
    ns = int(max(1, min(batch.pk.shape[0], 90.0 / (max(args.steps, 1) * t1))))
    evals = 0
    total = 0.0
    for _ in range(args.steps):
        e, dt, _ = cpu_eval(batch, ns, nthreads)
        evals += e
        total += dt
    v = evals / total
    line = {
        "metric": METRIC, "value": v, "unit": UNIT, "impl": "reference",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * total / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded BBKS spectra)",
        "config": {"workload": "cfg3-batched: 512 spectra x 6 z x l=0,2,4, ragged 20-400 seps",
                   "sample_spectra_per_step": ns, "fft_n": N_FFT},
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": nthreads, "kind": "port",
                         "sample": f"{ns} of 512 spectra per step ({evals // args.steps} evals)"},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# --------------------------------------------------------------------- GPU
def rel_err_vs(ref, got, batch):
    """max |got - ref| / max(|ref|, 1e-3 max_r |ref|) per (request, l)"""
    floor = np.zeros_like(ref)
    offs = batch.req_offset
    for q in range(len(batch.req_spectrum)):
        lo, hi = int(offs[q]), int(offs[q + 1])
        if hi > lo:
            floor[lo:hi] = 1e-3 * np.abs(ref[lo:hi]).max(axis=0)
    return float(np.max(np.abs(got - ref) / np.maximum(np.abs(ref), np.maximum(floor, 1e-300))))


def kernel_rooflines(kt, n_spectra, n_terms, n_pairs, peaks):
    """Roofline entries of the step's kernels from their event-timed average
    launch (kt[precision][kernel] in ms): achieved = algorithmic work per launch
    / that time, against the measured peak of the resource that bounds it."""
    hbm = peaks["hbm_gbs"]
    rows = []

    def add(prec, name, label, bound, work, unit, peak, note):
        ms = kt.get(prec, {}).get(name)
        if not ms:
            return
        achieved = work / (ms * 1e-3) / (1e9 if unit == "GB/s" else 1e12)
        rows.append({"kernel": label, "precision": prec, "launch_ms": ms, "bound": bound,
                     "achieved": achieved, "peak": peak, "unit": unit, "frac": achieved / peak,
                     "work_per_launch": work, "note": note})

    inv = n_spectra * n_terms
    add("mixed", "fftlog_tables_fused_kernel", "fftlog_tables_fused_kernel (table stage)", "hbm",
        n_spectra * TABLE_BYTES_PER_SPECTRUM, "GB/s", hbm,
        "bytes: FP64 spectra in, float tables out; latency-bound (2 blocks per SM, long "
        "scoreboard on the per-grid tables), far from HBM")
    add("mixed", "fftlog_tables_fused_kernel", "fftlog_tables_fused_kernel (table stage)",
        "fp32", n_spectra * (FWD_FLOP + n_terms * INV_FLOP), "TFLOP/s", peaks["fp32"],
        "FP64-equivalent FLOP of the forward and inverse transforms against the FP32 peak "
        "(the forward is double-float, ~10-20 FP32 operations per FP64 one)")
    add("mixed", "mp_poly_kernel", "mp_poly_kernel<3,3,U,float>", "fp32",
        n_pairs * FLOP_PER_PAIR_POLY, "TFLOP/s", peaks["fp32"],
        "its own FLOP per launch / event time; peak = measured fma.rn.f32 rate")
    add("fp64-fastalg", "mp_poly_kernel", "mp_poly_kernel<3,3,U,double> (FP64, mixed algorithm)",
        "fp64", n_pairs * FLOP_PER_PAIR_POLY, "TFLOP/s", peaks["fp64"],
        "the mixed kernel's algorithm in FP64")
    add("mixed", "mp_fast_kernel", "mp_fast_kernel<3,3,U,float>", "fp32",
        n_pairs * (NODES * FLOP_PER_NODE + FLOP_PER_PAIR_EXTRA), "TFLOP/s", peaks["fp32"],
        "FLOP per launch / event time; peak = measured fma.rn.f32 rate")
    add("mixed", "fftlog_inverse_f32_kernel", "fftlog_inverse_f32_kernel (FP32 c2r)", "hbm",
        inv * INV_BYTES["mixed"], "GB/s", hbm,
        "bytes: half spectra in, float tables out; %.0f FLOP per transform, %.1f FLOP/B, "
        "below the FP32 ridge" % (INV_FLOP, INV_FLOP / INV_BYTES["mixed"]))
    add("mixed", "fftlog_forward_df_kernel", "fftlog_forward_df_kernel (double-float r2c)", "fp32",
        n_spectra * FWD_FLOP, "TFLOP/s", peaks["fp32"],
        "FP64-equivalent FLOP of the transform; each is ~10-20 FP32 operations in "
        "double-float, so frac counts FP64-class work against the FP32 peak")
    add("mixed", "cspline_band_kernel", "cspline_band_kernel (spline split + band)", "hbm",
        n_spectra * 20 * N_FFT, "GB/s", hbm, "bytes: P(k) in (8 B), hi/lo pairs (8 B) and "
        "float curvature (4 B) out per knot")
    add("fp64", "mp_lane_kernel", "mp_lane_kernel<3,double> (FP64 parity path)", "fp64",
        n_pairs * (NODES * FLOP_PER_NODE_LANE + FLOP_PER_PAIR_EXTRA), "TFLOP/s", peaks["fp64"],
        "~170 FLOP per node (reference algebra, spline records); peak = measured fma.rn.f64")
    add("fp64-fastalg", "mp_fast_kernel", "mp_fast_kernel<3,3,U,double> (FP64, mixed algorithm)",
        "fp64", n_pairs * (NODES * FLOP_PER_NODE_FP64_FASTALG + FLOP_PER_PAIR_EXTRA), "TFLOP/s",
        peaks["fp64"], "the mixed kernel's algorithm in FP64")
    add("fp64", "fftlog_inverse_kernel", "fftlog_inverse_kernel (FP64 c2r)", "fp64",
        inv * INV_FLOP, "TFLOP/s", peaks["fp64"], "FLOP per transform x transforms")
    add("fp64", "fftlog_forward_kernel", "fftlog_forward_kernel (FP64 r2c)", "fp64",
        n_spectra * FWD_FLOP, "TFLOP/s", peaks["fp64"], "FLOP per transform x transforms")
    return rows


def measure_gemm_peak(torch, dtype, n=8192, reps=5):
    a = torch.randn(n, n, device="cuda", dtype=dtype)
    b = torch.randn(n, n, device="cuda", dtype=dtype)
    torch.matmul(a, b)
    torch.cuda.synchronize()
    best = 0.0
    for _ in range(reps):
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record()
        torch.matmul(a, b)
        e.record()
        e.synchronize()
        best = max(best, 2 * n ** 3 / (s.elapsed_time(e) * 1e-3))
    del a, b
    return best / 1e12


def extras(torch, ctx, stream):
    """Device timings of the other workloads of the path (one GB300, CUDA events
    on the library's stream): den+RSD+lensing multipoles (128 mu x 256 x rule),
    the 2D-FFTLog multipole covariance, the multipole gradient and the divergent
    integral with its renormalisation grid."""
    from coffe_gb300 import workloads

    out = {}

    def ev_time(fn, reps):
        fn()
        torch.cuda.synchronize()
        best = None
        for _ in range(reps):
            s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            s.record(stream)
            fn()
            e.record(stream)
            e.synchronize()
            t = s.elapsed_time(e)
            best = t if best is None else min(best, t)
        return best

    # lensing: l = 0,2,4,6 at z = 1.5, 200 separations
    c4 = workloads.cfg4()
    co = c4["cosmo"]
    ctx.background_init(co.omega_m, co.omega_baryon, co.omega_gamma, co.h, 10000)
    dev = torch.device("cuda", torch.cuda.current_device())
    sep = torch.tensor(c4["sep"], device=dev)
    rs = torch.zeros(1, dtype=torch.int32, device=dev)
    rz = torch.tensor([c4["z_mean"]], dtype=torch.float64, device=dev)
    ro = torch.tensor([0, len(c4["sep"])], dtype=torch.int64, device=dev)
    res = {}
    for prec, reps in (("mixed", 3), ("fp64", 1), ("fp64-fastalg", 1)):
        ctx.integrals_init(c4["k"], c4["pk"][None, :], c4["terms"], N=N_FFT,
                           precision="mixed" if prec == "mixed" else "fp64", small_r=True)
        ctx.set_lensing_rule(*c4["rule"])
        o = torch.empty((len(c4["sep"]), 4), dtype=torch.float64, device=dev)
        ms = ev_time(lambda: ctx.multipoles_async(rs, rz, ro, sep, len(c4["sep"]), c4["ls"], o,
                                                  contrib=7, precision=prec), reps)
        ctx.synchronize()
        res[prec] = (ms, o.cpu().numpy())
    # the gradient of the same call with respect to P(k) and the bias / growth
    # scales (FP64 adjoint through the lensing integrands, tables and sub-Mpc
    # QAG entries; den/RSD on their first GK61 panel)
    pk4 = torch.tensor(c4["pk"][None, :], device=dev)
    ctx.integrals_init_device(c4["k"], pk4, c4["terms"], N=N_FFT, precision="fp64",
                              small_r=True)
    ov = torch.empty((len(c4["sep"]), 4), dtype=torch.float64, device=dev)
    G4, gpk4 = torch.ones_like(ov), torch.empty_like(pk4)
    gb4, gf4 = (torch.empty(1, dtype=torch.float64, device=dev) for _ in range(2))
    grad_fwd = ev_time(lambda: ctx.multipoles_scaled(rs, rz, ro, sep, len(c4["sep"]), c4["ls"],
                                                     ov, contrib=7), 1)
    grad_adj = ev_time(lambda: ctx.multipoles_adjoint(rs, rz, ro, sep, len(c4["sep"]), c4["ls"],
                                                      G4, gpk4, gb4, gf4, contrib=7), 1)
    ctx.synchronize()
    fl = 1e-3 * np.abs(res["fp64"][1]).max(0)
    fl[3] = 1e-3 * np.abs(res["fp64"][1]).max()  # l = 6: see the lensing tests
    err = float(np.max(np.abs(res["mixed"][1] - res["fp64"][1]) /
                       np.maximum(np.abs(res["fp64"][1]), fl)))
    n4 = len(c4["sep"]) * 4
    out["lensing_cfg4"] = {
        "workload": "den+RSD+lensing multipoles l=0,2,4,6, z=1.5, 200 separations 20-300 "
                    "Mpc/h, Gauss-Legendre 128 mu x 256 x (split), FFTLog N=4096",
        "mixed_ms": res["mixed"][0], "fp64_ms": res["fp64"][0],
        "fp64_fastalg_ms": res["fp64-fastalg"][0],
        "mixed_over_fp64": res["fp64"][0] / res["mixed"][0],
        "mixed_over_fp64_matched": res["fp64-fastalg"][0] / res["mixed"][0],
        "matched_note": "fp64_fastalg = the mixed path's algorithm (line-of-sight "
                        "polynomials, five combined plane records, fast den/RSD kernel) in FP64",
        "mixed_evals_per_s": n4 / (res["mixed"][0] * 1e-3),
        "fp64_evals_per_s": n4 / (res["fp64"][0] * 1e-3),
        "lensing_rule_nodes_per_s_mixed": len(c4["sep"]) * 128 * 256 * 256 / (res["mixed"][0] * 1e-3),
        "mu_nodes_evaluated": 64,
        "note": "equal tracers and even multipoles: the rule's 64 mu > 0 nodes are evaluated "
                "and counted twice (the terms are even in mu)",
        "max_rel_err_mixed_vs_fp64": err,
        "gradient": {"forward_ms": grad_fwd, "adjoint_ms": grad_adj,
                     "finite": bool(torch.isfinite(gpk4).all().item()),
                     "note": "d(multipoles)/d(P(k), bias scale, growth scale) of this call "
                             "(den+RSD first panel + lensing), FP64"},
        "max_rel_err_fp64_fastalg_vs_fp64": float(np.max(
            np.abs(res["fp64-fastalg"][1] - res["fp64"][1]) /
            np.maximum(np.abs(res["fp64"][1]), fl)))}
    # covariance: 5 z bins x l = 0,2,4 x 128 x 128 separations, 2D FFTLog 2^11
    ctx.background_init(co.omega_m, co.omega_baryon, co.omega_gamma, co.h, 10000)
    bg = ctx.background(with_H=False)
    c5 = workloads.cfg5(lambda z: np.interp(z, bg["z"], bg["chi"]))
    cov_call = lambda: ctx.covariance_multipoles(
        c5["k"], c5["pk"], c5["N"], c5["z_mean"], c5["deltaz"], c5["fsky"], c5["density"],
        c5["density"], c5["pixelsize"], c5["ls"], c5["sep"])
    cov_call()
    t0 = time.perf_counter()
    for _ in range(3):
        cov = cov_call()
    cov_ms = (time.perf_counter() - t0) / 3 * 1e3
    out["covariance_cfg5"] = {
        "workload": "multipole covariance l=0,2,4, 5 z bins of 1 (Gpc/h)^3, n=1e-3 (h/Mpc)^3, "
                    "128 x 128 separations 20-300 Mpc/h, 2D FFTLog 2^11 x 2^11, FP64",
        "ms_per_call": cov_ms, "outputs": int(cov.size),
        "note": "host API wall time (host arrays in, covariance out), 12 2D transforms"}
    # gradient of the config-1 multipoles with respect to P(k), bias and growth scales
    c1 = workloads.cfg1()
    ctx.background_init(co.omega_m, co.omega_baryon, co.omega_gamma, co.h, 10000)
    pk1 = torch.tensor(c1["pk"][None, :], device=dev)
    sep1 = torch.tensor(c1["sep"], device=dev)
    ro1 = torch.tensor([0, len(c1["sep"])], dtype=torch.int64, device=dev)
    rz1 = torch.tensor([1.0], dtype=torch.float64, device=dev)
    ctx.integrals_init_device(c1["k"], pk1, TERMS, N=N_FFT, precision="fp64")
    G = torch.ones((len(c1["sep"]), 3), dtype=torch.float64, device=dev)
    gpk = torch.empty_like(pk1)
    gb = torch.empty(1, dtype=torch.float64, device=dev)
    gf = torch.empty(1, dtype=torch.float64, device=dev)
    grad_ms = ev_time(lambda: ctx.multipoles_adjoint(rs, rz1, ro1, sep1, len(c1["sep"]),
                                                     (0, 2, 4), G, gpk, gb, gf), 3)
    out["gradient_cfg1"] = {
        "workload": "d(multipoles)/d(P(k), bias scale, growth scale), den+RSD l=0,2,4, z=1, "
                    "100 separations, 4096 k nodes, FP64 adjoint",
        "ms_per_call": grad_ms}
    out.update(config_baselines(torch, ctx, ev_time, out))
    # divergent I^4_0 and its 201 x 201 renormalisation grid (integrals.c:773-914)
    # on the config-1 spectrum, chi in [0, chi(1.2)]
    c1 = workloads.cfg1()
    ctx.background_init(0.31, 0.05, 9e-5, 0.67, 10000)
    bgd = ctx.background(with_H=False)
    chi = np.arange(201) * np.interp(1.2, bgd["z"], bgd["chi"]) / 200
    ctx.renormalization_grid(c1["k"], c1["pk"], chi[:4])
    t0 = time.perf_counter()
    grid = ctx.renormalization_grid(c1["k"], c1["pk"], chi)
    t1 = time.perf_counter()
    _, r1d, _ = ctx.divergent_integral(c1["k"], c1["pk"])
    t2 = time.perf_counter()
    out["divergent_i40"] = {
        "workload": "r^4 I^4_0 and its r = 0 renormalisation on the 297 fixed separations; "
                    "renormalisation grid 201 x 201 over chi in [0, chi(z=1.2)]; config-1 P(k), "
                    "GK61 QAG at 1e-5 per value, FP64",
        "grid_ms": (t1 - t0) * 1e3, "separations_ms": (t2 - t1) * 1e3,
        "grid_values_per_s": grid.size / (t1 - t0),
        "finite": bool(np.isfinite(grid).all() and np.isfinite(r1d).all()),
        "note": "host API wall time (host arrays in, values out)"}
    return out


def _pool_map(fn, items, nthreads):
    """fn over items on nthreads host threads (the oracle's ctypes calls release
    the GIL)."""
    from concurrent.futures import ThreadPoolExecutor

    with ThreadPoolExecutor(max_workers=nthreads) as ex:
        return list(ex.map(fn, items))


def _err_scale_floor(got, ref):
    """(max abs error / max |ref|, relative error with a floor of 1e-3 max |ref|)"""
    sc = np.abs(ref).max()
    d = np.abs(got - ref)
    return float(d.max() / sc), float(np.max(d / np.maximum(np.abs(ref), 1e-3 * sc)))


def config_baselines(torch, ctx, ev_time, extras_so_far):
    """The other configurations of the path, each with its GPU time, its error
    against the FP64 oracle and the oracle timed on the host cores (OpenMP or a
    thread pool over independent items, all cores): config 1 through the
    Coffe mirror (cold and warm), config 2's 30 tables at 2^14, a sample of
    config 4's separations, config 5's covariance."""
    import oracle as orc
    from coffe_gb300 import workloads
    from coffe_gb300.api import Coffe

    nth = os.cpu_count() or 1
    dev = torch.device("cuda", torch.cuda.current_device())
    res = {}
    # ---- config 1: plain FP64 den+RSD, 100 separations, one z, l = 0, 2, 4
    c1 = workloads.cfg1()
    co = c1["cosmo"]
    kw = dict(omega_m=co.omega_m, omega_baryon=co.omega_baryon, omega_gamma=co.omega_gamma,
              h=co.h, sep=c1["sep"], l=list(c1["ls"]), z_mean=[c1["z_mean"]], has_density=True,
              has_rsd=True, integrals_fftlog_sampling=N_FFT, deltaz=[0.1])
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    cc = Coffe(**kw)
    cc.set_power_spectrum_linear(c1["k"], c1["pk"])
    mp = cc.compute_multipoles_bulk()
    cold = time.perf_counter() - t0
    t0 = time.perf_counter()
    cc.set_power_spectrum_linear(c1["k"], c1["pk"] * 1.0)  # new spectrum: tables rebuilt
    mp = cc.compute_multipoles_bulk()
    warm = time.perf_counter() - t0
    got1 = np.array([m.value for m in mp]).reshape(len(c1["ls"]), len(c1["sep"]))
    t0 = time.perf_counter()
    bg = orc.background_nodes(co.omega_m, co.omega_baryon, co.omega_gamma, co.h, 10000)
    m = orc.Model(bg, co.h, co.omega_m)
    for n, l in TERMS:
        m.set_integral(n, l, *orc.integral_table(c1["k"], c1["pk"], n, l, N_FFT,
                                                 with_small_r=True))
    ref1 = np.array([m.multipoles_batch(3, np.full(len(c1["sep"]), c1["z_mean"]), c1["sep"],
                                        np.full(len(c1["sep"]), l), nthreads=nth)
                     for l in c1["ls"]])
    cpu1 = time.perf_counter() - t0
    del cc
    n1 = ref1.size
    res["config1"] = {
        "workload": "den+RSD multipoles l=0,2,4, z=1, 100 separations 10-200 Mpc/h, FP64, one "
                    "spectrum of 4096 k (Coffe.compute_multipoles_bulk: background, FFTLog tables "
                    "with the r=0 and sub-Mpc points, multipoles)",
        "gpu_cold_ms": cold * 1e3, "gpu_warm_ms": warm * 1e3,
        "gpu_warm_evals_per_s": n1 / warm,
        "cpu_ms": cpu1 * 1e3, "cpu_evals_per_s": n1 / cpu1, "cpu_cores": nth, "cpu_kind": "port",
        "max_rel_err_fp64_vs_oracle": _err_scale_floor(got1, ref1)[1],
        "note": "host API wall time; cold includes the context, the device background and the "
                "lazy module loads, warm rebuilds the tables for a new spectrum"}
    # ---- config 2: all 30 I_l^n at 2^14, resampled on 2^14 log-spaced r
    c2 = workloads.cfg2()
    k2, terms2, N2, r2 = c2["k"], c2["terms"], c2["N"], c2["r_out"]
    pk2 = torch.tensor(c2["pk"][None, :], device=dev)
    t0 = time.perf_counter()
    refs = _pool_map(lambda t: orc.integral_table(k2, c2["pk"], t[0], t[1], N2,
                                                  with_small_r=False), terms2, nth)
    cpu2 = time.perf_counter() - t0
    mask = (refs[0][0] >= 1.0 / co.h) & (refs[0][0] <= 1e4 / co.h)
    mask[:43] = False
    ref_r = [orc.spline_eval("akima", x[43:], y[43:], r2) for x, y in refs]
    res2 = {}
    for key, prec, df in (("fp64", "fp64", False), ("mixed", "mixed", False),
                          ("mixed_tables_df", "mixed", True)):
        ctx.integrals_init_device(k2, pk2, terms2, N=N2, precision=prec, sync=True, tables_df=df)
        ms = ev_time(lambda p=prec, d=df: ctx.integrals_init_device(
            k2, pk2, terms2, N=N2, precision=p, sync=False, tables_df=d), 5)
        ctx.synchronize()
        e_tab, e_res = (0.0, 0.0), (0.0, 0.0)
        t0 = time.perf_counter()
        vals = [ctx.integral_eval(0, n, l, r2) for n, l in terms2]
        rs_ms = (time.perf_counter() - t0) * 1e3
        for i, (n, l) in enumerate(terms2):
            y = ctx.integral_table(0, n, l)[1]
            e_tab = tuple(max(a, b) for a, b in
                          zip(e_tab, _err_scale_floor(y[mask], refs[i][1][mask])))
            e_res = tuple(max(a, b) for a, b in zip(e_res, _err_scale_floor(vals[i], ref_r[i])))
        res2[key] = {"tables_ms": ms, "resample_ms": rs_ms,
                     "table_err_abs_over_scale": e_tab[0], "table_err_rel_floor": e_tab[1],
                     "resampled_err_abs_over_scale": e_res[0], "resampled_err_rel_floor": e_res[1]}
    res["config2"] = {
        "workload": "30 tables I_l^n, l = 0..4, n = -1..4, BAO-modulated BBKS spectrum, FFTLog "
                    "N = 2^14; resampled by their Akima splines at 2^14 log-spaced r in "
                    "[1, 1e4] Mpc/h",
        "gpu": res2, "cpu_ms": cpu2 * 1e3, "cpu_cores": nth, "cpu_kind": "port",
        "error_convention": "worst over the 30 tables and r in [1, 1e4] Mpc/h against the FP64 "
                            "oracle: max abs error / the table's max |value|, and the relative "
                            "error with a floor of 1e-3 of that max",
        "note": "tables_ms: CUDA events on the library's stream, tables of all 30 terms; "
                "resample_ms: 30 host API calls (host r in, values out)"}
    # ---- config 4: a sample of its separations on the host
    c4 = workloads.cfg4()
    sample = c4["sep"][::25]  # 8 of the 200 separations
    bg4 = orc.background_nodes(co.omega_m, co.omega_baryon, co.omega_gamma, co.h, 10000)
    m4 = orc.Model(bg4, co.h, co.omega_m)
    for n, l in c4["terms"]:
        m4.set_integral(n, l, *orc.integral_table(c4["k"], c4["pk"], n, l, N_FFT,
                                                  with_small_r=True))
    t0 = time.perf_counter()
    lens = m4.multipoles_lensing(7, c4["z_mean"], sample, c4["ls"], *c4["rule"], nthreads=nth)
    nonint = np.array([m4.multipoles_batch(3, np.full(len(sample), c4["z_mean"]), sample,
                                           np.full(len(sample), l), nthreads=nth)
                       for l in c4["ls"]]).T
    cpu4 = time.perf_counter() - t0
    ref4 = lens + nonint
    ctx.background_init(co.omega_m, co.omega_baryon, co.omega_gamma, co.h, 10000)
    err4 = {}
    for prec in ("fp64", "mixed"):
        ctx.integrals_init(c4["k"], c4["pk"][None, :], c4["terms"], N=N_FFT, precision=prec,
                           small_r=True)
        ctx.set_lensing_rule(*c4["rule"])
        g4 = ctx.multipoles([0], [c4["z_mean"]], [0, len(sample)], sample, c4["ls"], contrib=7,
                            precision=prec)
        fl = 1e-3 * np.abs(ref4).max(axis=0)
        fl[3] = 1e-3 * np.abs(ref4).max()  # l = 6: a fraction of the whole output
        err4[prec] = float(np.max(np.abs(g4 - ref4) / np.maximum(np.abs(ref4), fl)))
    c4x = extras_so_far.get("lensing_cfg4", {})
    res["config4"] = {
        "workload": "den+RSD+lensing l=0,2,4,6, z=1.5, 128 mu x 256 x Gauss-Legendre rule; "
                    "host sample: 8 of the 200 separations",
        "cpu_ms": cpu4 * 1e3, "cpu_evals_per_s": sample.size * len(c4["ls"]) / cpu4,
        "cpu_cores": nth, "cpu_kind": "port",
        "gpu_mixed_evals_per_s": c4x.get("mixed_evals_per_s"),
        "gpu_fp64_evals_per_s": c4x.get("fp64_evals_per_s"),
        "max_rel_err_vs_oracle": err4,
        "error_convention": "relative, floor 1e-3 of each multipole's largest |value| (l = 6: "
                            "of the output's)"}
    # ---- config 5: covariance, all five bins, 128 x 128 separations, 2D FFTLog 2^11
    gbg = ctx.background(with_H=False)
    c5 = workloads.cfg5(lambda z: np.interp(z, gbg["z"], gbg["chi"]))
    ls5, sep5, N5 = c5["ls"], c5["sep"], c5["N"]
    nl, ns = len(ls5), len(sep5)
    t0 = time.perf_counter()
    jobs = [(p, i, j) for p in (1, 2) for i in range(nl) for j in range(i, nl)]
    blocks = _pool_map(lambda jb: orc.covariance_fftlog(c5["k"], c5["pk"], jb[0], ls5[jb[1]],
                                                        ls5[jb[2]], N5, sep5), jobs, nth)
    ipk = np.zeros((nl, nl, ns, ns))
    ipk2 = np.zeros_like(ipk)
    for (p, i, j), blk in zip(jobs, blocks):
        f = (2 * ls5[i] + 1) * (2 * ls5[j] + 1) / np.pi ** 2
        if p == 1:
            ipk[i, j] = blk * 2 * f
        else:
            ipk2[i, j] = blk * f
    for i in range(nl):
        for j in range(i):
            ipk[i, j] = ipk[j, i].T
            ipk2[i, j] = ipk2[j, i].T
    bg5 = orc.background_nodes(co.omega_m, co.omega_baryon, co.omega_gamma, co.h, 10000)
    ref5 = orc.Model(bg5, co.h, co.omega_m).covariance_multipoles(
        3, c5["z_mean"], c5["deltaz"], c5["fsky"], c5["density"], c5["pixelsize"], ls5, sep5,
        ipk, ipk2)
    cpu5 = time.perf_counter() - t0
    got5 = ctx.covariance_multipoles(c5["k"], c5["pk"], N5, c5["z_mean"], c5["deltaz"],
                                     c5["fsky"], c5["density"], c5["density"], c5["pixelsize"],
                                     ls5, sep5)
    g = np.moveaxis(got5, 3, 2)
    r = np.moveaxis(ref5, 3, 2)
    err5 = float(np.max(np.abs(g - r) / np.abs(r).max(axis=(-1, -2), keepdims=True)))
    res["config5"] = {
        "workload": "multipole covariance l=0,2,4, 5 z bins, 128 x 128 separations, 2D FFTLog "
                    "2^11 x 2^11 (12 transforms) + assembly, FP64",
        "gpu_ms": extras_so_far.get("covariance_cfg5", {}).get("ms_per_call"),
        "cpu_ms": cpu5 * 1e3, "cpu_cores": nth, "cpu_kind": "port",
        "max_err_vs_oracle_of_block_max": err5,
        "error_convention": "max |GPU - oracle| over each (z, l1, l2) block / the block's "
                            "largest |value|"}
    return res


def gradient_batch(torch, ctx, stream, batch, pk_d, rs_d, rz_d, ro_d, sep_d, n_sep):
    """The differentiable den+RSD multipoles of the whole batch (FP64 tables,
    first-panel values) and their reverse-mode derivative with respect to all
    512 spectra and every request's bias and growth scales: CUDA events on the
    library's stream, best of three."""
    dev = pk_d.device
    ctx.integrals_init_device(batch.k, pk_d, TERMS, N=N_FFT, precision="fp64", sync=True)
    out = torch.empty((n_sep, len(batch.ls)), dtype=torch.float64, device=dev)
    G = torch.ones_like(out)
    gpk = torch.empty_like(pk_d)
    nq = len(batch.req_spectrum)
    gb = torch.empty(nq, dtype=torch.float64, device=dev)
    gf = torch.empty_like(gb)

    def best(fn):
        fn()
        torch.cuda.synchronize()
        t = None
        for _ in range(3):
            s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            s.record(stream)
            fn()
            e.record(stream)
            e.synchronize()
            t = s.elapsed_time(e) if t is None else min(t, s.elapsed_time(e))
        return t

    fwd = best(lambda: ctx.multipoles_scaled(rs_d, rz_d, ro_d, sep_d, n_sep, batch.ls, out))
    rejected = ctx.last_retries()
    adj = best(lambda: ctx.multipoles_adjoint(rs_d, rz_d, ro_d, sep_d, n_sep, batch.ls, G, gpk,
                                              gb, gf))
    return {"workload": "d(multipoles)/d(P(k) of 512 spectra, bias and growth scale of 3072 "
                        "requests), den+RSD l=0,2,4, the config-3 batch (646,853 separations), "
                        "FP64 adjoint; forward = the differentiable first-panel values",
            "forward_ms": fwd, "adjoint_ms": adj, "outputs": n_sep * len(batch.ls),
            "first_panels_rejected": rejected,
            "finite": bool(torch.isfinite(gpk).all().item())}


def ours(args, rank, world, local_rank):
    import torch

    from coffe_gb300 import Context, workloads

    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    batch = workloads.cfg3(n_spectra=args.n_spectra, seed=workloads.CFG3_SEED + rank)
    c = batch.cosmo
    n_sep = len(batch.sep)
    n_evals = batch.n_evals
    ctx = Context(local_rank)
    # a dedicated (non-default) stream shared by our kernels and the CUDA events
    stream = torch.cuda.Stream(device=dev)
    torch.cuda.set_stream(stream)
    ctx.set_stream(stream.cuda_stream)
    ctx.background_init(c.omega_m, c.omega_baryon, c.omega_gamma, c.h, 10000)
    pk_d = torch.from_numpy(batch.pk).to(dev)
    rs_d = torch.from_numpy(batch.req_spectrum).to(dev)
    rz_d = torch.from_numpy(batch.req_z_mean).to(dev)
    ro_d = torch.from_numpy(batch.req_offset).to(dev)
    sep_d = torch.from_numpy(batch.sep).to(dev)
    outs = {p: torch.empty((n_sep, len(batch.ls)), dtype=torch.float64, device=dev)
            for p in PRECISIONS}
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)  # > 129 MB L2

    def evict_l2():
        """Evicts the previous step's tables and inputs from L2 (outside the
        timed events): a 256 MiB write, then a read of it, so that the lines
        left in L2 are clean and the next step neither finds its inputs there
        nor pays for writing the flush's dirty lines back to HBM."""
        flush.zero_()
        flush.view(torch.int32).max()

    def step(prec):
        # fp64-fastalg: FP64 tables, the mixed path's multipole algorithm in FP64
        tprec = "mixed" if prec == "mixed" else "fp64"
        ctx.integrals_init_device(batch.k, pk_d, TERMS, N=N_FFT, precision=tprec, sync=False)
        ctx.multipoles_async(rs_d, rz_d, ro_d, sep_d, n_sep, batch.ls, outs[prec], precision=prec)

    def barrier():
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    # launch shapes: the first build and multipole call of each shape time the
    # candidate configurations (benchmark mode), later calls and the captured
    # graph reuse the choice
    if args.launch_config:
        ctx.set_tuning(**{k: int(v) for k, v in
                          (kv.split("=") for kv in args.launch_config.split(","))})
    elif not args.no_autotune and not args.kernel_only:
        ctx.set_autotune(True)
    # build the per-grid tables once (synchronous), then warm up
    for prec in ("mixed", "fp64"):
        ctx.integrals_init_device(batch.k, pk_d, TERMS, N=N_FFT, precision=prec, sync=True)
    for _ in range(max(args.warmup, 0)):
        step("mixed")
    ctx.synchronize()

    # one step per precision captured once as a CUDA graph (tables, FFTs,
    # multipole quadrature and retries), replayed every timed step
    graphs = {}
    if not args.no_graph:
        for prec in PRECISIONS:
            try:
                step(prec)
                ctx.synchronize()
                g = torch.cuda.CUDAGraph()
                l0 = ctx.launch_count()
                with torch.cuda.graph(g, stream=stream):
                    step(prec)
                graphs[prec] = (g, ctx.launch_count() - l0)
            except Exception as exc:  # capture unsupported here: launch directly
                print(f"CUDA graph capture of the {prec} step failed ({exc}); launching directly",
                      file=sys.stderr)
                graphs.clear()
                break

    def timed(prec, k):
        starts = [torch.cuda.Event(enable_timing=True) for _ in range(k)]
        ends = [torch.cuda.Event(enable_timing=True) for _ in range(k)]
        barrier()
        l0 = ctx.launch_count()
        w0 = time.perf_counter()
        for i in range(k):
            evict_l2()
            starts[i].record(stream)
            if prec in graphs:
                graphs[prec][0].replay()
            else:
                step(prec)
            ends[i].record(stream)
        barrier()
        wall = time.perf_counter() - w0
        ctx.synchronize()
        dev_s = sum(s.elapsed_time(e) for s, e in zip(starts, ends)) * 1e-3
        launches = graphs[prec][1] * k if prec in graphs else ctx.launch_count() - l0
        return dev_s, wall, launches

    if args.kernel_only == "lensing-mixed":
        # profiling aid: the config-4 lensing multipoles on the first separations
        c4 = workloads.cfg4()
        co = c4["cosmo"]
        ctx.background_init(co.omega_m, co.omega_baryon, co.omega_gamma, co.h, 10000)
        ctx.integrals_init(c4["k"], c4["pk"][None, :], c4["terms"], N=N_FFT, precision="mixed",
                           small_r=True)
        ctx.set_lensing_rule(*c4["rule"])
        ns = max(1, min(args.lensing_seps, len(c4["sep"])))
        dev = torch.device("cuda", torch.cuda.current_device())
        sep = torch.tensor(c4["sep"][:ns], device=dev)
        rs = torch.zeros(1, dtype=torch.int32, device=dev)
        rz = torch.tensor([c4["z_mean"]], dtype=torch.float64, device=dev)
        ro = torch.tensor([0, ns], dtype=torch.int64, device=dev)
        o = torch.empty((ns, len(c4["ls"])), dtype=torch.float64, device=dev)
        for _ in range(args.steps):
            ctx.multipoles_async(rs, rz, ro, sep, ns, c4["ls"], o, contrib=7, precision="mixed")
        ctx.synchronize()
        return
    if args.kernel_only:
        # profiling aid: only one stage of one precision
        prec = args.kernel_only.split("-")[-1]
        ctx.integrals_init_device(batch.k, pk_d, TERMS, N=N_FFT, precision=prec, sync=True)
        for _ in range(args.steps):
            if args.kernel_only.startswith("tables"):
                ctx.integrals_init_device(batch.k, pk_d, TERMS, N=N_FFT, precision=prec, sync=False)
            else:
                ctx.multipoles_async(rs_d, rz_d, ro_d, sep_d, n_sep, batch.ls, outs[prec],
                                     precision=prec)
        ctx.synchronize()
        return

    with ClockSampler(local_rank, enabled=not args.no_clocks and rank == 0) as clk:
        dev_mixed, wall_mixed, launches = timed("mixed", args.steps)
    clocks = clk.summary()
    tuning = ctx.tuning()
    k64 = args.fp64_steps or max(3, args.steps // 50)
    for _ in range(2):
        step("fp64")
        step("fp64-fastalg")
    ctx.synchronize()
    dev_fp64, wall_fp64, _ = timed("fp64", k64)
    dev_fast64, _, _ = timed("fp64-fastalg", k64)

    # accuracy of the mixed path against the FP64 path on the full batch (the
    # FP64 path itself matches the CPU oracle to 1e-10 in the parity tests);
    # the replayed graph must give the direct launch's output bit for bit
    graph_equal = None
    if "mixed" in graphs:
        graphs["mixed"][0].replay()
        ctx.synchronize()
        replayed = outs["mixed"].clone()
    step("mixed")
    retries = {"mixed": ctx.last_retries()}
    if "mixed" in graphs:
        ctx.synchronize()
        graph_equal = bool(torch.equal(replayed, outs["mixed"]))
    step("fp64")
    retries["fp64"] = ctx.last_retries()
    step("fp64-fastalg")
    retries["fp64-fastalg"] = ctx.last_retries()
    ctx.synchronize()
    ref64 = outs["fp64"].cpu().numpy()
    err = rel_err_vs(ref64, outs["mixed"].cpu().numpy(), batch)
    err_fast64 = rel_err_vs(ref64, outs["fp64-fastalg"].cpu().numpy(), batch)

    # per-kernel device times (CUDA events after every launch, direct launches)
    kt = {}
    for prec, reps in (("mixed", 10), ("fp64", 2), ("fp64-fastalg", 2)):
        ctx.set_kernel_timing(True)
        ctx.kernel_times(reset=True)
        for _ in range(reps):
            evict_l2()
            step(prec)
        kt[prec] = {name: ms / n for name, (n, ms) in ctx.kernel_times(reset=True).items()}
        ctx.set_kernel_timing(False)

    # dominant kernel: the mixed multipole kernel alone, CUDA events on our stream
    ctx.integrals_init_device(batch.k, pk_d, TERMS, N=N_FFT, precision="mixed", sync=True)
    nk_rep = 20
    s_ev, e_ev = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    barrier()
    s_ev.record(stream)
    for _ in range(nk_rep):
        ctx.multipoles_async(rs_d, rz_d, ro_d, sep_d, n_sep, batch.ls, outs["mixed"],
                             precision="mixed")
    e_ev.record(stream)
    e_ev.synchronize()
    kern_s = s_ev.elapsed_time(e_ev) * 1e-3 / nk_rep
    poly = bool(ctx.tuning().get("lane_poly"))
    flop_launch = n_sep * (FLOP_PER_PAIR_POLY if poly else
                           NODES * FLOP_PER_NODE + FLOP_PER_PAIR_EXTRA)

    # end to end through the public API with pinned host buffers
    e2e = None
    if not args.no_e2e:
        pin = lambda a: torch.from_numpy(np.ascontiguousarray(a)).pin_memory().numpy()
        h_pk, h_rs, h_rz = pin(batch.pk), pin(batch.req_spectrum), pin(batch.req_z_mean)
        h_ro, h_sep = pin(batch.req_offset), pin(batch.sep)
        h_out = pin(np.zeros((len(batch.sep), len(batch.ls))))
        ctx.set_stream(None)
        ctx.integrals_init(batch.k, h_pk, TERMS, N=N_FFT, precision="mixed", small_r=False)
        ctx.multipoles(h_rs, h_rz, h_ro, h_sep, batch.ls, precision="mixed", out=h_out)
        ke = max(3, min(args.steps, 20))
        barrier()
        t0 = time.perf_counter()
        for _ in range(ke):
            # the tables are enqueued (the call returns once P(k) is on the device) and
            # the multipole call uploads its requests while they are being made; it
            # returns when the results are in h_out and reports any device error
            ctx.integrals_init(batch.k, h_pk, TERMS, N=N_FFT, precision="mixed", small_r=False,
                               sync=False)
            res = ctx.multipoles(h_rs, h_rz, h_ro, h_sep, batch.ls, precision="mixed", out=h_out)
        barrier()
        te = time.perf_counter() - t0
        h2d = h_pk.nbytes + h_rs.nbytes + h_rz.nbytes + h_ro.nbytes + h_sep.nbytes
        e2e = {"value": n_evals * ke / te, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
               "d2h_bytes_per_step": int(res.nbytes), "steps": ke,
               "ms_per_step": 1e3 * te / ke}
        ctx.set_stream(stream.cuda_stream)

    # reduce over ranks (max time)
    dev_mixed, dev_fp64, dev_fast64, kern_s = reduce_over_ranks(
        torch, [dev_mixed, dev_fp64, dev_fast64, kern_s], world, dev)
    if e2e is not None and world > 1:
        (ms,) = reduce_over_ranks(torch, [e2e["ms_per_step"]], world, dev)
        e2e["ms_per_step"] = ms
        e2e["value"] = job_throughput(n_evals, 1, world, ms * 1e-3)
    if rank != 0:
        ctx.close()
        return

    value = job_throughput(n_evals, args.steps, world, dev_mixed)
    fp64_value = job_throughput(n_evals, k64, world, dev_fp64)
    fast64_value = job_throughput(n_evals, k64, world, dev_fast64)
    sgemm = measure_gemm_peak(torch, torch.float32)
    peak32 = ctx.measure_peak("fp32") / 1e12
    peak64 = ctx.measure_peak("fp64") / 1e12
    peak32x2 = ctx.measure_peak("fp32x2") / 1e12
    achieved = flop_launch / kern_s / 1e12
    peaks = {}
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            peaks = json.load(fh)
    except OSError:
        pass
    cpu = None
    if not args.no_cpu:
        nthreads = os.cpu_count() or 1
        ce, cdt, cout = cpu_eval(batch, args.cpu_spectra, nthreads)
        sub_err = rel_err_vs(cout, outs["fp64"].cpu().numpy()[: cout.shape[0]],
                             workloads.subset(batch, args.cpu_spectra))
        cpu = {"value": ce / cdt, "unit": UNIT, "cores": nthreads, "kind": "port",
               "sample": f"first {args.cpu_spectra} of {args.n_spectra} spectra, all their "
                         f"requests ({ce} evals, {cdt:.1f} s)",
               "gpu_fp64_vs_cpu_max_rel_err": sub_err}
    extra = None
    if not args.no_extras:
        extra = extras(torch, ctx, stream)
        extra["gradient_cfg3"] = gradient_batch(torch, ctx, stream, batch, pk_d, rs_d, rz_d,
                                                ro_d, sep_d, n_sep)
    # the dominant kernel of the step: the table stage (the fused kernel when the
    # tuner picks it), against HBM with its algorithmic bytes
    hbm = peaks.get("hbm_gbs") or 6755.5
    t_ms = kt.get("mixed", {}).get("fftlog_tables_fused_kernel")
    table_roofline = None
    if t_ms:
        tb = args.n_spectra * TABLE_BYTES_PER_SPECTRUM
        table_roofline = {
            "kernel": "fftlog_tables_fused_kernel (spline band, double-float forward and FP32 "
                      "inverse transforms of one spectrum per block)",
            "bound": "hbm", "achieved": tb / (t_ms * 1e-3) / 1e9, "peak": hbm, "unit": "GB/s",
            "frac": tb / (t_ms * 1e-3) / 1e9 / hbm, "launch_ms": t_ms,
            "bytes_per_launch": tb,
            "traffic": TABLE_DRAM_BYTES_PER_LAUNCH * args.n_spectra / 512,
            "traffic_unit": "bytes per launch (ncu dram read+write of the 512-spectrum batch)",
            "peak_source": "MEASURED_PEAKS.json hbm_gbs (copy bandwidth)",
            "note": "latency-bound: 2 blocks per SM, long-scoreboard stalls on per-grid tables"}
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * dev_mixed / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64",
        "data": "synthetic (seeded BBKS spectra, seed 20261203 + rank)",
        "config": {"workload": "cfg3-batched: 512 spectra x 6 z_mean x l=0,2,4, ragged 20-400 "
                               "separations in [5,250] Mpc/h, FFTLog N=4096",
                   "n_spectra": args.n_spectra, "requests": len(batch.req_spectrum),
                   "separations": n_sep, "evals_per_step": n_evals,
                   "l2": "flushed between timed steps outside the events: 256 MiB write, then a read "
                         "of it (the step starts with clean, cold L2 lines)",
                   "cuda_graph": bool(graphs), "graph_output_equals_direct": graph_equal,
                   "launch_config": tuning,
                   "autotuned": not (args.no_autotune or args.launch_config),
                   "parallelism": f"replicas x{world}"},
        "fp64": {"value": fp64_value, "unit": UNIT, "steps": k64,
                 "ms_per_step": 1e3 * dev_fp64 / k64,
                 "algorithm": "reference algebra per node (the 1e-10 parity path)"},
        "fp64_fastalg": {"value": fast64_value, "unit": UNIT, "steps": k64,
                         "ms_per_step": 1e3 * dev_fast64 / k64,
                         "algorithm": "the mixed path's algorithm in FP64 (FP64 tables and "
                                      "transforms; per-request background polynomials, the "
                                      "integrand as a polynomial in mu^2 when the tuner "
                                      "picks it for both)",
                         "max_rel_err_vs_fp64": err_fast64},
        "mixed_over_fp64": value / fast64_value,
        "mixed_over_fp64_note": "matched algorithms: the mixed step against the same "
                                "algorithms in FP64 (fp64_fastalg); against the parity "
                                "path's reference algebra see mixed_over_fp64_parity_path",
        "mixed_over_fp64_parity_path": value / fp64_value,
        "max_rel_err_mixed_vs_fp64": err,
        "adaptive_retries": retries,
        "gpu_launches": int(launches),
        "measured_peaks": {"fp32_fma_tflops": peak32, "fp32x2_fma_tflops": peak32x2,
                           "fp64_fma_tflops": peak64, "sgemm_tflops": sgemm,
                           "hbm_gbs": peaks.get("hbm_gbs"),
                           "source": "FMA-chain kernels of coffe_gpu_measure_peak and cuBLAS "
                                     "SGEMM 8192^3 (TF32 off) in this run; HBM from "
                                     "MEASURED_PEAKS.json"},
        "roofline": table_roofline,
        "roofline_multipoles": {
            "kernel": ("mp_poly_kernel<3, 3>" if poly else "mp_fast_kernel<3, 3>") +
                      " (mixed multipole quadrature, unit biases; the multipole call: "
                      "background fit included)",
            "bound": "fp32", "achieved": achieved,
            "peak": peak32, "unit": "TFLOP/s", "frac": achieved / peak32,
            "peak_source": "measured fma.rn.f32 rate of this GPU in this run "
                           "(coffe_gpu_measure_peak); FP32-issue bound, neither HBM nor tensor",
            "flop_per_launch": flop_launch, "launch_ms": kern_s * 1e3},
        "rooflines": kernel_rooflines(kt, args.n_spectra, len(TERMS), n_sep,
                                      {"fp32": peak32, "fp64": peak64,
                                       "hbm_gbs": peaks.get("hbm_gbs") or 6755.5}),
        "kernel_ms": kt,
        "clocks": clocks,
        "e2e": e2e,
        "cpu_baseline": cpu,
        "extras": extra,
    }
    print(json.dumps(line), flush=True)
    ctx.close()


def main():
    args = parse()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        reference_arm(args, rank, world)
        return
    import torch

    torch.backends.cuda.matmul.allow_tf32 = False
    if world > 1:
        torch.cuda.set_device(local_rank)
        torch.distributed.init_process_group("nccl")
    try:
        ours(args, rank, world, local_rank)
    finally:
        if world > 1:
            torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
