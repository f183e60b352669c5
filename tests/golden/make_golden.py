"""Extract the golden vectors the oracle is pinned to from the reference's own
test fixtures (tests/benchmarks/*.dat and PkL_CLASS.dat of JCGoran/coffe).

Run once where the reference tree is available:
    python tests/golden/make_golden.py /path/to/coffe
It writes golden.npz next to this script.  The integral tables (10001 rows
each) are thinned to the rows the reference's Python test checks
(1.5 < r < 20000 Mpc, tests/test_coffe.py:196-233), every 8th row; all other
files are copied whole except the background (every 4th of its 10001 rows) and
the renormalisation grid of the divergent integral (every 10th chi node).  The values are the reference's published outputs,
not recomputed.
"""
import sys
from pathlib import Path

import numpy as np

H = 0.67
COFFE_H0 = 1.0 / 2997.92458


def main(ref: Path):
    bench = ref / "tests" / "benchmarks"
    out = {}
    out["pk_class"] = np.loadtxt(ref / "PkL_CLASS.dat")
    out["background"] = np.loadtxt(bench / "benchmark_background.dat")[::4]
    for i in range(8):
        d = np.loadtxt(bench / f"benchmark_integral{i}.dat")
        r = d[:, 0] / (COFFE_H0 * H)
        keep = np.where((r > 1.5) & (r < 20000))[0][::8]
        out[f"integral{i}"] = d[keep]
        with open(bench / f"benchmark_integral{i}.dat") as fh:
            out[f"integral{i}_header"] = np.array(fh.readline().strip())
    for name in ("den", "rsd", "std", "len", "std_len", "flatsky_lensing_lensing",
                 "flatsky_density_lensing"):
        for l in (0, 2, 4):
            out[f"{name}_multipoles{l}"] = np.loadtxt(bench / f"benchmark_{name}_multipoles{l}.dat")
    # redshift-averaged den+rsd multipoles, z in [0.9, 1.1]
    for l in (0, 2, 4):
        out[f"avg_multipoles{l}"] = np.loadtxt(bench / f"benchmark_avg_multipoles{l}.dat")
    # correlation function at z = 1, mu = 0, 0.2, 0.5, 0.8, 0.95 (index 0..4)
    for name in ("den", "rsd", "std", "len", "std_len"):
        for i in range(5):
            out[f"{name}_corrfunc{i}"] = np.loadtxt(bench / f"benchmark_{name}_corrfunc{i}.dat")
    for a in (0, 2, 4):
        for b in (0, 2, 4):
            out[f"multipoles_covariance_{a}{b}"] = np.loadtxt(
                bench / f"benchmark_multipoles_covariance_{a}{b}.dat")
            out[f"avg_multipoles_covariance_{a}{b}"] = np.loadtxt(
                bench / f"benchmark_avg_multipoles_covariance_{a}{b}.dat")
    # the divergent I^4_0 (every row) and its renormalisation grid (every 10th
    # of the 201 chi nodes in each direction: 21 x 21 of its 40401 rows)
    out["integral8"] = np.loadtxt(bench / "benchmark_integral8.dat")
    ren = np.loadtxt(bench / "benchmark_integral8_renormalization.dat").reshape(201, 201, 3)
    out["integral8_renormalization"] = ren[::10, ::10].reshape(-1, 3)
    dst = Path(__file__).resolve().parent / "golden.npz"
    np.savez_compressed(dst, **out)
    print(dst, dst.stat().st_size, "bytes")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py <path of the reference tree>")
    main(Path(sys.argv[1]))
