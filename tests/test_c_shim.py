"""The C drop-in drivers (coffe_gb300/shim/coffe_gpu_shim.c) compiled as C99 by the
system C compiler against include/coffe_gpu.h and stand-ins of the reference's
headers (tests/c/standin), linked to libcoffe_gpu.so, and run through the
sequence a reference C caller runs (src/main.c:138-151): a caller-built
background, coffe_integrals_init_gpu, coffe_multipoles_init_gpu, the
(z_mean, l, sep) output order of multipoles.c:76-86.

CPU tests: the public header and the shim compile as strict C99, and the
program rejects a non-power-of-two bessel_bins before touching a device.
GPU tests: tables and multipoles against the oracle (FP64 1e-10 relative with
the parity floors of test_gpu_parity; mixed 1e-4).
"""
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

from conftest import H, ROOT

CC = shutil.which("cc") or shutil.which("gcc")
LIBDIR = ROOT / "coffe_gb300" / "_build"
SRCS = [ROOT / "coffe_gb300" / "shim" / "coffe_gpu_shim.c", ROOT / "tests" / "c" / "standin" / "standin.c",
        ROOT / "tests" / "c" / "shim_test.c"]
CFLAGS = ["-std=c99", "-pedantic", "-Wall", "-Wextra", "-Werror", "-O2",
          f"-I{ROOT / 'include'}", f"-I{ROOT / 'coffe_gb300' / 'shim'}",
          f"-I{ROOT / 'tests' / 'c' / 'standin'}"]

pytestmark = pytest.mark.skipif(CC is None, reason="no C compiler")


def _compile(tmp: Path) -> Path:
    if not (LIBDIR / "libcoffe_gpu.so").exists():
        from coffe_gb300 import build

        build.build()
    exe = tmp / "shim_test"
    cmd = [CC, *CFLAGS, *map(str, SRCS), "-o", str(exe), f"-L{LIBDIR}", "-lcoffe_gpu",
           f"-Wl,-rpath,{LIBDIR}", "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    return exe


def _write_input(path: Path, k, pk, bg, z_mean, ls, sep, bessel_bins, contrib, precision,
                 omega_cdm=0.26, omega_b=0.05, epsrel=1e-5):
    hdr = np.array([len(k), len(bg["z"]), len(z_mean), len(ls), len(sep), bessel_bins, contrib,
                    precision], dtype=np.int64)
    body = np.concatenate([k, pk, bg["z"], bg["chi"], bg["D1"], bg["f"], bg["a"], bg["confH"],
                           np.asarray(z_mean, float), np.asarray(ls, float), sep,
                           [omega_cdm, omega_b, H, epsrel]]).astype(np.float64)
    with open(path, "wb") as f:
        f.write(hdr.tobytes())
        f.write(body.tobytes())


def _read_output(path: Path):
    raw = path.read_bytes()
    pos = 0

    def i64():
        nonlocal pos
        v = int(np.frombuffer(raw, np.int64, 1, pos)[0])
        pos += 8
        return v

    def f64(n):
        nonlocal pos
        v = np.frombuffer(raw, np.float64, n, pos).copy()
        pos += 8 * n
        return v

    tables = []
    for _ in range(i64()):
        n, l, m = i64(), i64(), i64()
        tables.append((n, l, f64(m), f64(m)))
    nmp = i64()
    mp = f64(4 * nmp).reshape(nmp, 4)
    return tables, mp


def test_header_compiles_as_c99(tmp_path):
    src = tmp_path / "h.c"
    src.write_text('#include "coffe_gpu.h"\nint main(void) { coffe_gpu_ctx_t *c = 0; '
                   'return c == 0 ? COFFE_GPU_OK : COFFE_GPU_EINVAL; }\n')
    r = subprocess.run([CC, *CFLAGS, "-c", str(src), "-o", str(tmp_path / "h.o")],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_shim_builds_and_rejects_bad_bessel_bins(tmp_path, oracle):
    """Compiles and links the drop-in; the size check fails before any device use."""
    from coffe_gb300 import workloads

    exe = _compile(tmp_path)
    c = workloads.cfg1()
    bg = oracle.background_nodes(0.31, 0.05, 9e-5, H, 64)
    inp = tmp_path / "in.bin"
    _write_input(inp, c["k"], c["pk"], bg, [1.0], (0, 2, 4), c["sep"][:4], 1000, 3, 0)
    r = subprocess.run([str(exe), str(inp), str(tmp_path / "out.bin")], capture_output=True,
                       text=True, timeout=60)
    assert r.returncode == 1
    assert "power of two" in r.stderr
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60)
    assert r.returncode == 2


def _table_err(gy, oy, mask, floor):
    a = np.nan_to_num(np.abs(oy), nan=0.0)
    env = np.array([a[max(0, i - 64): i + 65].max() for i in range(len(a))])
    return np.max((np.abs(gy - oy) / np.maximum(np.abs(oy), floor * env))[mask])


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [0, 1])
def test_shim_sequence_matches_oracle(tmp_path, oracle, precision):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from coffe_gb300 import workloads

    exe = _compile(tmp_path)
    c = workloads.cfg1()
    k, pk, sep = c["k"], c["pk"], c["sep"]
    bg = oracle.background_nodes(0.31, 0.05, 9e-5, H, 10000)
    z_mean, ls, N = [1.0, 1.5], (0, 2, 4), 4096
    inp, outp = tmp_path / "in.bin", tmp_path / "out.bin"
    _write_input(inp, k, pk, bg, z_mean, ls, sep, N, 3, precision)
    r = subprocess.run([str(exe), str(inp), str(outp)], capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stderr
    tables, mp = _read_output(outp)

    # the integral array: the three den/RSD tables, r = 0 and sub-Mpc entries included
    assert [(n, l) for n, l, _, _ in tables] == [(0, 0), (0, 2), (0, 4)]
    model = oracle.Model(bg, H, 0.31)
    for n, l, gx, gy in tables:
        ox, oy = oracle.integral_table(k, pk, n, l, N, with_small_r=True)
        model.set_integral(n, l, ox, oy)
        assert np.max(np.abs(gx - ox) / ox.clip(1e-300)) < 1e-14
        mask = np.zeros(len(ox), bool)
        mask[43:] = True
        if precision == 0:
            assert _table_err(gy, oy, mask & (ox >= 1.0) & (ox <= 1e4), 1e-8) < 1e-10, (n, l)
            assert np.max(np.abs(gy[:43] - oy[:43]) / np.maximum(np.abs(oy[:43]),
                                                             1e-8 * np.abs(oy[:43]).max())) < 1e-9
        else:  # FP32 inverse transforms: the criterion of the mixed table tests
            m = mask & (ox >= 5 / H) & (ox <= 300 / H)
            e = np.max(np.abs(gy[m] - oy[m]) / np.maximum(np.abs(oy[m]),
                                                          1e-3 * np.abs(oy[m]).max()))
            assert e < 1e-5, (n, l, e)

    # the multipole array in the reference's (z_mean, l, sep) order
    assert mp.shape == (len(z_mean) * len(ls) * len(sep), 4)
    zz, ll, ss = np.meshgrid(z_mean, ls, sep, indexing="ij")
    assert np.array_equal(mp[:, 0], zz.ravel())
    assert np.array_equal(mp[:, 1], ll.ravel())
    assert np.array_equal(mp[:, 2], ss.ravel())
    got = mp[:, 3].reshape(len(z_mean), len(ls), len(sep))
    tol = 1e-10 if precision == 0 else 1e-4
    for i, z in enumerate(z_mean):
        for j, l in enumerate(ls):
            ref = model.multipoles_batch(3, np.full(len(sep), z), sep, np.full(len(sep), l))
            e = np.max(np.abs(got[i, j] - ref) / np.maximum(np.abs(ref), 1e-3 * np.abs(ref).max()))
            assert e < tol, (z, l, e)
