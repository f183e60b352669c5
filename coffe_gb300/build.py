"""Build the CUDA library ``coffe_gb300/_build/libcoffe_gpu.so`` for sm_103a.

Each ``csrc/*.cu`` is compiled by nvcc in parallel, then linked into one shared
library with a static CUDA runtime; the C ABI is ``include/coffe_gpu.h``.
Usage: ``python -m coffe_gb300.build`` (or ``build()`` from Python).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
OUT_DIR = PKG / "_build"
LIB = OUT_DIR / "libcoffe_gpu.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr"]


def _nvcc() -> str:
    p = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(p).exists():
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build coffe_gb300")
    return p


def _sources():
    return sorted(CSRC.glob("*.cu"))


def _deps():
    return sorted(CSRC.glob("*.cuh")) + sorted(CSRC.glob("*.h")) + [PKG.parent / "include" / "coffe_gpu.h"]


def _stale(obj: Path, src: Path) -> bool:
    if not obj.exists():
        return True
    t = obj.stat().st_mtime
    return src.stat().st_mtime > t or any(d.stat().st_mtime > t for d in _deps())


def build(force: bool = False, verbose: bool = False, ptxas_info: bool = False) -> Path:
    OUT_DIR.mkdir(exist_ok=True)
    nvcc = _nvcc()
    srcs = _sources()
    objs = [OUT_DIR / (s.stem + ".o") for s in srcs]
    todo = [(s, o) for s, o in zip(srcs, objs) if force or ptxas_info or _stale(o, s)]

    def compile_one(so):
        s, o = so
        cmd = [nvcc, *ARCH, *NVCC_FLAGS, "-c", str(s), "-o", str(o)]
        if ptxas_info:
            cmd.insert(1, "-Xptxas=-v")
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {s.name}:\n{r.stdout}\n{r.stderr}")
        return s.name, r.stdout + r.stderr

    if todo:
        with cf.ThreadPoolExecutor(max_workers=min(len(todo), os.cpu_count() or 4)) as ex:
            for name, log in ex.map(compile_one, todo):
                if verbose or ptxas_info:
                    print(f"[nvcc] {name}\n{log}")
    if force or todo or not LIB.exists():
        cmd = [nvcc, *ARCH, "-shared", "-o", str(LIB), *map(str, objs), "-cudart", "static"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    return LIB


if __name__ == "__main__":
    import sys

    print(build(force="--force" in sys.argv, verbose=True, ptxas_info="--ptxas" in sys.argv))
