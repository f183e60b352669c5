"""The C ABI library builds for sm_103a, loads without a GPU, and exports every
function include/coffe_gpu.h declares; creating a context without a GPU fails
with a status code instead of crashing (no CPU fallback exists)."""
import ctypes
import re
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def declared_functions():
    src = (ROOT / "include" / "coffe_gpu.h").read_text()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    names = re.findall(r"\b(coffe_gpu_[a-z0-9_]+)\s*\(", src)
    return sorted(set(names))


@pytest.fixture(scope="module")
def libpath():
    from coffe_gb300 import build

    return build.build()


def test_header_declares_the_python_binding():
    from coffe_gb300 import _lib

    assert sorted(_lib.EXPORTS) == declared_functions()


def test_library_exports_every_declared_symbol(libpath):
    out = subprocess.run(["nm", "-D", "--defined-only", str(libpath)], capture_output=True,
                         text=True, check=True).stdout
    exported = set(re.findall(r"\bT (coffe_gpu_[a-z0-9_]+)", out))
    missing = set(declared_functions()) - exported
    assert not missing, missing


def test_build_targets_sm103a_only():
    from coffe_gb300 import build

    assert build.ARCH == ["-gencode", "arch=compute_103a,code=sm_103a"]


def test_library_loads_and_reports_errors_without_gpu(libpath):
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present; covered by the gpu tests")
    from coffe_gb300 import _lib

    L = _lib.load()
    assert L.coffe_gpu_strerror(-1) == b"invalid argument"
    assert L.coffe_gpu_integral_table_len(4096) == 4096 + 43
    ctx = ctypes.c_void_p()
    st = L.coffe_gpu_ctx_create(0, ctypes.byref(ctx))
    assert st == -2 and not ctx.value  # COFFE_GPU_ECUDA, no context, no fallback
    assert L.coffe_gpu_ctx_destroy(None) == 0


def test_divergent_separations_equal_the_oracle(libpath, oracle):
    """The library's copy of the reference's fixed separations of I^4_0
    (integrals.c:76-103) is the oracle's, value for value (a host-only call)."""
    import numpy as np

    from coffe_gb300 import divergent_separations

    got = divergent_separations()
    assert len(got) == 297 and np.array_equal(got, oracle.divergent_separations())
