"""Shared fixtures.  Tests marked ``gpu`` need a CUDA device; everything else
runs on the CPU (the oracle against the reference's golden vectors, host logic,
and the C ABI library's symbol table)."""
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

H = 0.67
COFFE_H0 = 1.0 / 2997.92458


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def golden():
    return dict(np.load(ROOT / "tests" / "golden" / "golden.npz"))


@pytest.fixture(scope="session")
def oracle():
    import oracle as orc

    orc.build()
    return orc


@pytest.fixture(scope="session")
def class_pk(golden):
    """The reference's default linear spectrum (PkL_CLASS.dat) in 1/Mpc, Mpc^3."""
    k, pk = golden["pk_class"].T
    return k * H, pk / H ** 3


@pytest.fixture(scope="session")
def ref_bg(oracle):
    """Oracle background at the reference's default cosmology."""
    return oracle.background_nodes(0.3, 0.05, 9e-5, H, 10000)


@pytest.fixture(scope="session")
def gpu_ctx():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from coffe_gb300.api import Context

    ctx = Context(0)
    yield ctx
    ctx.close()
