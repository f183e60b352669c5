"""GB300-native (sm_103a) implementation of COFFE's correlation-function hot path.

The compute path is the CUDA library ``_build/libcoffe_gpu.so`` behind the C ABI
of ``include/coffe_gpu.h``; this package is its Python host side:

* :class:`Context` -- one device context (background, FFTLog tables, batched
  multipoles) mirroring the C entry points;
* :class:`Coffe` -- a mirror of the reference's ``coffe.Coffe`` for this path;
* :mod:`workloads` -- seeded synthetic inputs of the benchmark configurations.

There is no CPU fallback: without the library or a CUDA device the calls raise.
"""
from .api import (DEFAULT_TERMS, DEN_RSD_TERMS, AverageCovariance, AverageMultipoles,  # noqa: F401
                  Coffe, Context, Corrfunc, Covariance, Multipoles, divergent_separations)
from ._lib import CoffeGpuError  # noqa: F401

__all__ = ["AverageCovariance", "AverageMultipoles", "Coffe", "Covariance", "Context", "Corrfunc", "Multipoles", "CoffeGpuError", "DEFAULT_TERMS",
           "DEN_RSD_TERMS", "divergent_separations"]
