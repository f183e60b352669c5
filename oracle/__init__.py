"""CPU oracle for the COFFE hot path -- TEST INFRASTRUCTURE ONLY.

The C restatement in ``coffe_oracle.c`` is loaded through ctypes.  Only the test
suite, ``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py`` may
use this package; the product (``coffe_gb300``) never imports it.
"""
from .oracle import *  # noqa: F401,F403
