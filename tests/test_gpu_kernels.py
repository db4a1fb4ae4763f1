"""Device building blocks checked on the GPU through the C ABI."""
import ctypes as C

import numpy as np
import pytest

from magudi_gb300 import capi
from magudi_gb300.solver import load_library

pytestmark = pytest.mark.gpu


def test_table_driven_pow_matches_cuda_pow():
    """The viscosity law uses a table-driven x^n (Tang's method); its error
    against CUDA's pow stays below 4e-15 relative on x in [1e-3, 1e3]."""
    L = load_library()
    L.mgd_selftest_pow.argtypes = [C.POINTER(C.c_double), C.c_int, C.c_double,
                                   C.POINTER(C.c_double), C.POINTER(C.c_double)]
    rng = np.random.default_rng(0)
    x = np.ascontiguousarray(10.0 ** rng.uniform(-3, 3, 200000))
    for e in (0.666, 0.76, 0.5, 1.5):
        fast = np.zeros_like(x)
        ref = np.zeros_like(x)
        assert L.mgd_selftest_pow(capi.dptr(x), x.size, e, capi.dptr(fast), capi.dptr(ref)) == 0
        rel = np.abs(fast - ref) / ref
        assert rel.max() < 4e-15, (e, rel.max())
