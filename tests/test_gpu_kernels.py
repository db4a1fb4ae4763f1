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


def test_fp64_rate_probe_runs_and_is_refused_outside_its_range():
    """mgd_selftest_fp64_rate: a positive rate per warp count, no more than
    the 2 DFMA lane-operations per clock per SM that any count can reach by
    more than clock noise; warp counts outside 1..32 are refused."""
    L = load_library()
    rates = []
    for w in (1, 4):
        r = C.c_double()
        assert L.mgd_selftest_fp64_rate(w, C.byref(r)) == 0
        assert 0.0 < r.value < 2.5
        rates.append(r.value)
    assert rates[1] > rates[0]
    r = C.c_double()
    assert L.mgd_selftest_fp64_rate(0, C.byref(r)) == 1
    assert L.mgd_selftest_fp64_rate(33, C.byref(r)) == 1
