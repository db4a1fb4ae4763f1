"""mgd_forward_rhs_noalloc: the forward RHS for callers that must not
allocate device memory when they evaluate it (a host that reserved its
device-memory budget up front with its own pool, or a loop that cannot take
cudaMalloc's implicit device synchronisation). Its intermediates live in one
fixed array in device memory, so its result must equal the allocating path's
(mgd_compute_rhs) on consecutive calls, and blocks too large for that array
must be refused with an error.

Collected last on purpose (test_zz_*): a run that stops at the first failure
has already run every other test when it gets here.
"""
import ctypes as C

import numpy as np
import pytest

from helpers import random_full_rhs_state, rel_err, small_monopole
from magudi_gb300 import capi, configs
from magudi_gb300.solver import Solver

pytestmark = pytest.mark.gpu

RHS_TOL = 1e-12  # the per-RHS tolerance of the parity tests


def _bind(L):
    L.mgd_forward_rhs_noalloc.argtypes = [C.c_void_p, C.c_void_p, C.c_double, C.c_void_p]
    L.mgd_forward_rhs_noalloc.restype = C.c_int


@pytest.mark.parametrize("make", [small_monopole, lambda: configs.monopole_2d(n=201)])
def test_noalloc_forward_rhs_equals_allocating_path_on_two_calls(make):
    torch = pytest.importorskip("torch")
    P = make()
    s = Solver(P)
    _bind(s.L)
    for seed, t in ((3, 0.37), (8, 1.9)):  # two calls in a row, different states
        q, _ = random_full_rhs_state(P, seed)
        s.set_field(1, capi.FIELD_CONSERVED, q)
        s.update_state()
        s.compute_rhs(capi.FORWARD, t)
        expected = s.get_field(1, capi.FIELD_RHS)
        q_dev = torch.from_numpy(np.ascontiguousarray(q)).cuda()
        rhs_dev = torch.full_like(q_dev, float("nan"))
        torch.cuda.synchronize()
        rc = s.L.mgd_forward_rhs_noalloc(s.h, q_dev.data_ptr(), t, rhs_dev.data_ptr())
        assert rc == 0, s.L.mgd_last_error(s.h).decode()
        torch.cuda.synchronize()
        assert rel_err(rhs_dev.cpu().numpy(), expected) < RHS_TOL


def test_noalloc_refuses_blocks_above_its_fixed_scratch():
    torch = pytest.importorskip("torch")
    P = configs.monopole_2d(n=401)
    s = Solver(P)
    _bind(s.L)
    q_dev = torch.from_numpy(np.ascontiguousarray(P.blocks[0].initial_state)).cuda()
    rhs_dev = torch.zeros_like(q_dev)
    rc = s.L.mgd_forward_rhs_noalloc(s.h, q_dev.data_ptr(), 0.0, rhs_dev.data_ptr())
    assert rc != 0
    assert b"scratch" in s.L.mgd_last_error(s.h)
