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


def _noalloc(s, q, t):
    """One call of the entry point on a device copy of q; returns the RHS."""
    import torch
    q_dev = torch.from_numpy(np.ascontiguousarray(q)).cuda()
    rhs_dev = torch.full_like(q_dev, float("nan"))
    torch.cuda.synchronize()  # q must be complete on the device before the call
    rc = s.L.mgd_forward_rhs_noalloc(s.h, q_dev.data_ptr(), t, rhs_dev.data_ptr())
    assert rc == 0, s.L.mgd_last_error(s.h).decode()
    return rhs_dev.cpu().numpy()


def test_noalloc_adds_the_actuator_forcing_like_the_allocating_path():
    """With the controller on and a forcing handed to the actuators, both
    paths add ActuatorPatch%updateRhs's term (two calls, two forcings)."""
    pytest.importorskip("torch")
    P = small_monopole(controller_switch=True)
    s = Solver(P)
    _bind(s.L)
    rng = np.random.default_rng(5)
    q = configs.smooth_perturbed_state(P.blocks[0], 2, 1.4, rng)
    for t in (0.3, 0.8):
        f = 1e-2 * rng.standard_normal(s.actuator_points())
        s.set_patch_control_forcing(f)
        s.set_field(1, capi.FIELD_CONSERVED, q)
        s.update_state()
        s.compute_rhs(capi.FORWARD, t)
        expected = s.get_field(1, capi.FIELD_RHS)
        got = _noalloc(s, q, t)
        assert rel_err(got, expected) < RHS_TOL
        # the forcing changes the result, so the comparison covers it
        s.set_patch_control_forcing(np.zeros_like(f))
        s.compute_rhs(capi.FORWARD, t)
        assert rel_err(s.get_field(1, capi.FIELD_RHS), expected) > 1e-8


def test_noalloc_refuses_a_block_with_interface_patches():
    """One block whose x faces are joined by block-interface patches (an
    O-grid style cut) needs the interface SATs, which only mgd_compute_rhs runs."""
    pytest.importorskip("torch")
    from magudi_gb300.problem import Patch
    P = small_monopole()
    P.patches = [p for p in P.patches if p.name not in ("farField.W", "farField.E")]
    names = {p.name for p in P.patches}
    assert not ({"farField.W", "farField.E"} & names)
    P.patches += [Patch("cut.W", "SAT_BLOCK_INTERFACE", 1, 1, (1, 1, 1, -1, 1, -1), viscous_penalty_amount=0.5),
                  Patch("cut.E", "SAT_BLOCK_INTERFACE", 1, -1, (-1, -1, 1, -1, 1, -1), viscous_penalty_amount=0.5,
                        conforms_with="cut.W")]
    s = Solver(P)
    _bind(s.L)
    import torch
    q_dev = torch.from_numpy(np.ascontiguousarray(P.blocks[0].initial_state)).cuda()
    rhs_dev = torch.zeros_like(q_dev)
    torch.cuda.synchronize()
    rc = s.L.mgd_forward_rhs_noalloc(s.h, q_dev.data_ptr(), 0.0, rhs_dev.data_ptr())
    assert rc != 0
    assert b"interface" in s.L.mgd_last_error(s.h)


@pytest.mark.parametrize("resident", [False, True])
def test_noalloc_between_forward_and_adjoint_runs_leaves_the_gradient_bitwise(resident):
    """A call between mgd_run_forward and mgd_run_adjoint touches neither the
    checkpoints nor the trajectory nor the state the adjoint starts from."""
    pytest.importorskip("torch")
    P = small_monopole(n_steps=12, save_interval=4)
    ref, s = Solver(P), Solver(P)
    _bind(s.L)
    for x in (ref, s):
        x.set_trajectory_storage(resident)
    J0 = ref.run_forward(P.n_steps, P.save_interval)
    G0 = ref.run_adjoint()
    g0 = ref.gradient(4 * P.n_steps)
    J1 = s.run_forward(P.n_steps, P.save_interval)
    q = configs.smooth_perturbed_state(P.blocks[0], 2, 1.4, np.random.default_rng(9))
    _noalloc(s, q, 0.45)
    _noalloc(s, q, 0.55)
    G1 = s.run_adjoint()
    assert J1 == J0
    assert G1 == G0
    assert np.array_equal(s.gradient(4 * P.n_steps), g0)
