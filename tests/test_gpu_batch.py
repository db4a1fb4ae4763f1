"""Batched forward runs (mgd_batch_*) against the single-solve path and the
oracle (-m gpu): instances of different grid sizes and control amplitudes,
as in the reference's gradient-accuracy sweep (README.md:118-165)."""
import numpy as np
import pytest

import oracle_lib
from helpers import rel_err, small_monopole
from magudi_gb300 import capi
from magudi_gb300.solver import Batch, Solver

pytestmark = pytest.mark.gpu

SIZES = [(41, 37), (33, 45), (49, 29)]
N_STEPS = 12


def _gradient_direction(n, ny):
    P = small_monopole(n=n, ny=ny, n_steps=N_STEPS, save_interval=4)
    s = Solver(P)
    s.run_forward(N_STEPS, 4)
    s.run_adjoint()
    return s.gradient(4 * N_STEPS)


def _controlled(n, ny, forcing):
    P = small_monopole(n=n, ny=ny, n_steps=N_STEPS, controller_switch=True)
    s = Solver(P)
    s.set_control_forcing(forcing)
    return P, s


def test_batch_matches_single_solves_and_oracle():
    grads = {sz: _gradient_direction(*sz) for sz in SIZES}
    amps = [10.0 ** (-2.0 - 0.25 * k) for k in range(6)]
    cases = [(SIZES[i % len(SIZES)], amps[i]) for i in range(len(amps))]
    solvers = [_controlled(n, ny, a * grads[(n, ny)])[1] for (n, ny), a in cases]
    batch = Batch(solvers)
    batch.kernel_launches(reset=True)
    costs = batch.run_forward(N_STEPS)
    assert batch.kernel_launches() > 0
    for i, ((n, ny), a) in enumerate(cases):
        P, single = _controlled(n, ny, a * grads[(n, ny)])
        J = single.run_forward(N_STEPS, N_STEPS)
        # same per-point arithmetic and reduction layout; the batched and single
        # kernels are compiled separately, so allow FMA-contraction differences
        assert abs(costs[i] - J) <= 1e-12 * abs(J)
        assert rel_err(solvers[i].get_field(1, capi.FIELD_CONSERVED), single.get_field(1, capi.FIELD_CONSERVED)) < 1e-13
        o = oracle_lib.Oracle(P)
        o.set_control_forcing(a * grads[(n, ny)])
        Jo = o.run_forward(N_STEPS, keep_stages=False)
        assert abs(costs[i] - Jo) <= 1e-10 * abs(Jo)


def test_batch_rerun_and_reuse():
    """A batch can run again from new states; the captured graph is reused."""
    solvers = [Solver(small_monopole(n=n, ny=ny, n_steps=N_STEPS)) for n, ny in SIZES]
    batch = Batch(solvers)
    c1 = batch.run_forward(N_STEPS)
    for s in solvers:
        s.set_field(1, capi.FIELD_CONSERVED, s.problem.blocks[0].initial_state)
    c2 = batch.run_forward(N_STEPS)
    assert np.array_equal(c1, c2)  # deterministic: fixed reduction order, no atomics


def test_batch_rejects_mismatched_options():
    a = Solver(small_monopole())
    b = Solver(small_monopole(dt=0.04))
    with pytest.raises(Exception):
        Batch([a, b])


def test_persistent_launch_equals_per_step_graphs_and_oracle():
    """The default run is one persistent cooperative launch for all steps;
    its costs and final states equal the per-step graph path's bit for bit
    (same per-point arithmetic and reduction layout) and the oracle's."""
    grads = {sz: _gradient_direction(*sz) for sz in SIZES}
    cases = [(SIZES[i % len(SIZES)], 10.0 ** (-2.0 - 0.25 * i)) for i in range(5)]

    def make():
        return [_controlled(n, ny, a * grads[(n, ny)])[1] for (n, ny), a in cases]

    per_step, persistent = make(), make()
    b0, b1 = Batch(per_step), Batch(persistent)
    assert b0.persistent(0) == 0 and b1.persistent() == 1 and b1.persistent_grid() > 0
    b1.kernel_launches(reset=True)
    c0, c1 = b0.run_forward(N_STEPS), b1.run_forward(N_STEPS)
    assert b1.kernel_launches() == 1
    assert np.array_equal(c0, c1)
    for s0, s1 in zip(per_step, persistent):
        assert np.array_equal(s0.get_field(1, capi.FIELD_CONSERVED), s1.get_field(1, capi.FIELD_CONSERVED))
    for i, ((n, ny), a) in enumerate(cases):
        P = small_monopole(n=n, ny=ny, n_steps=N_STEPS, controller_switch=True)
        o = oracle_lib.Oracle(P)
        o.set_control_forcing(a * grads[(n, ny)])
        Jo = o.run_forward(N_STEPS, keep_stages=False)
        assert abs(c1[i] - Jo) <= 1e-10 * abs(Jo)
    # a second run of the same length reuses the captured launch
    for s in persistent:
        s.set_field(1, capi.FIELD_CONSERVED, s.problem.blocks[0].initial_state)
    assert np.array_equal(b1.run_forward(N_STEPS), c1)


def test_persistent_queue_many_instances_equals_per_step_graphs():
    """Sixteen instances of four sizes: the work queue interleaves their
    units, and a unit waits only for its own instance's previous phase;
    costs and states equal the per-step graph path's bit for bit."""
    sizes = [(41, 37), (65, 63), (33, 45), (97, 81)]

    def make():
        return [Solver(small_monopole(n=sizes[i % 4][0], ny=sizes[i % 4][1], n_steps=8)) for i in range(16)]

    per_step, persistent = make(), make()
    b0, b1 = Batch(per_step), Batch(persistent)
    b0.persistent(0)
    assert b1.persistent() == 1
    c0, c1 = b0.run_forward(8), b1.run_forward(8)
    assert np.array_equal(c0, c1)
    for s0, s1 in zip(per_step, persistent):
        assert np.array_equal(s0.get_field(1, capi.FIELD_CONSERVED), s1.get_field(1, capi.FIELD_CONSERVED))


def test_persistent_queue_3d_equals_per_step_graphs_and_single_solves():
    """3D instances (periodic Taylor-Green grids of two sizes at a fixed step
    size): the persistent kernel's 3D form equals the per-step graph path bit
    for bit, and the single-solve path to rounding."""
    from magudi_gb300 import configs

    def problem(n):
        P = configs.taylor_green_3d(n=n, n_steps=6, dt=2e-3, save_interval=6)
        P.options.enable_functional = False
        return P

    sizes = (12, 16, 12)
    per_step = [Solver(problem(n)) for n in sizes]
    persistent = [Solver(problem(n)) for n in sizes]
    b0, b1 = Batch(per_step), Batch(persistent)
    b0.persistent(0)
    assert b1.persistent() == 1
    b0.run_forward(6)
    b1.run_forward(6)
    for s0, s1 in zip(per_step, persistent):
        assert np.array_equal(s0.get_field(1, capi.FIELD_CONSERVED), s1.get_field(1, capi.FIELD_CONSERVED))
    single = Solver(problem(16))
    single.run_forward(6, 6)
    assert rel_err(persistent[1].get_field(1, capi.FIELD_CONSERVED), single.get_field(1, capi.FIELD_CONSERVED)) < 1e-13


def test_grid_barrier_completes_and_its_wait_runs_out_without_a_fault():
    """The persistent kernel's bounded wait, used as a grid barrier: 64 CTAs
    meet 50 times and see each other's writes; then a barrier that expects
    one CTA more than the launch has (an arrival that never comes) gives up
    after its poll limit, returns status 1, and the context stays usable."""
    import ctypes as C
    from magudi_gb300.solver import load_library
    L = load_library()
    status, checksum = C.c_int(-1), C.c_longlong(0)
    assert L.mgd_selftest_grid_barrier(64, 64, 50, 1 << 24, C.byref(status), C.byref(checksum)) == 0
    assert status.value == 0 and checksum.value == (50 * 51 // 2) * (64 * 65 // 2)
    assert L.mgd_selftest_grid_barrier(16, 17, 3, 2000, C.byref(status), C.byref(checksum)) == 0
    assert status.value == 1
    # the device still runs work afterwards
    s = Solver(small_monopole())
    s.compute_rhs(capi.FORWARD, 0.0)
    assert np.all(np.isfinite(s.get_field(1, capi.FIELD_RHS)))
