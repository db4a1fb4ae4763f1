"""Resident trajectory (-m gpu): the forward run stores every RK stage on the
device and the adjoint run reads it instead of recomputing checkpoint
segments. The adjoint consumes the same forward states either way, so J, the
sensitivity and the gradient are bitwise those of the checkpointed run, and
both match the oracle."""
import numpy as np
import pytest

import oracle_lib
from helpers import rel_err, small_monopole
from magudi_gb300 import capi, configs
from magudi_gb300.solver import Solver

pytestmark = pytest.mark.gpu


def _gradient(s, P):
    J = s.run_forward(P.n_steps, P.save_interval)
    G = s.run_adjoint()
    return J, G, s.gradient(4 * P.n_steps), s.get_field(1, capi.FIELD_ADJOINT)


@pytest.mark.parametrize("cfl", [False, True])
def test_resident_trajectory_is_bitwise_the_checkpointed_gradient(cfl):
    P = small_monopole(n_steps=30, save_interval=7, **({"cfl": 0.8} if cfl else {}))
    a, b = Solver(P), Solver(P)
    b.set_trajectory_storage(True)
    ra, rb = _gradient(a, P), _gradient(b, P)
    assert ra[0] == rb[0] and ra[1] == rb[1]
    assert np.array_equal(ra[2], rb[2]) and np.array_equal(ra[3], rb[3])
    o = oracle_lib.Oracle(P)
    ro = _gradient(o, P)
    assert abs(rb[0] - ro[0]) <= 1e-10 * abs(ro[0])
    assert abs(rb[1] - ro[1]) <= 1e-10 * abs(ro[1])
    assert rel_err(rb[2], ro[2]) < 1e-10


def test_budget_too_small_falls_back_to_checkpoints():
    P = small_monopole(n_steps=20, save_interval=5)
    a, b = Solver(P), Solver(P)
    b.set_trajectory_storage(True, max_bytes=1024.0)
    ra, rb = _gradient(a, P), _gradient(b, P)
    assert ra[0] == rb[0] and ra[1] == rb[1] and np.array_equal(ra[2], rb[2])


def test_tangent_run_reads_the_trajectory_and_keeps_it_for_the_adjoint():
    """A tangent run between the forward and adjoint runs reads the resident
    slots too: its result and the gradient after it are those of the
    checkpointed runs."""
    P = small_monopole(n_steps=16, save_interval=4)
    a, b = Solver(P), Solver(P)
    b.set_trajectory_storage(True)
    ra = _gradient(a, P)
    rng = np.random.default_rng(4)
    dq0 = 1e-3 * rng.standard_normal((4, P.blocks[0].n_points))
    t = Solver(P)  # checkpointed tangent run from the initial state
    t.run_forward(P.n_steps, P.save_interval)
    t.set_field(1, capi.FIELD_ADJOINT, dq0)
    t.run_linearized()
    dq_a = t.get_field(1, capi.FIELD_ADJOINT)
    Jb = b.run_forward(P.n_steps, P.save_interval)
    b.set_field(1, capi.FIELD_ADJOINT, dq0)
    b.run_linearized()
    assert np.array_equal(b.get_field(1, capi.FIELD_ADJOINT), dq_a)
    b.set_field(1, capi.FIELD_ADJOINT, np.zeros((4, P.blocks[0].n_points)))
    Gb = b.run_adjoint()
    assert Jb == ra[0] and Gb == ra[1]
    assert np.array_equal(b.gradient(4 * P.n_steps), ra[2])


def test_wall_channel_with_resident_trajectory():
    P = configs.wall_channel_2d(wall="SAT_ISOTHERMAL_WALL", n_steps=12)
    a, b = Solver(P), Solver(P)
    b.set_trajectory_storage(True)
    for s in (a, b):
        s.run_forward(P.n_steps, 5)
        s.set_field(1, capi.FIELD_ADJOINT, np.full((4, P.blocks[0].n_points), 1e-3))
        s.set_adjoint_nonzero_initial_condition(True)
        s.run_adjoint()
    assert np.array_equal(a.get_field(1, capi.FIELD_ADJOINT), b.get_field(1, capi.FIELD_ADJOINT))


@pytest.mark.parametrize("rotate", [False, True])
def test_two_block_resident_trajectory_is_bitwise_the_checkpointed_gradient(rotate):
    """A region of two blocks meeting at an interface (a transposing one with
    `rotate`): with trajectory storage the forward run keeps every block's
    stage slots and the adjoint and tangent runs read them, with no
    recomputation; J, the sensitivity, the gradient, both blocks' adjoint
    states and a tangent run in between are those of the checkpointed runs,
    bit for bit."""
    P = configs.two_block_2d(functional=True, rotate_second=rotate, n_steps=24, dt=0.05)
    a, b = Solver(P), Solver(P)
    b.set_trajectory_storage(True)
    rng = np.random.default_rng(8)
    dq0 = [1e-3 * rng.standard_normal((4, blk.n_points)) for blk in P.blocks]
    results = []
    for s in (a, b):
        J = s.run_forward(P.n_steps, 5)
        lam_before = [s.get_field(bi, capi.FIELD_ADJOINT) for bi in (1, 2)]
        for bi in (1, 2):
            s.set_field(bi, capi.FIELD_ADJOINT, dq0[bi - 1])
        s.run_linearized()
        tangent = [s.get_field(bi, capi.FIELD_ADJOINT) for bi in (1, 2)]
        for bi in (1, 2):
            s.set_field(bi, capi.FIELD_ADJOINT, lam_before[bi - 1])
        G = s.run_adjoint()
        results.append((J, G, s.gradient(4 * P.n_steps), [s.get_field(bi, capi.FIELD_ADJOINT) for bi in (1, 2)],
                        tangent))
    ra, rb = results
    assert ra[0] == rb[0] and ra[1] == rb[1]
    assert np.array_equal(ra[2], rb[2])
    for k in (3, 4):
        for x, y in zip(ra[k], rb[k]):
            assert np.array_equal(x, y)
    o = oracle_lib.Oracle(P)
    Jo = o.run_forward(P.n_steps, 5)
    Go = o.run_adjoint()
    assert abs(rb[0] - Jo) <= 1e-10 * abs(Jo) and abs(rb[1] - Go) <= 1e-10 * abs(Go)
