"""Multi-block regions with block-interface SATs on the GPU against the oracle
(-m gpu): forward and adjoint RHS of every block on random states, with a
plain and a transposing (rotated) interface, and RK4 substeps."""
import numpy as np
import pytest

import oracle_lib
from helpers import rel_err
from magudi_gb300 import capi, configs
from magudi_gb300.solver import MagudiError, Solver

pytestmark = pytest.mark.gpu


def _random_states(P, seed):
    rng = np.random.default_rng(seed)
    g = P.options.ratio_of_specific_heats
    qs = [configs.random_state(b.n_points, 2, g, rng) for b in P.blocks]
    lams = [rng.uniform(0.0, 1.0, (4, b.n_points)) for b in P.blocks]
    return qs, lams


def _set(s, qs, lams):
    for bi, (q, l) in enumerate(zip(qs, lams), start=1):
        s.set_field(bi, capi.FIELD_CONSERVED, q)
        s.set_field(bi, capi.FIELD_ADJOINT, l)


@pytest.mark.parametrize("rotate", [False, True])
@pytest.mark.parametrize("viscous", [True, False])
def test_two_block_rhs_matches_oracle(rotate, viscous):
    P = configs.two_block_2d(rotate_second=rotate, viscous=viscous)
    qs, lams = _random_states(P, 31)
    pair = (Solver(P), oracle_lib.Oracle(P))
    for s in pair:
        _set(s, qs, lams)
        s.update_state()
        s.compute_rhs(capi.FORWARD, 0.0)
    for bi in (1, 2):
        assert rel_err(pair[0].get_field(bi, capi.FIELD_RHS), pair[1].get_field(bi, capi.FIELD_RHS)) < 1e-12
    for s in pair:
        s.compute_rhs(capi.ADJOINT, 0.0, 1.0)
    for bi in (1, 2):
        assert rel_err(pair[0].get_field(bi, capi.FIELD_RHS), pair[1].get_field(bi, capi.FIELD_RHS)) < 1e-12


def test_two_block_rk4_substeps_match_oracle():
    P = configs.two_block_2d(rotate_second=True)
    rng = np.random.default_rng(2)
    qs = [configs.smooth_perturbed_state(b, 2, 1.4, rng) for b in P.blocks]
    lams = [rng.uniform(0.0, 1.0, (4, b.n_points)) for b in P.blocks]
    pair = (Solver(P), oracle_lib.Oracle(P))
    for s in pair:
        _set(s, qs, lams)
        s.update_state()
        t = 0.0
        for stage in (1, 2, 3, 4):
            t = s.rk4_substep(capi.FORWARD, t, 0.02, stage)
        t = 1.0
        for stage in (4, 3, 2, 1):
            t = s.rk4_substep(capi.ADJOINT, t, 0.02, stage)
    for bi in (1, 2):
        for f in (capi.FIELD_CONSERVED, capi.FIELD_ADJOINT):
            assert rel_err(pair[0].get_field(bi, f), pair[1].get_field(bi, f)) < 1e-12


@pytest.mark.parametrize("rotate", [False, True])
def test_two_block_constant_cfl_runs_match_oracle(rotate):
    """Constant-CFL checkpointed runs across a block interface: the step size of
    each step is the minimum over both blocks (Region%getTimeStepSize,
    src/RegionImpl.f90:1842-1875), recorded for the adjoint."""
    P = configs.two_block_2d(functional=True, rotate_second=rotate, n_steps=30, dt=0.05)
    P.options.use_constant_cfl = True
    P.options.cfl = 0.6
    g, o = Solver(P), oracle_lib.Oracle(P)
    Jg, Jo = g.run_forward(P.n_steps, 7), o.run_forward(P.n_steps, 7)
    assert abs(Jg - Jo) <= 1e-10 * abs(Jo)
    assert rel_err(g.step_sizes(P.n_steps), o.step_sizes(P.n_steps)) < 1e-13
    Gg, Go = g.run_adjoint(), o.run_adjoint()
    assert abs(Gg - Go) <= 1e-10 * abs(Go)
    n = 4 * P.n_steps
    assert rel_err(g.gradient(n), o.gradient(n)) < 1e-10


@pytest.mark.parametrize("rotate", [False, True])
def test_two_block_runs_match_oracle(rotate):
    """Checkpointed forward and adjoint runs across a block interface."""
    P = configs.two_block_2d(functional=True, rotate_second=rotate, n_steps=40, dt=0.05)
    g, o = Solver(P), oracle_lib.Oracle(P)
    Jg, Jo = g.run_forward(P.n_steps, 7), o.run_forward(P.n_steps, 7)
    assert abs(Jg - Jo) <= 1e-10 * abs(Jo)
    for bi in (1, 2):
        assert rel_err(g.get_field(bi, capi.FIELD_CONSERVED), o.get_field(bi, capi.FIELD_CONSERVED)) < 1e-11
    Gg, Go = g.run_adjoint(), o.run_adjoint()
    assert abs(Gg - Go) <= 1e-10 * abs(Go)
    n = 4 * P.n_steps
    assert rel_err(g.gradient(n), o.gradient(n)) < 1e-10


@pytest.mark.parametrize("rotate", [False, True])
def test_two_block_tangent_run_matches_oracle(rotate):
    """Tangent run of a two-block region against the oracle: the final
    perturbation from a random initial one, and the functional's tangent along
    a control perturbation from a zero initial one."""
    P = configs.two_block_2d(functional=True, rotate_second=rotate, n_steps=12, dt=0.05)
    rng = np.random.default_rng(6)
    dq0 = [1e-3 * rng.standard_normal((4, b.n_points)) for b in P.blocks]
    zeros = [np.zeros((4, b.n_points)) for b in P.blocks]
    g, o = Solver(P), oracle_lib.Oracle(P)
    df = rng.standard_normal((4 * P.n_steps, g.actuator_points()))
    fields, dJ = [], []
    for s in (g, o):
        s.run_forward(P.n_steps, 5)
        for bi in (1, 2):
            s.set_field(bi, capi.FIELD_ADJOINT, dq0[bi - 1])
        s.run_linearized()
        fields.append([s.get_field(bi, capi.FIELD_ADJOINT) for bi in (1, 2)])
        for bi in (1, 2):
            s.set_field(bi, capi.FIELD_ADJOINT, zeros[bi - 1])
        dJ.append(s.run_linearized(df))
    for bi in (0, 1):
        assert rel_err(fields[0][bi], fields[1][bi]) < 1e-10
    assert abs(dJ[0] - dJ[1]) <= 1e-10 * abs(dJ[1])
