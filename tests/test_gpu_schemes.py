"""The SBP 1-2, 2-4 and 3-6 schemes (defaults/discretization_scheme) on the
GPU against the oracle (-m gpu): forward and adjoint RHS on full_rhs-style
random states with composite and non-composite dissipation (SBP 1-2 has only
the composite one), curvilinear and 3D periodic grids, and a short
checkpointed forward + adjoint run. Tolerances: 1e-12 per RHS, 1e-10 for J,
Grad0 and the gradient vector."""
import numpy as np
import pytest

import oracle_lib
from helpers import random_full_rhs_state, rel_err, small_monopole
from magudi_gb300 import capi, configs
from magudi_gb300.solver import Solver

pytestmark = pytest.mark.gpu

CASES = [(capi.SBP_12, True), (capi.SBP_24, True), (capi.SBP_24, False), (capi.SBP_36, True),
         (capi.SBP_36, False)]


def _problem(scheme, composite, **kw):
    P = small_monopole(**kw)
    P.options.discretization_scheme = scheme
    P.options.composite_dissipation = composite
    if not composite:
        P.options.dissipation_amount = 1e-3
    return P


@pytest.mark.parametrize("scheme,composite", CASES)
def test_forward_and_adjoint_rhs_match_oracle(scheme, composite):
    P = _problem(scheme, composite)
    q, lam = random_full_rhs_state(P, 13)
    pair = (Solver(P), oracle_lib.Oracle(P))
    for s in pair:
        s.set_field(1, capi.FIELD_CONSERVED, q)
        s.set_field(1, capi.FIELD_ADJOINT, lam)
        s.update_state()
        s.update_adjoint_forcing(False)
    for s in pair:
        s.compute_rhs(capi.FORWARD, 0.6)
    assert rel_err(pair[0].get_field(1, capi.FIELD_RHS), pair[1].get_field(1, capi.FIELD_RHS)) < 1e-12
    for s in pair:
        s.compute_rhs(capi.ADJOINT, 0.6, 2.0)
    assert rel_err(pair[0].get_field(1, capi.FIELD_RHS), pair[1].get_field(1, capi.FIELD_RHS)) < 1e-12
    # the grid norm follows the scheme's boundary norm
    assert rel_err(pair[0].get_field(1, capi.FIELD_NORM), pair[1].get_field(1, capi.FIELD_NORM)) < 1e-14


@pytest.mark.parametrize("scheme", [capi.SBP_24, capi.SBP_36])
def test_curvilinear_rhs_matches_oracle(scheme):
    P = _problem(scheme, False)
    P.options.curvilinear = True
    blk = P.blocks[0]
    x, y = blk.coordinates
    blk.coordinates = np.ascontiguousarray(np.stack([x + 0.1 * np.sin(0.4 * y), y + 0.05 * np.sin(0.3 * x)]))
    q, lam = random_full_rhs_state(P, 3)
    pair = (Solver(P), oracle_lib.Oracle(P))
    for s in pair:
        s.set_field(1, capi.FIELD_CONSERVED, q)
        s.set_field(1, capi.FIELD_ADJOINT, lam)
        s.update_state()
        s.compute_rhs(capi.FORWARD, 0.1)
    assert rel_err(pair[0].get_field(1, capi.FIELD_RHS), pair[1].get_field(1, capi.FIELD_RHS)) < 1e-12
    for s in pair:
        s.compute_rhs(capi.ADJOINT, 0.1, 1.0)
    assert rel_err(pair[0].get_field(1, capi.FIELD_RHS), pair[1].get_field(1, capi.FIELD_RHS)) < 1e-12


@pytest.mark.parametrize("scheme", [capi.SBP_12, capi.SBP_24, capi.SBP_36])
def test_periodic_3d_rhs_matches_oracle(scheme):
    P = configs.taylor_green_3d(n=20, dt=0.01)
    P.options.discretization_scheme = scheme
    lam = np.random.default_rng(2).uniform(0.0, 1.0, P.blocks[0].initial_state.shape)
    pair = (Solver(P), oracle_lib.Oracle(P))
    for s in pair:
        s.set_field(1, capi.FIELD_ADJOINT, lam)
        s.update_state()
        s.compute_rhs(capi.FORWARD, 0.0)
    assert rel_err(pair[0].get_field(1, capi.FIELD_RHS), pair[1].get_field(1, capi.FIELD_RHS)) < 1e-12
    for s in pair:
        s.compute_rhs(capi.ADJOINT, 0.0, 1.0)
    assert rel_err(pair[0].get_field(1, capi.FIELD_RHS), pair[1].get_field(1, capi.FIELD_RHS)) < 1e-12


@pytest.mark.parametrize("scheme,composite", [(capi.SBP_24, True), (capi.SBP_36, False)])
def test_checkpointed_gradient_run_matches_oracle(scheme, composite):
    P = _problem(scheme, composite, n_steps=16, save_interval=5)
    g, o = Solver(P), oracle_lib.Oracle(P)
    Jg, Jo = g.run_forward(16, 5), o.run_forward(16, 5)
    assert abs(Jg - Jo) <= 1e-10 * abs(Jo)
    Gg, Go = g.run_adjoint(), o.run_adjoint()
    assert abs(Gg - Go) <= 1e-10 * abs(Go)
    assert rel_err(g.gradient(64), o.gradient(64)) < 1e-10
