"""Wall SATs on the GPU against the oracle (-m gpu): slip, isothermal (wall
temperature from the target state or given) and adiabatic walls, forward and
adjoint RHS on random states and a short forward run."""
import numpy as np
import pytest

import oracle_lib
from helpers import random_full_rhs_state, rel_err
from magudi_gb300 import capi, configs
from magudi_gb300.solver import Solver

pytestmark = pytest.mark.gpu

CASES = [("SAT_SLIP_WALL", 0.0), ("SAT_ISOTHERMAL_WALL", 0.0), ("SAT_ISOTHERMAL_WALL", 2.5),
         ("SAT_ADIABATIC_WALL", 0.0)]


@pytest.mark.parametrize("wall,tw", CASES)
@pytest.mark.parametrize("viscous", [True, False])
def test_wall_rhs_random_state(wall, tw, viscous):
    P = configs.wall_channel_2d(wall=wall, wall_temperature=tw, viscous=viscous)
    q, lam = random_full_rhs_state(P, 21)
    pair = (Solver(P), oracle_lib.Oracle(P))
    for s in pair:
        s.set_field(1, capi.FIELD_CONSERVED, q)
        s.set_field(1, capi.FIELD_ADJOINT, lam)
        s.update_state()
        s.compute_rhs(capi.FORWARD, 0.0)
    assert rel_err(pair[0].get_field(1, capi.FIELD_RHS), pair[1].get_field(1, capi.FIELD_RHS)) < 1e-12
    for s in pair:
        s.compute_rhs(capi.ADJOINT, 0.0, 1.0)
    assert rel_err(pair[0].get_field(1, capi.FIELD_RHS), pair[1].get_field(1, capi.FIELD_RHS)) < 1e-12


def test_wall_channel_run_matches_oracle():
    P = configs.wall_channel_2d(wall="SAT_ISOTHERMAL_WALL", n_steps=20)
    g, o = Solver(P), oracle_lib.Oracle(P)
    g.run_forward(P.n_steps, 5)
    o.run_forward(P.n_steps, 5)
    assert rel_err(g.get_field(1, capi.FIELD_CONSERVED), o.get_field(1, capi.FIELD_CONSERVED)) < 1e-11
