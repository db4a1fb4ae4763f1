"""The reference's own AcousticMonopole example, magudi.inp and bc.dat
unchanged (SBP 3-6, non-composite dissipation, solution limits, off-centre
acoustic source, B-spline/tanh mollifiers of the example's config.py), on
the GPU against the oracle (-m gpu): the forward and adjoint RHS of a
perturbed state, and a 40-step checkpointed forward + adjoint run."""
import numpy as np
import pytest

import oracle_lib
from helpers import rel_err
from magudi_gb300 import capi
from magudi_gb300.solver import Solver
from test_dropin_inputs import example_problem

pytestmark = pytest.mark.gpu


def test_example_rhs_matches_oracle():
    P = example_problem()
    rng = np.random.default_rng(8)
    q = P.blocks[0].initial_state * (1.0 + 1e-2 * rng.standard_normal(P.blocks[0].initial_state.shape))
    q[1:3] = 1e-2 * rng.standard_normal((2, q.shape[1]))
    lam = rng.uniform(-1.0, 1.0, q.shape)
    pair = (Solver(P), oracle_lib.Oracle(P))
    for s in pair:
        s.set_field(1, capi.FIELD_CONSERVED, q)
        s.set_field(1, capi.FIELD_ADJOINT, lam)
        s.update_state()
        s.update_adjoint_forcing(False)
        s.compute_rhs(capi.FORWARD, 1.3)
    assert rel_err(pair[0].get_field(1, capi.FIELD_RHS), pair[1].get_field(1, capi.FIELD_RHS)) < 1e-12
    for s in pair:
        s.compute_rhs(capi.ADJOINT, 1.3, 1.0)
    assert rel_err(pair[0].get_field(1, capi.FIELD_RHS), pair[1].get_field(1, capi.FIELD_RHS)) < 1e-12


def test_example_run_matches_oracle():
    P = example_problem()
    g, o = Solver(P), oracle_lib.Oracle(P)
    Jg, Jo = g.run_forward(40, 10), o.run_forward(40, 10)
    assert g.limit_violation is None and o.run_status == 0
    assert abs(Jg - Jo) <= 1e-10 * abs(Jo)
    Gg, Go = g.run_adjoint(), o.run_adjoint()
    assert abs(Gg - Go) <= 1e-10 * abs(Go)
    assert rel_err(g.gradient(160), o.gradient(160)) < 1e-10
