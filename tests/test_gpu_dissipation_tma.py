"""The composite dissipation of fully periodic 3D blocks with its operands
staged in shared memory by the tensor memory accelerator (kDissipationTma3,
selected with mgd_dissipation_tma) against the default form that reads them
through L1 and against the oracle (-m gpu): forward and adjoint RHS of a perturbed
Taylor-Green state, and a checkpointed constant-CFL forward + adjoint run.
The two forms evaluate the same operations in the same order; the compiler
may contract their multiply-adds differently, so they agree to rounding
(measured 9e-15 and 2e-14 relative in the forward RHS at 32^3 and 64^3)."""
import numpy as np
import pytest

import oracle_lib
from helpers import rel_err
from magudi_gb300 import capi, configs
from magudi_gb300.solver import Solver

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n", [32, 64])
def test_tma_form_equals_the_l1_form_and_the_oracle(n):
    P = configs.taylor_green_3d(n=n, n_steps=4, save_interval=2)
    tma, l1 = Solver(P), Solver(P)
    assert l1.dissipation_tma() == 0
    assert tma.dissipation_tma(1) == 1
    rng = np.random.default_rng(n)
    q = P.blocks[0].initial_state * (1.0 + 1e-3 * rng.standard_normal(P.blocks[0].initial_state.shape))
    lam = rng.uniform(-1.0, 1.0, q.shape)
    o = oracle_lib.Oracle(P)
    for s in (tma, l1, o):
        s.set_field(1, capi.FIELD_CONSERVED, q)
        s.set_field(1, capi.FIELD_ADJOINT, lam)
        s.update_state()
    for mode in (capi.FORWARD, capi.ADJOINT):
        for s in (tma, l1, o):
            s.compute_rhs(mode, 0.0, 1.0)
        r = [s.get_field(1, capi.FIELD_RHS) for s in (tma, l1, o)]
        assert rel_err(r[0], r[1]) < 1e-13
        assert rel_err(r[0], r[2]) < 1e-12
    res = []
    for s in (tma, l1):
        s.set_field(1, capi.FIELD_CONSERVED, P.blocks[0].initial_state)
        J = s.run_forward(P.n_steps, P.save_interval)
        s.run_adjoint()
        res.append((J, s.get_field(1, capi.FIELD_ADJOINT)))
    assert abs(res[0][0] - res[1][0]) <= 1e-12 * abs(res[1][0])
    assert rel_err(res[0][1], res[1][1]) < 1e-12
