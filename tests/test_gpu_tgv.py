"""3D periodic Taylor-Green vortex with the terminal kinetic-energy functional
(-m gpu): J and the adjoint state at t = 0 against the oracle in constant-dt
and constant-CFL mode, and the GPU gradient against central differences."""
import numpy as np
import pytest

import oracle_lib
from helpers import rel_err
from magudi_gb300 import capi, configs
from magudi_gb300.solver import Solver

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("dt", [0.02, None])
def test_tgv_terminal_energy_matches_oracle(dt):
    P = configs.taylor_green_3d(n=16, dt=dt, n_steps=8, save_interval=3)
    g, o = Solver(P), oracle_lib.Oracle(P)
    Jg = g.run_forward(P.n_steps, P.save_interval)
    Jo = o.run_forward(P.n_steps, P.save_interval)
    assert abs(Jg - Jo) <= 1e-12 * abs(Jo)
    g.run_adjoint()
    o.run_adjoint()
    assert rel_err(g.get_field(1, capi.FIELD_ADJOINT), o.get_field(1, capi.FIELD_ADJOINT)) < 1e-10


def test_tgv_terminal_energy_gradient_finite_differences():
    P = configs.taylor_green_3d(n=16, dt=0.02, n_steps=6, save_interval=2)
    q0 = P.blocks[0].initial_state.copy()
    dq = np.random.default_rng(6).standard_normal(q0.shape) * 1e-2
    s = Solver(P)
    norm = s.get_field(1, capi.FIELD_NORM)

    def J(q):
        s.set_field(1, capi.FIELD_CONSERVED, q)
        return s.run_forward(P.n_steps, P.save_interval)

    J(q0)
    s.run_adjoint()
    an = np.sum(norm * s.get_field(1, capi.FIELD_ADJOINT) * dq)
    eps = 1e-4
    fd = (J(q0 + eps * dq) - J(q0 - eps * dq)) / (2 * eps)
    assert abs(fd - an) <= 1e-7 * abs(an)
