"""Parity at the headline configurations (-m gpu), through the C ABI.

- The 2D acoustic monopole exactly as the benchmark builds it: 201 x 201 on
  [-14, 14]^2, 960 RK4 steps at dt = 0.05, checkpoints every 10 steps. J,
  Grad0 (the sensitivity) and the whole gradient vector (3840 stage entries
  of every actuator point) after the complete forward + adjoint run, with the
  forward recomputed between checkpoints on the device and with the
  trajectory kept resident; the final forward state too.
- The adjoint RHS of the 201 x 201 monopole on a smooth state.
- The 3D periodic Taylor-Green vortex at 48^3 for 20 constant-CFL steps:
  terminal kinetic energy, every step size, and the adjoint state at t = 0.

Tolerances: J, Grad0 and the gradient vector 1e-10 relative (norm-wise for
vectors); per-RHS 1e-12.
"""
import os

import numpy as np
import pytest

import oracle_lib
from helpers import rel_err
from magudi_gb300 import capi, configs
from magudi_gb300.solver import Solver

pytestmark = pytest.mark.gpu

RUN_TOL = 1e-10
RHS_TOL = 1e-12


def _monopole_201():
    return configs.monopole_2d(n=201, n_steps=960, save_interval=10)


@pytest.fixture(scope="module")
def monopole_oracle_run():
    """The oracle's complete 960-step forward + adjoint run of the monopole
    (about 20 s on 16 cores), shared by the two storage modes."""
    oracle_lib.set_threads(os.cpu_count())
    P = _monopole_201()
    o = oracle_lib.Oracle(P)
    J = o.run_forward(P.n_steps, P.save_interval)
    q_final = o.get_field(1, capi.FIELD_CONSERVED)
    G = o.run_adjoint()
    n = 4 * P.n_steps
    return {"J": J, "G": G, "q": q_final, "grad": o.gradient(n), "lam0": o.get_field(1, capi.FIELD_ADJOINT)}


@pytest.mark.parametrize("resident", [False, True], ids=["checkpoint_recompute", "resident_trajectory"])
def test_monopole_201_gradient_matches_oracle_after_960_steps(monopole_oracle_run, resident):
    ref = monopole_oracle_run
    P = _monopole_201()
    s = Solver(P)
    s.set_trajectory_storage(resident)
    J = s.run_forward(P.n_steps, P.save_interval)
    assert abs(J - ref["J"]) <= RUN_TOL * abs(ref["J"])
    assert rel_err(s.get_field(1, capi.FIELD_CONSERVED), ref["q"]) < RUN_TOL
    G = s.run_adjoint()
    assert abs(G - ref["G"]) <= RUN_TOL * abs(ref["G"])
    assert rel_err(s.gradient(4 * P.n_steps), ref["grad"]) < RUN_TOL
    assert rel_err(s.get_field(1, capi.FIELD_ADJOINT), ref["lam0"]) < RUN_TOL


def test_monopole_201_adjoint_rhs_matches_oracle():
    P = configs.monopole_2d(n=201)
    rng = np.random.default_rng(12)
    q = configs.smooth_perturbed_state(P.blocks[0], 2, 1.4, rng)
    lam = rng.uniform(-1.0, 1.0, q.shape)
    pair = (Solver(P), oracle_lib.Oracle(P))
    for s in pair:
        s.set_field(1, capi.FIELD_CONSERVED, q)
        s.set_field(1, capi.FIELD_ADJOINT, lam)
        s.update_state()
        s.update_adjoint_forcing(False)
        s.compute_rhs(capi.ADJOINT, 4.1, 2.0)
    assert rel_err(pair[0].get_field(1, capi.FIELD_RHS), pair[1].get_field(1, capi.FIELD_RHS)) < RHS_TOL


def test_tgv_48_constant_cfl_run_matches_oracle():
    oracle_lib.set_threads(os.cpu_count())
    P = configs.taylor_green_3d(n=48, n_steps=20, save_interval=5)
    assert P.options.use_constant_cfl
    g, o = Solver(P), oracle_lib.Oracle(P)
    Jg = g.run_forward(P.n_steps, P.save_interval)
    Jo = o.run_forward(P.n_steps, P.save_interval)
    assert abs(Jg - Jo) <= RUN_TOL * abs(Jo)
    dg, do = g.step_sizes(P.n_steps), o.step_sizes(P.n_steps)
    assert np.max(np.abs(dg - do) / do) < 1e-12
    assert np.ptp(do) > 0.0  # the step size follows the flow
    assert rel_err(g.get_field(1, capi.FIELD_CONSERVED), o.get_field(1, capi.FIELD_CONSERVED)) < RUN_TOL
    g.run_adjoint()
    o.run_adjoint()
    assert rel_err(g.get_field(1, capi.FIELD_ADJOINT), o.get_field(1, capi.FIELD_ADJOINT)) < RUN_TOL
