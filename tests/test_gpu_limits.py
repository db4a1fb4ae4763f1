"""Solution limits (enable_solution_limits; checkSolutionLimits,
src/SolverImpl.f90:189-304) on the GPU against the oracle (-m gpu).

Every violation is made on the host: a state with a NaN, a density below
the minimum set with mgd_set_field, or a temperature range that the
monopole's source crosses after some steps. GPU and oracle both return
J = HUGE with status MGD_SOLUTION_LIMITS, stop on the same stage (the
conserved variables left at the violating state agree), and the adjoint
after such a run returns HUGE too. A run that stays inside the limits gives
the same J and gradient as a run without them, bit for bit.
"""
import sys

import numpy as np
import pytest

import oracle_lib
from helpers import rel_err, small_monopole
from magudi_gb300 import capi
from magudi_gb300.solver import Solver

pytestmark = pytest.mark.gpu

HUGE = sys.float_info.max


def _limited(**kw):
    P = small_monopole(n_steps=12, save_interval=4)
    o = P.options
    o.enable_solution_limits = True
    o.minimum_density, o.maximum_density = kw.get("rho", (0.5, 2.0))
    o.minimum_temperature, o.maximum_temperature = kw.get("T", (1.0, 5.0))
    return P


def _both(P, q=None):
    g, o = Solver(P), oracle_lib.Oracle(P)
    if q is not None:
        for s in (g, o):
            s.set_field(1, capi.FIELD_CONSERVED, q)
    return g, o


def test_state_inside_the_limits_runs_unchanged_bitwise():
    P = _limited()
    ref = small_monopole(n_steps=12, save_interval=4)
    g, r = Solver(P), Solver(ref)
    J, Jr = g.run_forward(12, 4), r.run_forward(12, 4)
    assert g.limit_violation is None
    assert J == Jr
    assert g.run_adjoint() == r.run_adjoint()
    assert np.array_equal(g.gradient(48), r.gradient(48))
    assert g.check_solution_limits()


def test_nan_in_the_initial_state_gives_huge_on_gpu_and_oracle():
    P = _limited()
    q = P.blocks[0].initial_state.copy()
    q[3, 700] = np.nan  # energy at one point: its temperature is NaN
    g, o = _both(P, q)
    assert g.run_forward(12, 4) == HUGE
    assert o.run_forward(12, 4) == HUGE and o.run_status == capi.SOLUTION_LIMITS
    assert "Temperature on grid 1" in g.limit_violation and "step 1, stage 1" in g.limit_violation
    # the run stopped on the initial state, which it left unchanged
    assert np.array_equal(g.get_field(1, capi.FIELD_CONSERVED), q, equal_nan=True)
    assert g.run_adjoint() == HUGE and o.run_adjoint() == HUGE


def test_density_below_the_minimum_gives_huge_on_gpu_and_oracle():
    P = _limited()
    q = P.blocks[0].initial_state.copy()
    N = q.shape[1]
    q[0, N // 3] = 0.4  # below minimum_density = 0.5
    g, o = _both(P, q)
    assert g.run_forward(12, 4) == HUGE
    assert o.run_forward(12, 4) == HUGE
    nx = P.blocks[0].grid_size[0]
    p = N // 3
    assert f"Density on grid 1 at ({p % nx + 1}, {p // nx + 1}, 1)" in g.limit_violation
    assert g.check_solution_limits() is False


def test_run_crossing_the_temperature_limit_stops_on_the_same_stage():
    """The monopole's source heats the gas near the origin: with a maximum
    temperature 2e-4 above the ambient 2.5 the run stops a few steps in."""
    P = _limited(T=(1.0, 2.5 + 2e-4))
    g, o = _both(P)
    Jg, Jo = g.run_forward(12, 4), o.run_forward(12, 4)
    assert Jg == HUGE and Jo == HUGE
    assert "Temperature" in g.limit_violation
    step = int(g.limit_violation.split("forward step ")[1].split(",")[0])
    assert step > 1 and step == len(o.step_sizes(12))  # the oracle's last step is the violating one
    assert rel_err(g.get_field(1, capi.FIELD_CONSERVED), o.get_field(1, capi.FIELD_CONSERVED)) < 1e-12
