"""Constant-CFL mode (Region%getTimeStepSize, src/RegionImpl.f90:1842-1875;
computeTimeStepSize, src/CNSHelperImpl.f90:913-982): the device step size
against the oracle, and forward/adjoint runs whose step size changes every
step (-m gpu)."""
import numpy as np
import pytest

import oracle_lib
from helpers import random_full_rhs_state, rel_err, small_monopole
from magudi_gb300 import capi, configs
from magudi_gb300.solver import Solver

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("seed", [5, 9])
def test_time_step_size_random_state(seed):
    P = small_monopole(cfl=0.5)
    q, _ = random_full_rhs_state(P, seed)
    g, o = Solver(P), oracle_lib.Oracle(P)
    for s in (g, o):
        s.set_field(1, capi.FIELD_CONSERVED, q)
        s.update_state()
    dg, do = g.time_step_size(), o.time_step_size()
    assert abs(dg - do) <= 1e-14 * do


def test_time_step_size_taylor_green():
    P = configs.taylor_green_3d(n=16, cfl=0.5)
    g, o = Solver(P), oracle_lib.Oracle(P)
    for s in (g, o):
        s.update_state()
    dg, do = g.time_step_size(), o.time_step_size()
    assert abs(dg - do) <= 1e-14 * do


def test_constant_dt_mode_returns_the_option():
    P = small_monopole(dt=0.05)
    assert Solver(P).time_step_size() == 0.05


def test_cfl_run_forward_adjoint_matches_oracle():
    P = small_monopole(cfl=0.8, n_steps=24, save_interval=7)
    g, o = Solver(P), oracle_lib.Oracle(P)
    Jg = g.run_forward(P.n_steps, P.save_interval)
    Jo = o.run_forward(P.n_steps, P.save_interval)
    dts_g, dts_o = g.step_sizes(P.n_steps), o.step_sizes(P.n_steps)
    assert np.max(np.abs(dts_g - dts_o) / dts_o) < 1e-13
    assert np.ptp(dts_o) > 0.0  # the step size does change along the run
    assert abs(Jg - Jo) <= 1e-10 * abs(Jo)
    assert rel_err(g.get_field(1, capi.FIELD_CONSERVED), o.get_field(1, capi.FIELD_CONSERVED)) < 1e-11
    Gg, Go = g.run_adjoint(), o.run_adjoint()
    assert abs(Gg - Go) <= 1e-10 * abs(Go)
    ng = 4 * P.n_steps
    assert rel_err(g.gradient(ng), o.gradient(ng)) < 1e-10
