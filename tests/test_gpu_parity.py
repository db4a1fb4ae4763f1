"""Parity of the CUDA path against the CPU oracle (-m gpu).

Every comparison goes through the C ABI (magudi_gb300.solver -> libmagudi_gb300.so).
Tolerances: per-RHS norm-wise relative error <= 1e-12 (FP64); time-integrated
J and gradient magnitude <= 1e-10 relative after a run.
"""
import math

import numpy as np
import pytest

import oracle_lib
from helpers import random_full_rhs_state, rel_err, small_monopole
from magudi_gb300 import capi, configs
from magudi_gb300.solver import Solver

pytestmark = pytest.mark.gpu

RHS_TOL = 1e-12
RUN_TOL = 1e-10


def _pair(problem):
    return Solver(problem), oracle_lib.Oracle(problem)


def _set_both(pair, field, arr):
    for s in pair:
        s.set_field(1, field, arr)


def test_library_is_the_cuda_path():
    """The solver runs on the GPU: kernels are counted by the library itself."""
    P = small_monopole()
    s = Solver(P)
    s.kernel_launches(reset=True)
    s.compute_rhs(capi.FORWARD, 0.0)
    assert s.kernel_launches() >= 3


def test_grid_metrics_match_oracle():
    P = small_monopole()
    g, o = _pair(P)
    for f in (capi.FIELD_METRICS, capi.FIELD_JACOBIAN, capi.FIELD_NORM, capi.FIELD_ARC_LENGTHS):
        assert rel_err(g.get_field(1, f), o.get_field(1, f)) < 1e-14


@pytest.mark.parametrize("seed", [3, 11])
def test_forward_rhs_random_state(seed):
    P = small_monopole()
    q, lam = random_full_rhs_state(P, seed)
    pair = _pair(P)
    _set_both(pair, capi.FIELD_CONSERVED, q)
    for s in pair:
        s.update_state()
        s.compute_rhs(capi.FORWARD, 0.37)
    g, o = (s.get_field(1, capi.FIELD_RHS) for s in pair)
    assert rel_err(g, o) < RHS_TOL


@pytest.mark.parametrize("seed", [3, 11])
def test_adjoint_rhs_random_state(seed):
    P = small_monopole()
    q, lam = random_full_rhs_state(P, seed)
    pair = _pair(P)
    _set_both(pair, capi.FIELD_CONSERVED, q)
    _set_both(pair, capi.FIELD_ADJOINT, lam)
    for s in pair:
        s.update_state()
        s.update_adjoint_forcing(False)
    o = pair[1]
    o.compute_rhs(capi.ADJOINT, 0.0, 2.0)
    pair[0].compute_rhs(capi.ADJOINT, 0.0, 2.0)
    g, r = pair[0].get_field(1, capi.FIELD_RHS), o.get_field(1, capi.FIELD_RHS)
    assert rel_err(g, r) < RHS_TOL


@pytest.mark.parametrize("composite", [True, False])
def test_rhs_dissipation_variants(composite):
    P = small_monopole()
    P.options.composite_dissipation = composite
    q, lam = random_full_rhs_state(P, 21)
    pair = _pair(P)
    _set_both(pair, capi.FIELD_CONSERVED, q)
    _set_both(pair, capi.FIELD_ADJOINT, lam)
    for s in pair:
        s.update_state()
        s.update_adjoint_forcing(False)
        s.compute_rhs(capi.FORWARD, 0.1)
    assert rel_err(pair[0].get_field(1, capi.FIELD_RHS), pair[1].get_field(1, capi.FIELD_RHS)) < RHS_TOL
    for s in pair:
        s.compute_rhs(capi.ADJOINT, 0.0, 0.5)
    assert rel_err(pair[0].get_field(1, capi.FIELD_RHS), pair[1].get_field(1, capi.FIELD_RHS)) < RHS_TOL


def test_rhs_inviscid_no_dissipation():
    P = small_monopole()
    P.options.viscous = False
    P.options.dissipation = False
    q, lam = random_full_rhs_state(P, 5)
    pair = _pair(P)
    _set_both(pair, capi.FIELD_CONSERVED, q)
    _set_both(pair, capi.FIELD_ADJOINT, lam)
    for s in pair:
        s.update_state()
        s.compute_rhs(capi.FORWARD, 1.0)
    assert rel_err(pair[0].get_field(1, capi.FIELD_RHS), pair[1].get_field(1, capi.FIELD_RHS)) < RHS_TOL
    for s in pair:
        s.compute_rhs(capi.ADJOINT, 0.0, 1.0)
    assert rel_err(pair[0].get_field(1, capi.FIELD_RHS), pair[1].get_field(1, capi.FIELD_RHS)) < RHS_TOL


def test_curvilinear_metrics_and_rhs():
    P = small_monopole()
    P.options.curvilinear = True
    blk = P.blocks[0]
    x, y = blk.coordinates
    # smooth, non-orthogonal mapping
    blk.coordinates = np.ascontiguousarray(np.stack([x + 0.1 * np.sin(0.4 * y), y + 0.05 * np.sin(0.3 * x)]))
    q, lam = random_full_rhs_state(P, 9)
    pair = _pair(P)
    assert rel_err(pair[0].get_field(1, capi.FIELD_METRICS), pair[1].get_field(1, capi.FIELD_METRICS)) < 1e-14
    _set_both(pair, capi.FIELD_CONSERVED, q)
    _set_both(pair, capi.FIELD_ADJOINT, lam)
    for s in pair:
        s.update_state()
        s.compute_rhs(capi.FORWARD, 0.2)
    assert rel_err(pair[0].get_field(1, capi.FIELD_RHS), pair[1].get_field(1, capi.FIELD_RHS)) < RHS_TOL
    for s in pair:
        s.compute_rhs(capi.ADJOINT, 0.0, 1.0)
    assert rel_err(pair[0].get_field(1, capi.FIELD_RHS), pair[1].get_field(1, capi.FIELD_RHS)) < RHS_TOL


def test_rhs_monopole_201_smooth_state():
    P = configs.monopole_2d(n=201)
    rng = np.random.default_rng(1)
    q = configs.smooth_perturbed_state(P.blocks[0], 2, 1.4, rng)
    pair = _pair(P)
    _set_both(pair, capi.FIELD_CONSERVED, q)
    for s in pair:
        s.update_state()
        s.compute_rhs(capi.FORWARD, 3.3)
    assert rel_err(pair[0].get_field(1, capi.FIELD_RHS), pair[1].get_field(1, capi.FIELD_RHS)) < RHS_TOL


def test_periodic_3d_rhs():
    P = configs.taylor_green_3d(n=20)
    P.options.use_constant_cfl = False
    P.options.time_step_size = 0.01
    rng = np.random.default_rng(2)
    q = P.blocks[0].initial_state
    lam = rng.uniform(0.0, 1.0, q.shape)
    pair = _pair(P)
    _set_both(pair, capi.FIELD_ADJOINT, lam)
    for s in pair:
        s.update_state()
        s.compute_rhs(capi.FORWARD, 0.0)
    assert rel_err(pair[0].get_field(1, capi.FIELD_RHS), pair[1].get_field(1, capi.FIELD_RHS)) < RHS_TOL
    for s in pair:
        s.compute_rhs(capi.ADJOINT, 0.0, 1.0)
    assert rel_err(pair[0].get_field(1, capi.FIELD_RHS), pair[1].get_field(1, capi.FIELD_RHS)) < RHS_TOL


def test_rk4_substeps_forward_and_adjoint():
    P = small_monopole()
    q, lam = random_full_rhs_state(P, 4)
    q = configs.smooth_perturbed_state(P.blocks[0], 2, 1.4, np.random.default_rng(4))
    pair = _pair(P)
    _set_both(pair, capi.FIELD_CONSERVED, q)
    _set_both(pair, capi.FIELD_ADJOINT, lam)
    times = []
    for s in pair:
        s.update_state()
        t = 0.5
        for stage in (1, 2, 3, 4):
            t = s.rk4_substep(capi.FORWARD, t, 0.05, stage)
        times.append(t)
    assert times[0] == times[1]
    assert rel_err(pair[0].get_field(1, capi.FIELD_CONSERVED), pair[1].get_field(1, capi.FIELD_CONSERVED)) < RHS_TOL
    for s in pair:
        s.update_state()
        t = 1.0
        for stage in (4, 3, 2, 1):
            t = s.rk4_substep(capi.ADJOINT, t, 0.05, stage)
    assert rel_err(pair[0].get_field(1, capi.FIELD_ADJOINT), pair[1].get_field(1, capi.FIELD_ADJOINT)) < RHS_TOL


def test_run_forward_adjoint_gradient_matches_oracle():
    P = small_monopole(n_steps=30, save_interval=7)
    g, o = _pair(P)
    Jg = g.run_forward(P.n_steps, P.save_interval)
    Jo = o.run_forward(P.n_steps, P.save_interval)
    assert abs(Jg - Jo) <= RUN_TOL * abs(Jo)
    assert rel_err(g.get_field(1, capi.FIELD_CONSERVED), o.get_field(1, capi.FIELD_CONSERVED)) < 1e-11
    Gg = g.run_adjoint()
    Go = o.run_adjoint()
    assert abs(Gg - Go) <= RUN_TOL * abs(Go)
    ng = 4 * P.n_steps
    assert rel_err(g.gradient(ng), o.gradient(ng)) < 1e-10


def test_controlled_forward_matches_oracle():
    P = small_monopole(n_steps=20, save_interval=5)
    g, o = _pair(P)
    g.run_forward(P.n_steps, P.save_interval)
    o.run_forward(P.n_steps, P.save_interval)
    g.run_adjoint()
    o.run_adjoint()
    grad = o.gradient(4 * P.n_steps)
    P.options.controller_switch = True
    g2, o2 = _pair(P)
    g2.set_control_forcing(1e-2 * grad)
    o2.set_control_forcing(1e-2 * grad)
    J1g = g2.run_forward(P.n_steps, P.save_interval)
    J1o = o2.run_forward(P.n_steps, P.save_interval)
    assert abs(J1g - J1o) <= RUN_TOL * abs(J1o)


def test_per_call_control_flow_reproduces_the_runs_on_the_gpu():
    """The reference's solver loop over the per-call C entry points gives the
    J and gradient norm of mgd_run_forward / mgd_run_adjoint."""
    from magudi_gb300.drivers import per_call_gradient
    P = small_monopole(n_steps=13, save_interval=5)
    s = Solver(P)
    J = s.run_forward(P.n_steps, 5)
    G = s.run_adjoint()
    Jp, Gp = per_call_gradient(Solver(P), P, P.n_steps, 5)
    assert abs(Jp - J) <= 1e-12 * abs(J)
    assert abs(Gp - G) <= 1e-11 * abs(G)


def _holed_monopole(**kw):
    """Monopole grid with a rectangular hole (iblank = 0) away from the source and target."""
    P = small_monopole(**kw)
    nx, ny = P.blocks[0].grid_size[:2]
    ib = np.ones((ny, nx), dtype=np.int32)
    ib[24:29, 8:13] = 0
    P.blocks[0].iblank = ib.ravel()
    return P


def test_holes_metrics_rhs_and_runs_match_oracle():
    """iblank = 0 points: zero metrics and unit Jacobian (src/GridImpl.f90:787-1029),
    patches skip holes, and Region%computeRhs zeroes the RHS there
    (src/RegionImpl.f90:2015-2023)."""
    P = _holed_monopole(n_steps=12, save_interval=4)
    q, lam = random_full_rhs_state(P, 17)
    q = configs.smooth_perturbed_state(P.blocks[0], 2, 1.4, np.random.default_rng(17))
    pair = _pair(P)
    for f in (capi.FIELD_METRICS, capi.FIELD_JACOBIAN, capi.FIELD_NORM):
        assert rel_err(pair[0].get_field(1, f), pair[1].get_field(1, f)) < 1e-14
    _set_both(pair, capi.FIELD_CONSERVED, q)
    _set_both(pair, capi.FIELD_ADJOINT, lam)
    for s in pair:
        s.update_state()
        s.compute_rhs(capi.FORWARD, 0.4)
    g, o = (s.get_field(1, capi.FIELD_RHS) for s in pair)
    hole = P.blocks[0].iblank == 0
    assert np.all(g[:, hole] == 0.0)
    assert rel_err(g, o) < RHS_TOL
    for s in pair:
        s.compute_rhs(capi.ADJOINT, 0.4, 0.0)
    assert rel_err(*(s.get_field(1, capi.FIELD_RHS) for s in pair)) < RHS_TOL
    g, o = _pair(P)
    Jg, Jo = g.run_forward(P.n_steps, 4), o.run_forward(P.n_steps, 4)
    assert abs(Jg - Jo) <= RUN_TOL * abs(Jo)
    Gg, Go = g.run_adjoint(), o.run_adjoint()
    assert abs(Gg - Go) <= RUN_TOL * abs(Go)


def test_per_call_controlled_runs_match_the_graph_path():
    """mgd_set_patch_control_forcing: the per-call forward RHS adds the
    actuators' forcing; the per-call loop then reproduces a controlled run."""
    from magudi_gb300.drivers import per_call_forward, per_call_gradient
    P = small_monopole(n_steps=9, save_interval=4, controller_switch=True)
    s = Solver(P)
    f = 1e-2 * np.random.default_rng(3).standard_normal((4 * P.n_steps, s.actuator_points()))
    s.set_control_forcing(f)
    J = s.run_forward(P.n_steps, 4)
    G = s.run_adjoint()
    assert abs(per_call_forward(Solver(P), P, P.n_steps, f) - J) <= 1e-12 * abs(J)
    Jp, Gp = per_call_gradient(Solver(P), P, P.n_steps, 4, f)
    assert abs(Jp - J) <= 1e-12 * abs(J)
    assert abs(Gp - G) <= 1e-11 * abs(G)
    # per-call RHS with the forcing against the oracle's
    q = configs.smooth_perturbed_state(P.blocks[0], 2, 1.4, np.random.default_rng(4))
    pair = _pair(P)
    for x in pair:
        x.set_field(1, capi.FIELD_CONSERVED, q)
        x.update_state()
        x.set_patch_control_forcing(f[5])
        x.compute_rhs(capi.FORWARD, 0.3)
    assert rel_err(*(x.get_field(1, capi.FIELD_RHS) for x in pair)) < RHS_TOL
