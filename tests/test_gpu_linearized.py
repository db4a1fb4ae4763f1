"""Linearized (tangent) RHS on the GPU against the oracle (-m gpu):
computeRhsLinearized (src/RhsHelperImpl.f90:598-829) and substepLinearizedRK4
(src/RK4IntegratorImpl.f90:272-380). Per-RHS tolerance 1e-12."""
import numpy as np
import pytest

import oracle_lib
from helpers import rel_err, small_monopole
from magudi_gb300 import capi, configs
from magudi_gb300.solver import Solver

pytestmark = pytest.mark.gpu

RHS_TOL = 1e-12


def _case(P, seed):
    rng = np.random.default_rng(seed)
    q0 = configs.smooth_perturbed_state(P.blocks[0], P.options.n_dimensions, P.options.ratio_of_specific_heats,
                                        rng, amplitude=0.05)
    dq = rng.uniform(-1.0, 1.0, q0.shape) * np.abs(q0).mean(axis=1, keepdims=True)
    lam = rng.uniform(-1.0, 1.0, q0.shape)
    return q0, dq, lam


def _problems():
    P1 = small_monopole(n=33, ny=31, sponge_points=5)
    P2 = small_monopole(n=33, ny=31, sponge_points=5)
    P2.options.viscous = False
    P3 = small_monopole(n=29, ny=31, sponge_points=4)
    P3.options.curvilinear = True
    x, y = P3.blocks[0].coordinates
    P3.blocks[0].coordinates = np.ascontiguousarray(np.stack([x + 0.1 * np.sin(0.4 * y), y + 0.05 * np.sin(0.3 * x)]))
    P4 = configs.taylor_green_3d(n=16)
    P4.options.use_constant_cfl = False
    P4.options.time_step_size = 0.01
    return {"viscous": P1, "inviscid": P2, "curvilinear": P3, "periodic3d": P4}


@pytest.mark.parametrize("name", ["viscous", "inviscid", "curvilinear", "periodic3d"])
def test_linearized_rhs_matches_oracle(name):
    P = _problems()[name]
    q0, dq, _ = _case(P, 3)
    pair = Solver(P), oracle_lib.Oracle(P)
    for s in pair:
        s.set_field(1, capi.FIELD_CONSERVED, q0)
        s.set_field(1, capi.FIELD_ADJOINT, dq)
        s.update_state()
        s.compute_rhs(capi.LINEARIZED, 0.2, 0.0)
    assert rel_err(*(s.get_field(1, capi.FIELD_RHS) for s in pair)) < RHS_TOL


def test_linearized_substeps_match_oracle():
    P = _problems()["viscous"]
    q0, dq, _ = _case(P, 8)
    pair = Solver(P), oracle_lib.Oracle(P)
    times = []
    for s in pair:
        s.set_field(1, capi.FIELD_CONSERVED, q0)
        s.set_field(1, capi.FIELD_ADJOINT, dq)
        s.update_state()
        t = 0.4
        for stage in (1, 2, 3, 4):
            t = s.rk4_substep(capi.LINEARIZED, t, 0.02, stage)
        times.append(t)
    assert times[0] == times[1]
    assert rel_err(*(s.get_field(1, capi.FIELD_ADJOINT) for s in pair)) < RHS_TOL


def test_linearized_rhs_is_the_transpose_of_the_adjoint_rhs_on_the_gpu():
    P = _problems()["viscous"]
    q0, dq, lam = _case(P, 11)
    s = Solver(P)
    s.set_field(1, capi.FIELD_CONSERVED, q0)
    s.update_state()
    H = s.get_field(1, capi.FIELD_NORM)
    s.set_field(1, capi.FIELD_ADJOINT, dq)
    s.compute_rhs(capi.LINEARIZED, 0.3, 0.0)
    a = np.sum(lam * H * s.get_field(1, capi.FIELD_RHS))
    s.set_field(1, capi.FIELD_ADJOINT, lam)
    s.compute_rhs(capi.ADJOINT, 0.3, 0.0)
    b = np.sum(s.get_field(1, capi.FIELD_RHS) * H * dq)
    assert abs(a + b) <= 1e-11 * abs(a)


@pytest.mark.parametrize("wall", ["SAT_SLIP_WALL", "SAT_ISOTHERMAL_WALL", "SAT_ADIABATIC_WALL"])
def test_linearized_rhs_with_walls_matches_oracle(wall):
    P = configs.wall_channel_2d(wall=wall)
    q0, dq, _ = _case(P, 12)
    pair = Solver(P), oracle_lib.Oracle(P)
    for s in pair:
        s.set_field(1, capi.FIELD_CONSERVED, q0)
        s.set_field(1, capi.FIELD_ADJOINT, dq)
        s.update_state()
        s.compute_rhs(capi.LINEARIZED, 0.2, 0.0)
    assert rel_err(*(s.get_field(1, capi.FIELD_RHS) for s in pair)) < RHS_TOL


def _small_jet_without_excitation():
    P = configs.jet_3block_3d(nx=28, ny_core=25, ny_side=26, nz=25, length=4.0, n_steps=4, save_interval=2)
    P.patches = [p for p in P.patches if p.type != "SOLENOIDAL_EXCITATION"]
    return P


@pytest.mark.parametrize("name", ["two_block", "two_block_rotated", "jet3d"])
def test_linearized_rhs_with_block_interfaces_matches_oracle(name):
    if name == "jet3d":
        P = _small_jet_without_excitation()
    else:
        P = configs.two_block_2d(rotate_second=name.endswith("rotated"))
    rng = np.random.default_rng(8)
    states = []
    for b in P.blocks:
        q = configs.smooth_perturbed_state(b, P.options.n_dimensions, 1.4, rng, amplitude=0.05)
        dq = rng.uniform(-1.0, 1.0, q.shape) * np.abs(q).mean(axis=1, keepdims=True)
        states.append((q, dq))
    pair = Solver(P), oracle_lib.Oracle(P)
    for s in pair:
        for bi, (q, dq) in enumerate(states, start=1):
            s.set_field(bi, capi.FIELD_CONSERVED, q)
            s.set_field(bi, capi.FIELD_ADJOINT, dq)
        s.update_state()
        s.compute_rhs(capi.LINEARIZED, 0.2, 0.0)
    for bi in range(1, len(P.blocks) + 1):
        assert rel_err(*(s.get_field(bi, capi.FIELD_RHS) for s in pair)) < RHS_TOL


def test_linearized_rhs_refuses_solenoidal_excitation():
    from helpers import add_solenoidal_excitation
    from magudi_gb300.solver import MagudiError
    P = small_monopole(n=31, ny=29, sponge_points=5)
    add_solenoidal_excitation(P, extent=(4, 26, 3, 25, 1, -1))
    s = Solver(P)
    with pytest.raises(MagudiError):
        s.compute_rhs(capi.LINEARIZED, 0.0, 0.0)


@pytest.mark.parametrize("save_interval", [4, 12])
def test_linearized_run_matches_oracle(save_interval):
    P = small_monopole(n=29, ny=29, n_steps=12, save_interval=save_interval)
    q0, dq, _ = _case(P, 4)
    out = []
    for s in (Solver(P), oracle_lib.Oracle(P)):
        s.set_field(1, capi.FIELD_CONSERVED, q0)
        s.run_forward(P.n_steps, save_interval)
        s.set_field(1, capi.FIELD_ADJOINT, dq)
        s.run_linearized()
        out.append((s.get_field(1, capi.FIELD_ADJOINT), s.get_field(1, capi.FIELD_CONSERVED)))
    assert rel_err(out[0][0], out[1][0]) < 1e-11
    assert rel_err(out[0][1], out[1][1]) < 1e-11


def test_linearized_and_adjoint_runs_are_dual_on_the_gpu():
    P = small_monopole(n=29, ny=29, n_steps=12, save_interval=4)
    P.options.adjoint_forcing_switch = False
    q0, dq, lamT = _case(P, 6)
    s = Solver(P)
    s.set_field(1, capi.FIELD_CONSERVED, q0)
    s.run_forward(P.n_steps, 4)
    H = s.get_field(1, capi.FIELD_NORM)
    s.set_field(1, capi.FIELD_ADJOINT, dq)
    s.run_linearized()
    b = np.sum(lamT * H * s.get_field(1, capi.FIELD_ADJOINT))
    s.set_field(1, capi.FIELD_ADJOINT, lamT)
    s.set_adjoint_nonzero_initial_condition(True)
    s.run_adjoint()
    a = np.sum(s.get_field(1, capi.FIELD_ADJOINT) * H * dq)
    assert abs(a - b) <= 1e-11 * abs(b)
