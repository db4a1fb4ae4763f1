"""Both forms of the 2D gradient/flux kernel and of the 2D adjoint core
against the oracle (-m gpu): one thread per point, and one thread per point
and axis (gradient/flux: results swapped by shuffle; adjoint core: shares
summed in shared memory). The tuners keep the faster forms;
mgd_gradient_lanes and mgd_adjoint_core_lanes set them, so every form is
checked here on every path that launches the kernels: forward and adjoint RHS
(curvilinear grid, walls, block interfaces), checkpointed forward + adjoint
runs with the concurrent recomputation, and the tangent run."""
import numpy as np
import pytest

import oracle_lib
from helpers import random_full_rhs_state, rel_err, small_monopole
from magudi_gb300 import capi, configs
from magudi_gb300.solver import MagudiError, Solver

pytestmark = pytest.mark.gpu

# (gradient/flux threads per point, adjoint core threads per point)
LANES = [(1, 1), (2, 1), (1, 2)]


def _gpu(P, lanes):
    s = Solver(P)
    assert s.gradient_lanes() in (1, 2) and s.adjoint_core_lanes() in (1, 2)
    assert s.gradient_lanes(lanes[0]) == lanes[0]
    assert s.adjoint_core_lanes(lanes[1]) == lanes[1]
    return s


def _rhs_pair(g, o, nblocks, q, lam):
    for s in (g, o):
        for bi in range(1, nblocks + 1):
            s.set_field(bi, capi.FIELD_CONSERVED, q[bi - 1])
            s.set_field(bi, capi.FIELD_ADJOINT, lam[bi - 1])
        s.update_state()
        s.compute_rhs(capi.FORWARD, 0.3)
    for bi in range(1, nblocks + 1):
        assert rel_err(g.get_field(bi, capi.FIELD_RHS), o.get_field(bi, capi.FIELD_RHS)) < 1e-12
    for s in (g, o):
        s.compute_rhs(capi.ADJOINT, 0.0, 1.0)
    for bi in range(1, nblocks + 1):
        assert rel_err(g.get_field(bi, capi.FIELD_RHS), o.get_field(bi, capi.FIELD_RHS)) < 1e-12


def test_lanes_argument_is_checked():
    s = Solver(small_monopole())
    with pytest.raises(MagudiError):
        s.gradient_lanes(3)
    with pytest.raises(MagudiError):
        s.adjoint_core_lanes(-1)


@pytest.mark.parametrize("lanes", LANES)
def test_curvilinear_far_field_rhs(lanes):
    P = small_monopole()
    P.options.curvilinear = True
    blk = P.blocks[0]
    x, y = blk.coordinates
    blk.coordinates = np.ascontiguousarray(np.stack([x + 0.1 * np.sin(0.4 * y), y + 0.05 * np.sin(0.3 * x)]))
    q, lam = random_full_rhs_state(P, 13)
    _rhs_pair(_gpu(P, lanes), oracle_lib.Oracle(P), 1, [q], [lam])


@pytest.mark.parametrize("lanes", LANES)
@pytest.mark.parametrize("wall", ["SAT_ISOTHERMAL_WALL", "SAT_SLIP_WALL"])
def test_wall_rhs(lanes, wall):
    P = configs.wall_channel_2d(wall=wall, wall_temperature=2.0)
    q, lam = random_full_rhs_state(P, 17)
    _rhs_pair(_gpu(P, lanes), oracle_lib.Oracle(P), 1, [q], [lam])


@pytest.mark.parametrize("lanes", LANES)
def test_two_block_interface_rhs(lanes):
    P = configs.two_block_2d(rotate_second=True, viscous=True)
    rng = np.random.default_rng(41)
    g_ = P.options.ratio_of_specific_heats
    qs = [configs.random_state(b.n_points, 2, g_, rng) for b in P.blocks]
    lams = [rng.uniform(0.0, 1.0, (4, b.n_points)) for b in P.blocks]
    _rhs_pair(_gpu(P, lanes), oracle_lib.Oracle(P), 2, qs, lams)


@pytest.mark.parametrize("lanes", LANES)
def test_gradient_run(lanes):
    """Forward + adjoint with checkpoint recomputation into full stage slots
    (the recomputation stores stress and heat flux from this kernel)."""
    P = small_monopole(n_steps=30, save_interval=7)
    g, o = _gpu(P, lanes), oracle_lib.Oracle(P)
    Jg, Jo = g.run_forward(P.n_steps, P.save_interval), o.run_forward(P.n_steps, P.save_interval)
    assert abs(Jg - Jo) <= 1e-10 * abs(Jo)
    Gg, Go = g.run_adjoint(), o.run_adjoint()
    assert abs(Gg - Go) <= 1e-10 * abs(Go)
    n = 4 * P.n_steps
    assert rel_err(g.gradient(n), o.gradient(n)) < 1e-10


@pytest.mark.parametrize("lanes", LANES)
def test_tangent_run(lanes):
    P = small_monopole(n_steps=12, save_interval=5)
    g, o = _gpu(P, lanes), oracle_lib.Oracle(P)
    rng = np.random.default_rng(8)
    df = rng.standard_normal((4 * P.n_steps, g.actuator_points()))
    dJ = []
    for s in (g, o):
        s.run_forward(P.n_steps, P.save_interval)
        s.set_field(1, capi.FIELD_ADJOINT, np.zeros((4, P.blocks[0].n_points)))
        dJ.append(s.run_linearized(df))
    assert abs(dJ[0] - dJ[1]) <= 1e-10 * abs(dJ[1])
    assert rel_err(g.get_field(1, capi.FIELD_ADJOINT), o.get_field(1, capi.FIELD_ADJOINT)) < 1e-10


def test_run_level_tuning_restores_the_state_and_keeps_parity():
    """mgd_tune_run times short checkpointed runs under other tiles: the state
    and adjoint fields come back unchanged, and the runs after it (on the tiles
    it chose) still match the oracle."""
    P = small_monopole(n_steps=24, save_interval=6)
    g, o = Solver(P), oracle_lib.Oracle(P)
    q0 = g.get_field(1, capi.FIELD_CONSERVED).copy()
    lam0 = np.random.default_rng(2).standard_normal((4, P.blocks[0].n_points))
    g.set_field(1, capi.FIELD_ADJOINT, lam0)
    ms = g.tune_run(8, 4)
    assert ms > 0.0
    assert np.array_equal(g.get_field(1, capi.FIELD_CONSERVED), q0)
    assert np.array_equal(g.get_field(1, capi.FIELD_ADJOINT), lam0)
    assert all(len(g.stage_tile(k)) == 3 for k in range(6))
    with pytest.raises(MagudiError):
        g.run_adjoint()  # the tuning runs leave no trajectory
    Jg, Jo = g.run_forward(P.n_steps, P.save_interval), o.run_forward(P.n_steps, P.save_interval)
    assert abs(Jg - Jo) <= 1e-10 * abs(Jo)
    Gg, Go = g.run_adjoint(), o.run_adjoint()
    assert abs(Gg - Go) <= 1e-10 * abs(Go)
    n = 4 * P.n_steps
    assert rel_err(g.gradient(n), o.gradient(n)) < 1e-10
    # a later context of the same grid starts from the tuned tiles
    g2 = Solver(P)
    assert [g2.stage_tile(k) for k in range(6)] == [g.stage_tile(k) for k in range(6)]
    assert g2.gradient_lanes() == g.gradient_lanes()
    assert g2.adjoint_core_lanes() == g.adjoint_core_lanes()


def test_stage_tile_hook_checks_its_arguments():
    s = Solver(small_monopole())
    with pytest.raises(MagudiError):
        s.stage_tile(6)
    with pytest.raises(MagudiError):
        s.stage_tile(0, (32, 16, 1))  # 512 threads
    assert s.stage_tile(2, (16, 8, 1)) == (16, 8, 1)


@pytest.mark.parametrize("tile", [(12, 10, 1), (7, 9, 1)])
def test_tiles_that_are_not_powers_of_two(tile):
    """Tiles of any shape: the kernels split CTA indices with reciprocals of
    the tile's extents, exact for any divisor."""
    P = small_monopole(n_steps=12, save_interval=5)
    g, o = Solver(P), oracle_lib.Oracle(P)
    for k in range(6):
        assert g.stage_tile(k, tile) == tile
    q, lam = random_full_rhs_state(P, 23)
    _rhs_pair(g, o, 1, [q], [lam])
    for s in (g, o):
        s.set_field(1, capi.FIELD_CONSERVED, P.blocks[0].initial_state)
    Jg, Jo = g.run_forward(P.n_steps, P.save_interval), o.run_forward(P.n_steps, P.save_interval)
    assert abs(Jg - Jo) <= 1e-10 * abs(Jo)
    Gg, Go = g.run_adjoint(), o.run_adjoint()
    assert abs(Gg - Go) <= 1e-10 * abs(Go)
