"""Block sizes at the edge of what the stencils allow (-m gpu): the smallest
accepted grid in each periodicity runs its forward and adjoint RHS to the
oracle's results, and one point fewer is refused with an error before
anything is allocated. A periodic tap i +- 4 wraps once, so PLANE needs 4
points and OVERLAP (period n - 1) 5; a non-periodic direction needs the
25 points of the operators' closure windows."""
import numpy as np
import pytest

import oracle_lib
from helpers import annulus_o_grid, rel_err, small_monopole
from magudi_gb300 import capi, configs
from magudi_gb300.solver import MagudiError, Solver

pytestmark = pytest.mark.gpu

RHS_TOL = 1e-12


def _periodic(n, periodicity):
    """PLANE: a Taylor-Green box of n^3 points; OVERLAP: a 2D O-grid of n
    points around an annulus (the periodic coordinates repeat their first
    point, so the grid must close on itself)."""
    if periodicity == capi.PERIODIC_OVERLAP:
        return annulus_o_grid(n_theta=n)
    return configs.taylor_green_3d(n=n, dt=0.01)


def _rhs_parity(P, seed):
    rng = np.random.default_rng(seed)
    N = P.blocks[0].n_points
    nD = P.options.n_dimensions
    q = configs.random_state(N, nD, P.options.ratio_of_specific_heats, rng)
    lam = rng.uniform(0.0, 1.0, (nD + 2, N))
    g, o = Solver(P), oracle_lib.Oracle(P)
    for s in (g, o):
        s.set_field(1, capi.FIELD_CONSERVED, q)
        s.set_field(1, capi.FIELD_ADJOINT, lam)
        s.update_state()
        s.compute_rhs(capi.FORWARD, 0.2)
    assert rel_err(g.get_field(1, capi.FIELD_RHS), o.get_field(1, capi.FIELD_RHS)) < RHS_TOL
    for s in (g, o):
        s.compute_rhs(capi.ADJOINT, 0.0, 1.0)
    assert rel_err(g.get_field(1, capi.FIELD_RHS), o.get_field(1, capi.FIELD_RHS)) < RHS_TOL


@pytest.mark.parametrize("periodicity, n", [(capi.PERIODIC_PLANE, 4), (capi.PERIODIC_OVERLAP, 5)])
def test_smallest_periodic_block_matches_oracle(periodicity, n):
    _rhs_parity(_periodic(n, periodicity), seed=n)


@pytest.mark.parametrize("n_theta", [5, 33])
def test_o_grid_overlap_run_matches_oracle(n_theta):
    """Forward run, terminal kinetic energy and adjoint run on the O-grid,
    with the checkpoint recomputation (6 steps, snapshots every 3)."""
    P = annulus_o_grid(n_theta=n_theta)
    g, o = Solver(P), oracle_lib.Oracle(P)
    Jg = g.run_forward(P.n_steps, P.save_interval)
    Jo = o.run_forward(P.n_steps, P.save_interval)
    assert abs(Jg - Jo) <= 1e-12 * abs(Jo)
    g.run_adjoint()
    o.run_adjoint()
    assert rel_err(g.get_field(1, capi.FIELD_ADJOINT), o.get_field(1, capi.FIELD_ADJOINT)) < 1e-10


def test_smallest_non_periodic_block_matches_oracle():
    _rhs_parity(small_monopole(n=25, ny=25, sponge_points=4), seed=3)


@pytest.mark.parametrize("periodicity, n", [(capi.PERIODIC_PLANE, 3), (capi.PERIODIC_OVERLAP, 4)])
def test_too_small_periodic_block_is_refused(periodicity, n):
    P = _periodic(n, periodicity)
    with pytest.raises(MagudiError, match="periodic direction needs at least"):
        Solver(P)
    with pytest.raises(RuntimeError, match="periodic direction needs at least"):
        oracle_lib.Oracle(P)


def test_too_small_non_periodic_block_is_refused():
    with pytest.raises(MagudiError, match="at least 25 points"):
        Solver(small_monopole(n=24, ny=25, sponge_points=4))


def test_unknown_periodicity_is_refused():
    P = configs.taylor_green_3d(n=8, dt=0.01)
    P.blocks[0].periodicity_type = (1, 3, 1)
    with pytest.raises(MagudiError, match="periodicity_type"):
        Solver(P)
