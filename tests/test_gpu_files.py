"""Files through a context on the GPU (-m gpu): asynchronous PLOT3D solution
saves, loads, grid files, gradient / control-forcing streams and the device
ZAXPY of the gradient-check loop (README.md:118-165, bin/ZAXPY.f90)."""
import numpy as np
import pytest

from helpers import small_monopole
from magudi_gb300 import capi, configs
from magudi_gb300.solver import Solver

pytestmark = pytest.mark.gpu


def test_solution_save_load_round_trip(tmp_path):
    P = configs.two_block_2d()
    s = Solver(P)
    rng = np.random.default_rng(1)
    qs = [configs.random_state(b.n_points, 2, 1.4, rng) for b in P.blocks]
    for bi, q in enumerate(qs, start=1):
        s.set_field(bi, capi.FIELD_CONSERVED, q)
    f = tmp_path / "state.q"
    s.save_solution(f, capi.FIELD_CONSERVED, timestep=7, time=3.25)
    # work issued after the save must not change what is written
    for bi in (1, 2):
        s.set_field(bi, capi.FIELD_CONSERVED, np.ones_like(qs[bi - 1]))
    s.wait_io()
    t = s.load_solution(f, capi.FIELD_CONSERVED)
    assert t == 3.25
    for bi, q in enumerate(qs, start=1):
        assert np.array_equal(s.get_field(bi, capi.FIELD_CONSERVED), q)
    raw = np.fromfile(f, dtype=np.int32, count=10)
    assert list(raw[:3]) == [4, 2, 4]  # record marker, 2 blocks, record marker
    s.save_grid(tmp_path / "grid.xyz")
    assert (tmp_path / "grid.xyz").stat().st_size > 0


def test_gradient_streams_and_device_zaxpy(tmp_path):
    P = small_monopole(n_steps=8, save_interval=4, controller_switch=True)
    s = Solver(P)
    n = 4 * P.n_steps
    s.set_control_forcing(np.zeros((n, s.actuator_points())))
    s.run_forward(P.n_steps, P.save_interval)
    s.run_adjoint()
    g = s.gradient(n)
    prefix = tmp_path / "AcousticMonopole"
    s.save_gradient(prefix, n)
    raw = np.fromfile(str(prefix) + ".gradient_controlRegion.dat", dtype=np.float64).reshape(n, -1)
    assert np.array_equal(raw, g)
    # zaxpy on the device vs the host: forcing = a g, then forcing = a g + forcing
    s.control_zaxpy(1e-3)
    s.set_field(1, capi.FIELD_CONSERVED, P.blocks[0].initial_state)
    J1 = s.run_forward(P.n_steps, P.save_interval)
    t = Solver(P)
    t.set_control_forcing(1e-3 * g)
    assert J1 == t.run_forward(P.n_steps, P.save_interval)
    # the control_forcing stream read back drives the same run
    (1e-3 * g).tofile(str(prefix) + ".control_forcing_controlRegion.dat")
    u = Solver(P)
    u.load_control_forcing(prefix, n)
    assert J1 == u.run_forward(P.n_steps, P.save_interval)
