"""The oracle against numbers the reference's own Fortran build printed.

The reference's TestForcing example (tests/golden/test_forcing, written by
make_test_forcing_golden.py from the example's files and its notebook's cell
outputs): a 4 x 4 PLANE-periodic grid whose coordinate file repeats the end
point (config.py's linspace(0, 1, 4)), SBP 2-4, non-composite dissipation
1e-4, viscous (Re 200, Pr 0.7, constant viscosity), a thermal actuator and
the sound functional over the whole grid, 8 RK4 steps of 0.05 from the
example's initial condition, with the baseline control forcing of
baseline.dat. The reference's gradient-accuracy loop ran ./zaxpy (control
forcing = A x gradient + baseline) and ./forward for 32 amplitudes A and
printed each cost functional J(A) in full precision: the oracle's J(A),
with the gradient of its own adjoint run, matches every one of them to
1e-12 (the observed differences are 1e-13 and below). The notebook's
printed QoI0 is the cost of the loop's last forcing (its cells ran out of
order; J(A_32) - QoI0 is exactly zero in its table), and its printed Grad0,
the adjoint sensitivity, agrees with the oracle's to 2e-10.
"""
import json
import os

import numpy as np

import oracle_lib
from magudi_gb300 import capi
from magudi_gb300.inputs import problem_from_inputs
from magudi_gb300.problem import Block

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "test_forcing")
N_STEPS = 8
COST_TOL = 1e-12
SENSITIVITY_TOL = 2e-10


def forcing_problem():
    """The example as its magudi.inp and bc.dat (unchanged) and fields.npz
    describe it. The mean pressure of the sound functional is the target
    state's pressure (AcousticNoise setup with use_target_state and no
    mean_pressure_file, src/AcousticNoiseImpl.f90:61-73); the target state is
    the quiescent one (src/SolverImpl.f90:509-520)."""
    f = np.load(os.path.join(HERE, "fields.npz"))
    blk = Block(grid_size=tuple(int(x) for x in f["grid_size"]), coordinates=np.ascontiguousarray(f["coordinates"]),
                initial_state=np.ascontiguousarray(f["initial_state"]),
                control_mollifier=np.ascontiguousarray(f["control_mollifier"]),
                target_mollifier=np.ascontiguousarray(f["target_mollifier"]))
    P = problem_from_inputs(os.path.join(HERE, "magudi.inp"), os.path.join(HERE, "bc.dat"), [blk])
    g = P.options.ratio_of_specific_heats
    t = P.blocks[0].target_state
    P.blocks[0].mean_pressure = (g - 1.0) * (t[3] - 0.5 * (t[1] ** 2 + t[2] ** 2) / t[0])
    return P


def baseline_forcing():
    return np.fromfile(os.path.join(HERE, "baseline.dat"), dtype="<f8")


def reference_outputs():
    return json.load(open(os.path.join(HERE, "reference_outputs.json")))


def test_the_example_parses_as_the_reference_ran_it():
    P = forcing_problem()
    o = P.options
    assert o.discretization_scheme == capi.SBP_24
    assert o.viscous and not o.use_constant_cfl and o.enable_controller and o.controller_switch
    assert o.dissipation and not o.composite_dissipation and o.dissipation_amount == 1e-4
    assert P.n_steps == N_STEPS and P.save_interval == N_STEPS and o.time_step_size == 0.05
    assert P.blocks[0].periodicity_type[:2] == (1, 1) and P.blocks[0].periodic_length[:2] == (1.0, 1.0)
    assert baseline_forcing().size == 4 * N_STEPS * 16


def test_oracle_costs_and_sensitivity_match_the_reference_build():
    P = forcing_problem()
    ref = reference_outputs()
    base = baseline_forcing()
    o = oracle_lib.Oracle(P)
    o.set_control_forcing(base)
    o.run_forward(N_STEPS, N_STEPS)
    G = o.run_adjoint()
    grad = o.gradient(4 * N_STEPS).ravel()
    costs = []
    for A, J_ref in zip(ref["amplitudes"], ref["costs"]):
        o2 = oracle_lib.Oracle(P)
        o2.set_control_forcing(A * grad + base)
        J = o2.run_forward(N_STEPS, N_STEPS)
        assert o2.run_status == 0
        assert abs(J - J_ref) <= COST_TOL * J_ref, (A, J, J_ref)
        costs.append(J)
    assert float(f"{costs[-1]:.12g}") == ref["printed_cost"]
    assert abs(G - ref["printed_sensitivity"]) <= SENSITIVITY_TOL * abs(ref["printed_sensitivity"])
