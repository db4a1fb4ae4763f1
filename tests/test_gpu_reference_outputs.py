"""The GPU path against numbers the reference's own Fortran build printed
(-m gpu): the TestForcing example of test_reference_outputs.py through the C
ABI, with the reference's own files read by the library's readers (the
initial condition by mgd_load_solution, the baseline control forcing by
mgd_load_control_forcing) and the gradient-accuracy loop's control forcing
A x gradient + baseline formed on the device (mgd_control_zaxpy, the
reference's ./zaxpy). Every cost J(A) the reference printed matches to
1e-12, the adjoint sensitivity to 2e-10, and both match the oracle."""
import os
import shutil

import numpy as np
import pytest

import oracle_lib
from magudi_gb300 import capi
from magudi_gb300.solver import Solver
from test_reference_outputs import (COST_TOL, HERE, N_STEPS, SENSITIVITY_TOL, baseline_forcing, forcing_problem,
                                    reference_outputs)

pytestmark = pytest.mark.gpu


def test_gpu_costs_and_sensitivity_match_the_reference_build(tmp_path):
    P = forcing_problem()
    ref = reference_outputs()
    s = Solver(P)
    # the reference's initial-condition file, read by the library
    s.load_solution(os.path.join(HERE, "TestForcing.ic.q"))
    assert np.array_equal(s.get_field(1, capi.FIELD_CONSERVED), P.blocks[0].initial_state)
    # the reference's baseline control forcing file, read by the library
    prefix = str(tmp_path / "TestForcing")
    shutil.copyfile(os.path.join(HERE, "baseline.dat"), prefix + ".control_forcing_controlRegion.dat")
    s.load_control_forcing(prefix, 4 * N_STEPS)
    s.run_forward(N_STEPS, N_STEPS)
    G = s.run_adjoint()
    assert abs(G - ref["printed_sensitivity"]) <= SENSITIVITY_TOL * abs(ref["printed_sensitivity"])
    o = oracle_lib.Oracle(P)
    o.set_control_forcing(baseline_forcing())
    o.run_forward(N_STEPS, N_STEPS)
    assert abs(G - o.run_adjoint()) <= 1e-12 * abs(G)
    for A, J_ref in zip(ref["amplitudes"], ref["costs"]):
        s.load_control_forcing(prefix, 4 * N_STEPS)
        s.control_zaxpy(A, accumulate=True)
        s.load_solution(os.path.join(HERE, "TestForcing.ic.q"))
        J = s.run_forward(N_STEPS, N_STEPS)
        assert s.limit_violation is None
        assert abs(J - J_ref) <= COST_TOL * J_ref, (A, J, J_ref)
