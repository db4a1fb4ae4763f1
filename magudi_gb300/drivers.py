"""The reference's solver loop over the per-call entry points.

per_call_gradient runs Solver%runForward and Solver%runAdjoint with
UniformCheckpointer (src/SolverImpl.f90:672-1245,
src/UniformCheckpointerImpl.f90:80-208) through mgd_rk4_substep,
mgd_compute_functional, mgd_update_adjoint_forcing and
mgd_compute_sensitivity only, one call per stage, with the checkpoints and each
segment's stage states in host memory as the reference keeps them. It is the
control flow of a host that drives the library only at the computeRhs seam,
and it gives the same J and gradient norm as mgd_run_forward / mgd_run_adjoint.
Any object with those methods serves (the Solver, or the oracle in tests).
"""
import numpy as np

from . import capi

RK_NORM = (1.0 / 6.0, 1.0 / 3.0, 1.0 / 3.0, 1.0 / 6.0)


def per_call_gradient(s, problem, n_steps, save_interval, forcing=None):
    """J and the gradient norm (sensitivity) of n_steps constant-dt steps from
    the problem's initial state, checkpoints every save_interval steps. With
    forcing (4 n_steps entries x actuator points, file order), the stage's
    entry is handed to the actuators before each forward substep, as the
    controller's updateForcing does (src/ThermalActuatorImpl.f90:161-233)."""
    dt = problem.options.time_step_size
    N, nU = problem.blocks[0].n_points, problem.n_unknowns
    s.set_field(1, capi.FIELD_CONSERVED, problem.blocks[0].initial_state)
    s.update_state()
    t, J = 0.0, 0.0
    snaps = {}
    for step in range(1, n_steps + 1):
        if (step - 1) % save_interval == 0:
            snaps[step - 1] = (s.get_field(1, capi.FIELD_CONSERVED), t)
        for i in range(1, 5):
            if forcing is not None:
                s.set_patch_control_forcing(forcing[(n_steps - step) * 4 + (4 - i)])
            t = s.rk4_substep(capi.FORWARD, t, dt, i)
            J += RK_NORM[i - 1] * dt * s.functional()
    # loadInitialCondition(ADJOINT): lambda(T) = (-dt/6) x the cost-target forcing at T
    s.update_adjoint_forcing(False)
    s.set_field(1, capi.FIELD_ADJOINT, np.zeros((nU, N)))
    s.compute_rhs(capi.ADJOINT, t, -dt / 6.0)
    s.set_field(1, capi.FIELD_ADJOINT, s.get_field(1, capi.FIELD_RHS))
    G = 0.0
    for L in range(((n_steps - 1) // save_interval) * save_interval, -1, -save_interval):
        end = min(n_steps, L + save_interval)
        q, tl = snaps[L]
        s.set_field(1, capi.FIELD_CONSERVED, q)
        s.update_state()
        stages = {}
        for step in range(L + 1, end + 1):
            for i in range(1, 5):
                stages[(step, i)] = s.get_field(1, capi.FIELD_CONSERVED)
                if forcing is not None:
                    s.set_patch_control_forcing(forcing[(n_steps - step) * 4 + (4 - i)])
                tl = s.rk4_substep(capi.FORWARD, tl, dt, i)
        for step in range(end, L, -1):
            for i in range(4, 0, -1):
                s.set_field(1, capi.FIELD_CONSERVED, stages[(step, i)])
                s.update_state()
                G += RK_NORM[i - 1] * dt * s.sensitivity()
                s.update_adjoint_forcing(step == 1 and i == 1)
                t = s.rk4_substep(capi.ADJOINT, t, dt, i)
    if forcing is not None:
        s.set_patch_control_forcing(None)
    return J, G


def per_call_forward(s, problem, n_steps, forcing=None):
    """J of n_steps constant-dt forward steps through mgd_rk4_substep and the
    functional, one call per stage (Solver%runForward, src/SolverImpl.f90:672-912),
    handing each stage's forcing entry to the actuators when forcing is given."""
    dt = problem.options.time_step_size
    s.set_field(1, capi.FIELD_CONSERVED, problem.blocks[0].initial_state)
    s.update_state()
    t, J = 0.0, 0.0
    for step in range(1, n_steps + 1):
        for i in range(1, 5):
            if forcing is not None:
                s.set_patch_control_forcing(forcing[(n_steps - step) * 4 + (4 - i)])
            t = s.rk4_substep(capi.FORWARD, t, dt, i)
            J += RK_NORM[i - 1] * dt * s.functional()
    if forcing is not None:
        s.set_patch_control_forcing(None)
    return J
