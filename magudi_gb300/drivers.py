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


def per_call_gradient(s, problem, n_steps, save_interval):
    """J and the gradient norm (sensitivity) of n_steps constant-dt steps from
    the problem's initial state, checkpoints every save_interval steps."""
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
                tl = s.rk4_substep(capi.FORWARD, tl, dt, i)
        for step in range(end, L, -1):
            for i in range(4, 0, -1):
                s.set_field(1, capi.FIELD_CONSERVED, stages[(step, i)])
                s.update_state()
                G += RK_NORM[i - 1] * dt * s.sensitivity()
                s.update_adjoint_forcing(step == 1 and i == 1)
                t = s.rk4_substep(capi.ADJOINT, t, dt, i)
    return J, G
