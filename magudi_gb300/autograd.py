"""torch.autograd.Function front end of the forward run and its discrete adjoint.

J(f) is the time-integrated cost functional of a forward run (Solver%runForward,
src/SolverImpl.f90:672-912) driven by the control forcing f, one row of
actuator-patch values per RK4 stage in the reference's file order (rows count
backwards from the last stage, src/ThermalActuatorImpl.f90:161-233). The
backward pass is the hand-written discrete adjoint run (Solver%runAdjoint,
src/SolverImpl.f90:914-1245, with UniformCheckpointer recomputation from
device snapshots). magudi's gradient file holds g = lambda_E * m_c per stage
(src/ThermalActuatorImpl.f90:383-443) and its sensitivity is the weighted
inner product sum_e w_e dt H det g_e^2 (:83-159), so the Euclidean gradient of
J with respect to the forcing entries is dJ/df[e, i] = w_s(e) dt_n(e) W_i g[e, i],
with w = (1/6, 1/3, 1/3, 1/6) the RK4 stage weights and W_i the actuator-point
quadrature weights. Everything runs through the C ABI; forcing and gradient
stay in device memory when the tensors are CUDA tensors.
"""
import ctypes as C

import numpy as np
import torch

from . import capi
from .solver import Solver

RK_NORM = (1.0 / 6.0, 1.0 / 3.0, 1.0 / 3.0, 1.0 / 6.0)


def _ptr(t):
    return C.cast(t.data_ptr(), C.POINTER(C.c_double))


class ForwardRun(torch.autograd.Function):
    """J = ForwardRun.apply(forcing, solver, n_steps, save_interval).

    forcing: float64 tensor (4 * n_steps, P) on the CPU or the solver's GPU.
    Each call restarts the run from the problem's initial state. With
    solver.set_trajectory_storage(True) the forward run keeps every stage on
    the device and backward() reads it instead of recomputing checkpoint
    segments (same gradient)."""

    @staticmethod
    def forward(ctx, forcing, solver, n_steps, save_interval):
        if forcing.dtype != torch.float64:
            raise TypeError("the control forcing is FP64")
        if not (solver.problem.options.enable_controller and solver.problem.options.controller_switch):
            raise ValueError("the problem must enable the controller (enable_controller, controller_switch)")
        P = solver.actuator_points()
        if forcing.shape != (4 * n_steps, P):
            raise ValueError(f"forcing must have shape {(4 * n_steps, P)}")
        f = forcing.detach().contiguous()
        solver.set_field(1, capi.FIELD_CONSERVED, solver.problem.blocks[0].initial_state)
        solver._check(solver.L.mgd_set_control_forcing(solver.h, _ptr(f), 4 * n_steps))
        J = solver.run_forward(n_steps, save_interval)
        ctx.solver, ctx.n_steps, ctx.device = solver, n_steps, forcing.device
        return torch.tensor(J, dtype=torch.float64, device=forcing.device)

    @staticmethod
    def backward(ctx, grad_J):
        s, n = ctx.solver, ctx.n_steps
        s.run_adjoint()
        g = torch.empty((4 * n, s.actuator_points()), dtype=torch.float64, device=ctx.device)
        s._check(s.L.mgd_get_gradient(s.h, _ptr(g), 4 * n))
        w = torch.from_numpy(quadrature_weights(s, n)).to(ctx.device)
        return grad_J * w * g, None, None, None


    @staticmethod
    def jvp(ctx, forcing_t, solver_t, n_t, s_t):
        """Forward mode: the tangent run (Solver%runLinearized) along the
        control perturbation forcing_t from a zero initial perturbation, on the
        checkpoints of this forward run; returns dJ = <dJ/df, forcing_t>."""
        s, n = ctx.solver, ctx.n_steps
        if forcing_t is None:
            return torch.zeros((), dtype=torch.float64, device=ctx.device)
        s.set_field(1, capi.FIELD_ADJOINT, np.zeros((s.nU, s.problem.blocks[0].n_points)))
        ft = forcing_t.detach().to(torch.float64).contiguous()
        v = C.c_double()
        s._check(s.L.mgd_run_linearized(s.h, _ptr(ft), 4 * n, C.byref(v)))
        return torch.tensor(v.value, dtype=torch.float64, device=ctx.device)


def quadrature_weights(solver, n_steps):
    """w_s(e) dt_n(e) W_i for every forcing entry e (rows) and actuator point i."""
    P = solver.actuator_points()
    W = np.zeros(P)
    if P:
        solver._check(solver.L.mgd_actuator_weights(solver.h, capi.dptr(W)))
    dts = solver.step_sizes(n_steps)
    rows = np.empty(4 * n_steps)
    for e in range(4 * n_steps):
        step = n_steps - e // 4          # 1-based forward step of entry e
        stage = 4 - e % 4                # RK4 stage of entry e
        rows[e] = RK_NORM[stage - 1] * dts[step - 1]
    return rows[:, None] * W[None, :]


def cost(problem, forcing, n_steps=None, save_interval=None, solver=None):
    """J(forcing) as a differentiable scalar; builds a Solver if none is given."""
    solver = solver or Solver(problem)
    n_steps = n_steps or problem.n_steps
    save_interval = save_interval or problem.save_interval
    return ForwardRun.apply(forcing, solver, n_steps, save_interval)
