"""The forward run / discrete adjoint as a torch.autograd.Function (-m gpu):
the backward pass against central finite differences of J and against the
oracle's adjoint gradient, with the forcing on the GPU and on the host."""
import numpy as np
import pytest
import torch

import oracle_lib
from helpers import small_monopole
from magudi_gb300.autograd import ForwardRun, quadrature_weights
from magudi_gb300.solver import Solver

pytestmark = pytest.mark.gpu

N_STEPS, S = 16, 4


def _problem():
    return small_monopole(n_steps=N_STEPS, save_interval=S, controller_switch=True)


@pytest.mark.parametrize("device", ["cuda", "cpu"])
def test_backward_matches_finite_differences(device):
    P = _problem()
    s = Solver(P)
    n_act = s.actuator_points()
    rng = np.random.default_rng(3)
    f0 = torch.tensor(1e-3 * rng.standard_normal((4 * N_STEPS, n_act)), dtype=torch.float64, device=device,
                      requires_grad=True)
    J = ForwardRun.apply(f0, s, N_STEPS, S)
    J.backward()
    grad = f0.grad.clone()
    d = grad / grad.norm()
    eps = 1e-2 * float(f0.detach().abs().max())
    with torch.no_grad():
        Jp = ForwardRun.apply(f0 + eps * d, s, N_STEPS, S)
        Jm = ForwardRun.apply(f0 - eps * d, s, N_STEPS, S)
    fd = float((Jp - Jm) / (2 * eps))
    an = float((grad * d).sum())
    assert abs(fd - an) <= 1e-6 * abs(an)


def test_backward_matches_oracle_gradient():
    P = _problem()
    s = Solver(P)
    n_act = s.actuator_points()
    rng = np.random.default_rng(8)
    f = 1e-3 * rng.standard_normal((4 * N_STEPS, n_act))
    ft = torch.tensor(f, dtype=torch.float64, device="cuda", requires_grad=True)
    J = ForwardRun.apply(ft, s, N_STEPS, S)
    J.backward()
    o = oracle_lib.Oracle(P)
    o.set_control_forcing(f)
    Jo = o.run_forward(N_STEPS, S)
    o.run_adjoint()
    go = o.gradient(4 * N_STEPS) * quadrature_weights(s, N_STEPS)
    assert abs(J.item() - Jo) <= 1e-10 * abs(Jo)
    g = ft.grad.cpu().numpy()
    assert np.linalg.norm(g - go) <= 1e-10 * np.linalg.norm(go)


@pytest.mark.parametrize("device", ["cuda", "cpu"])
def test_forward_mode_jvp_matches_the_adjoint_gradient(device):
    """torch forward-mode AD through the tangent run: <dJ/df, t> from the jvp
    equals the same inner product from the backward (adjoint) gradient, and
    the oracle's tangent run gives the same value."""
    import torch.autograd.forward_ad as fwAD
    P = _problem()
    s = Solver(P)
    n_act = s.actuator_points()
    rng = np.random.default_rng(5)
    f0 = torch.tensor(1e-3 * rng.standard_normal((4 * N_STEPS, n_act)), dtype=torch.float64, device=device)
    t = torch.tensor(rng.standard_normal((4 * N_STEPS, n_act)), dtype=torch.float64, device=device)
    with fwAD.dual_level():
        J = ForwardRun.apply(fwAD.make_dual(f0, t), s, N_STEPS, S)
        jvp = float(fwAD.unpack_dual(J).tangent)
    f1 = f0.clone().requires_grad_(True)
    ForwardRun.apply(f1, s, N_STEPS, S).backward()
    vjp = float((f1.grad * t).sum())
    assert abs(jvp - vjp) <= 1e-10 * abs(vjp)
    o = oracle_lib.Oracle(P)
    o.set_control_forcing(f0.cpu().numpy())
    o.run_forward(N_STEPS, S)
    o.set_field(1, 1, np.zeros((4, P.blocks[0].n_points)))
    dJ = o.run_linearized(t.cpu().numpy())
    assert abs(jvp - dJ) <= 1e-10 * abs(dJ)
