"""The CPU oracle against the reference's golden vectors and property tests
(CPU only). These pin the oracle before the GPU tests compare against it:

- SBP 4-8 first derivative vs the reference's own Python implementation
  (tests/golden/sbp48_first_derivative.npz, made by make_sbp_golden.py);
- SBP identity H D + (H D)^T = diag(-1, 0, ..., 0, 1) (test/SBP_property.f90:108-109);
- interior order 8 / boundary order 4 (test/operator_convergence.f90:86-130);
- adjoint operator: <A x, y>_H = <x, D y>_H (getAdjointOperator);
- dissipation self-adjointness (test/dissipation_self_adjoint.f90);
- full-RHS dual consistency, FD order >= 0.9 (test/adjoint_relation/full_rhs.f90:220-454);
- gradient finite-difference sweep J(eps) (README gradient-accuracy procedure).
"""
import os

import numpy as np
import pytest

import oracle_lib
from helpers import fd_order, random_full_rhs_state, small_monopole
from magudi_gb300 import capi, configs

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "sbp48_first_derivative.npz")


def dense(which, n):
    """Dense matrix of operator `which` on a non-periodic line of n points."""
    M = np.zeros((n, n))
    for k in range(n):
        e = np.zeros((1, n))
        e[0, k] = 1.0
        M[:, k] = oracle_lib.apply_operator(which, e, (n, 1, 1), 0)[0]
    return M


def norm_diag(n):
    _, _, _, h = oracle_lib.operator(0)
    H = np.ones(n)
    H[: len(h)] = h
    H[n - len(h):] = h[::-1]
    return H


def test_first_derivative_matches_reference_python():
    g = np.load(GOLDEN)
    for n in (24, 37, 64):
        x, d = g[f"x_{n}"], g[f"dx_{n}"]
        y = oracle_lib.apply_operator(0, x.T.copy(), (n, 1, 1), 0)
        assert np.max(np.abs(y - d.T)) <= 1e-14 * max(1.0, np.max(np.abs(d)))
    y = oracle_lib.apply_operator(0, g["x_sin"].T.copy(), (50, 1, 1), 0)
    assert np.max(np.abs(y - g["dx_sin"].T)) <= 1e-15


@pytest.mark.parametrize("n", [25, 40, 57])
def test_sbp_identity(n):
    D = dense(0, n)
    H = np.diag(norm_diag(n))
    Q = H @ D
    B = np.zeros((n, n))
    B[0, 0], B[-1, -1] = -1.0, 1.0
    assert np.max(np.abs(Q + Q.T - B)) < 10 * np.finfo(float).eps * n


def test_convergence_order():
    errs_int, errs_bnd, hs = [], [], []
    w = 10.0
    for n in (41, 61, 81, 121):
        x = np.linspace(0.0, 1.0, n)
        h = x[1] - x[0]
        f = np.sin(w * x + 0.3)
        d = oracle_lib.apply_operator(0, f[None, :], (n, 1, 1), 0)[0] / h
        e = np.abs(d - w * np.cos(w * x + 0.3))
        errs_int.append(e[12:-12].max())
        errs_bnd.append(e[:8].max())
        hs.append(h)
    o_int = fd_order(hs, errs_int)
    o_bnd = fd_order(hs, errs_bnd)
    assert np.all(o_int > 7.9), o_int
    assert o_bnd[-1] > 3.8 and np.all(np.diff(o_bnd) > 0), o_bnd


@pytest.mark.parametrize("n", [30, 45])
def test_adjoint_operator_is_h_adjoint(n):
    D, A = dense(0, n), dense(1, n)
    H = np.diag(norm_diag(n))
    assert np.max(np.abs(H @ A - (H @ D).T)) < 1e-13


def test_dissipation_self_adjoint():
    n = 40
    Dd, Dt = dense(2, n), dense(3, n)
    assert np.max(np.abs(Dt - Dd.T)) == 0.0
    H = norm_diag(n)
    arc = np.linspace(0.5, 1.5, n)
    M = np.diag(1.0 / H) @ Dt @ np.diag(-arc) @ Dd
    HM = np.diag(H) @ M
    assert np.max(np.abs(HM - HM.T)) < 1e-12


def _dual_consistency(P, seed=1):
    rng = np.random.default_rng(seed)
    q0, lam = random_full_rhs_state(P, seed)
    N = P.blocks[0].n_points
    nD = P.options.n_dimensions
    nU = nD + 2
    g = P.options.ratio_of_specific_heats
    dprim = rng.uniform(-1.0, 1.0, (nU, N))
    dq = np.zeros_like(q0)
    dq[0] = dprim[0]
    for j in range(nD):
        dq[1 + j] = q0[1 + j] / q0[0] * dprim[0] + q0[0] * dprim[1 + j]
    dq[nU - 1] = (q0[nU - 1] / q0[0] * dprim[0] + np.sum(q0[1:1 + nD] * dprim[1:1 + nD], axis=0)
                  + q0[0] / g * dprim[nU - 1])
    o = oracle_lib.Oracle(P)
    o.set_field(1, capi.FIELD_CONSERVED, q0)
    o.update_state()
    o.set_field(1, capi.FIELD_ADJOINT, lam)
    o.update_adjoint_forcing(True)
    o.compute_rhs(capi.FORWARD, 0.3)
    r0 = o.get_field(1, capi.FIELD_RHS)
    o.compute_rhs(capi.ADJOINT, 0.3, 1.0)
    ra = o.get_field(1, capi.FIELD_RHS)
    norm = o.get_field(1, capi.FIELD_NORM)
    s1 = np.sum(ra * norm * dq)
    hs, errs = [], []
    h = 1e-3
    for _ in range(12):
        o.set_field(1, capi.FIELD_CONSERVED, q0 + h * dq)
        o.update_state()
        o.compute_rhs(capi.FORWARD, 0.3)
        s2 = np.sum(lam * norm * (o.get_field(1, capi.FIELD_RHS) - r0))
        hs.append(h)
        errs.append(abs((s2 / h + s1) / s1))
        h *= 10 ** -0.25
    order = fd_order(hs, errs)
    order = np.sort(order)[1:-1]  # trimmed mean, as full_rhs.f90:443-451
    return order.mean()


@pytest.mark.parametrize("composite", [True, False])
def test_full_rhs_dual_consistency_2d(composite):
    P = small_monopole(n=31, ny=29, sponge_points=5, composite_dissipation=composite)
    assert _dual_consistency(P) >= 0.9


def test_full_rhs_dual_consistency_2d_curvilinear_inviscid_penalty_only():
    P = small_monopole(n=29, ny=31, sponge_points=4)
    P.options.curvilinear = True
    x, y = P.blocks[0].coordinates
    P.blocks[0].coordinates = np.ascontiguousarray(np.stack([x + 0.1 * np.sin(0.4 * y), y + 0.05 * np.sin(0.3 * x)]))
    for p in P.patches:
        if p.type == "SAT_FAR_FIELD":
            p.viscous_penalty_amount = 0.0
    assert _dual_consistency(P, 3) >= 0.9


def test_full_rhs_dual_consistency_3d_periodic():
    P = configs.taylor_green_3d(n=12)
    P.options.use_constant_cfl = False
    P.options.time_step_size = 0.01
    assert _dual_consistency(P, 2) >= 0.9


def test_gradient_finite_difference_sweep():
    P = small_monopole(n=33, ny=33, n_steps=24, save_interval=6)
    o = oracle_lib.Oracle(P)
    J0 = o.run_forward(P.n_steps)
    G0 = o.run_adjoint()
    grad = o.gradient(4 * P.n_steps)
    assert J0 > 0 and G0 > 0
    P.options.controller_switch = True
    best = 1.0
    for k in (0, 2, 4):
        eps = 10 ** (-2 - 0.25 * k)
        o2 = oracle_lib.Oracle(P)
        o2.set_control_forcing(eps * grad)
        J1 = o2.run_forward(P.n_steps, keep_stages=False)
        best = min(best, abs((J1 - J0) / eps - G0) / G0)
    # the error grows as eps shrinks (roundoff in J1 - J0); its minimum bounds the adjoint error
    assert best < 1e-5


def test_oracle_time_step_size_restated_in_numpy():
    """computeTimeStepSize (src/CNSHelperImpl.f90:913-982) restated with numpy
    from the oracle's own grid and state arrays pins the oracle's CFL rule."""
    P = small_monopole(cfl=0.7)
    q, _ = random_full_rhs_state(P, 12)
    o = oracle_lib.Oracle(P)
    o.set_field(1, capi.FIELD_CONSERVED, q)
    o.update_state()
    opt = P.options
    g = opt.ratio_of_specific_heats
    nD = 2
    N = q.shape[1]
    m = o.get_field(1, capi.FIELD_METRICS).reshape(nD * nD, N)
    jac = o.get_field(1, capi.FIELD_JACOBIAN)
    T = o.get_field(1, capi.FIELD_TEMPERATURE)
    u = q[1:1 + nD] / q[0]
    a = np.sqrt((g - 1.0) * T)
    rows = [m[nD * j:nD * (j + 1)] for j in range(nD)]
    w = a * np.sqrt(sum(np.sum(r ** 2, axis=0) for r in rows))
    w = w + sum(np.abs(np.sum(u * r, axis=0)) for r in rows)
    dt = np.min(opt.cfl / (jac * w))
    mu = ((g - 1.0) * T) ** opt.viscosity_power_law_exponent / opt.reynolds_number
    k = mu / opt.prandtl_number
    wv = jac ** 2 * np.sum(m ** 2, axis=0) * np.maximum(2.0 * mu, k)
    dt = min(dt, np.min(opt.cfl / wv))
    assert abs(o.time_step_size() - dt) <= 1e-13 * dt


@pytest.mark.parametrize("wall", ["SAT_SLIP_WALL", "SAT_ISOTHERMAL_WALL", "SAT_ADIABATIC_WALL"])
def test_full_rhs_dual_consistency_walls(wall):
    """Dual consistency of the full RHS with wall SATs on two faces
    (test/adjoint_relation/SAT_isothermal.f90 and full_rhs.f90)."""
    P = configs.wall_channel_2d(n=31, ny=29, wall=wall)
    assert _dual_consistency(P) >= 0.9


def test_isothermal_wall_sat_vanishes_on_wall_state():
    """The forward wall SAT is zero on a state that satisfies the wall
    conditions: no velocity and the wall temperature (isothermal_wall_SAT.f90:150-200)."""
    Tw = 2.7
    P = configs.wall_channel_2d(n=31, ny=29, wall="SAT_ISOTHERMAL_WALL", wall_temperature=Tw)
    Pref = configs.wall_channel_2d(n=31, ny=29, wall="SAT_SLIP_WALL")
    rng = np.random.default_rng(4)
    q, _ = random_full_rhs_state(P, 4)
    g = P.options.ratio_of_specific_heats
    n, ny = 31, 29
    for j in (0, ny - 1):
        k = np.arange(n) + n * j
        q[1, k] = 0.0
        q[2, k] = 0.0
        q[3, k] = q[0, k] * Tw / g  # rho T / gamma with u = 0
    rhs = []
    for prob in (P, Pref):
        o = oracle_lib.Oracle(prob)
        o.set_field(1, capi.FIELD_CONSERVED, q)
        o.update_state()
        o.compute_rhs(capi.FORWARD, 0.0)
        rhs.append(o.get_field(1, capi.FIELD_RHS))
    # the isothermal wall adds nothing beyond the (also vanishing) slip-wall penalty
    assert np.max(np.abs(rhs[0] - rhs[1])) <= 1e-12 * np.max(np.abs(rhs[1]))
    del rng


def test_terminal_kinetic_energy_gradient_finite_differences():
    """Terminal kinetic-energy functional on the 3D Taylor-Green vortex: the
    adjoint state at t = 0 is the H-weighted gradient of J(T) with respect to
    the initial state, checked against central differences."""
    P = configs.taylor_green_3d(n=12, dt=0.02, n_steps=6, save_interval=3)
    q0 = P.blocks[0].initial_state.copy()
    rng = np.random.default_rng(5)
    dq = rng.standard_normal(q0.shape) * 1e-2
    o = oracle_lib.Oracle(P)
    norm = o.get_field(1, capi.FIELD_NORM)

    def J(q):
        o.set_field(1, capi.FIELD_CONSERVED, q)
        return o.run_forward(P.n_steps, P.save_interval)

    J(q0)
    o.run_adjoint()
    lam0 = o.get_field(1, capi.FIELD_ADJOINT)
    an = np.sum(norm * lam0 * dq)
    eps = 1e-4
    fd = (J(q0 + eps * dq) - J(q0 - eps * dq)) / (2 * eps)
    assert abs(fd - an) <= 1e-7 * abs(an)


def _smooth_state_on(coords, gamma, phase):
    x, y = coords
    rho = 1.0 + 0.1 * np.sin(0.4 * x + phase) * np.cos(0.3 * y)
    u = 0.2 * np.cos(0.3 * x + 0.2 * y + phase)
    v = 0.15 * np.sin(0.25 * y - 0.1 * x)
    p = 1.0 / gamma + 0.05 * np.cos(0.35 * x - 0.15 * y)
    return np.stack([rho, rho * u, rho * v, p / (gamma - 1.0) + 0.5 * rho * (u * u + v * v)])


def _multiblock_rhs(P, states, mode=capi.FORWARD, lams=None):
    o = oracle_lib.Oracle(P)
    for bi, q in enumerate(states, start=1):
        o.set_field(bi, capi.FIELD_CONSERVED, q)
        if lams is not None:
            o.set_field(bi, capi.FIELD_ADJOINT, lams[bi - 1])
    o.update_state()
    o.compute_rhs(mode, 0.0, 1.0)
    return o, [o.get_field(bi, capi.FIELD_RHS) for bi in range(1, len(states) + 1)]


@pytest.mark.parametrize("rotate", [False, True])
def test_block_interface_sat_vanishes_on_continuous_state(rotate):
    """Inviscid: on a state that is continuous across the interface, the
    interface SAT (src/BlockInterfacePatchImpl.f90:237-262) adds nothing; a
    wrong point correspondence or index reordering would."""
    P = configs.two_block_2d(viscous=False, rotate_second=rotate)
    P0 = configs.two_block_2d(viscous=False, rotate_second=rotate, interfaces=False)
    states = [_smooth_state_on(b.coordinates, 1.4, 0.3) for b in P.blocks]
    _, r1 = _multiblock_rhs(P, states)
    _, r0 = _multiblock_rhs(P0, states)
    for a, b in zip(r1, r0):
        assert np.max(np.abs(a - b)) <= 1e-12 * np.max(np.abs(b))
    # a discontinuous state does feel the interface
    states[1] = states[1] * 1.01
    _, r1 = _multiblock_rhs(P, states)
    _, r0 = _multiblock_rhs(P0, states)
    assert np.max(np.abs(r1[0] - r0[0])) > 1e-6


def test_block_interface_rotated_layout_is_equivalent():
    """Storing block 2 rotated (a transposing interface, interface_index 2, 1, 3)
    gives the same viscous RHS after mapping the rotation back."""
    nx2, ny = 29, 31
    Pa = configs.two_block_2d(rotate_second=False, curvilinear=True)
    Pb = configs.two_block_2d(rotate_second=True)
    sa = [_smooth_state_on(b.coordinates, 1.4, 0.7) for b in Pa.blocks]
    sb = [_smooth_state_on(b.coordinates, 1.4, 0.7) for b in Pb.blocks]
    _, ra = _multiblock_rhs(Pa, sa)
    _, rb = _multiblock_rhs(Pb, sb)
    assert np.max(np.abs(ra[0] - rb[0])) <= 1e-11 * np.max(np.abs(ra[0]))
    # block 2: unrotated point (i, j) <-> rotated point (j, nx2 + 1 - i)
    ia = ra[1].reshape(4, ny, nx2)
    ib = rb[1].reshape(4, nx2, ny)[:, ::-1, :].transpose(0, 2, 1)
    assert np.max(np.abs(ia - ib)) <= 1e-11 * np.max(np.abs(ia))


@pytest.mark.parametrize("rotate", [False, True])
def test_block_interface_dual_consistency(rotate):
    """Full-RHS dual consistency across two blocks with viscous interface SATs
    (test/adjoint_relation/SAT_block_interface.f90)."""
    P = configs.two_block_2d(rotate_second=rotate)
    rng = np.random.default_rng(9)
    g = 1.4
    q0 = [_smooth_state_on(b.coordinates, g, 0.2) * (1.0 + 0.02 * rng.standard_normal((4, b.n_points)))
          for b in P.blocks]
    lam = [rng.uniform(0.0, 1.0, (4, b.n_points)) for b in P.blocks]
    dq = [rng.uniform(-1.0, 1.0, (4, b.n_points)) * q for q, b in zip(q0, P.blocks)]
    o, r0 = _multiblock_rhs(P, q0, capi.FORWARD)
    norms = [o.get_field(bi, capi.FIELD_NORM) for bi in (1, 2)]
    _, ra = _multiblock_rhs(P, q0, capi.ADJOINT, lam)
    s1 = sum(np.sum(a * n * d) for a, n, d in zip(ra, norms, dq))
    hs, errs = [], []
    h = 1e-3
    for _ in range(12):
        _, r = _multiblock_rhs(P, [q + h * d for q, d in zip(q0, dq)])
        s2 = sum(np.sum(l * n * (x - y)) for l, n, x, y in zip(lam, norms, r, r0))
        hs.append(h)
        errs.append(abs((s2 / h + s1) / s1))
        h *= 10 ** -0.25
    order = np.sort(fd_order(hs, errs))[1:-1]
    assert order.mean() >= 0.9


@pytest.mark.parametrize("rotate", [False, True])
def test_two_block_gradient_finite_difference_sweep(rotate):
    """The discrete adjoint across a block interface: sound from a source and an
    actuator in block 1 reaches the cost target in block 2 (README gradient check)."""
    P = configs.two_block_2d(functional=True, rotate_second=rotate, n_steps=40, dt=0.05)
    o = oracle_lib.Oracle(P)
    J0 = o.run_forward(P.n_steps, 7)
    G0 = o.run_adjoint()
    grad = o.gradient(4 * P.n_steps)
    assert J0 > 0 and G0 > 0
    P.options.controller_switch = True
    best = 1.0
    for k in (0, 2, 4, 6):
        eps = 10 ** (-2 - 0.25 * k)
        o2 = oracle_lib.Oracle(P)
        o2.set_control_forcing(eps * grad)
        J1 = o2.run_forward(P.n_steps, keep_stages=False)
        best = min(best, abs((J1 - J0) / eps - G0) / G0)
    assert best < 1e-5


def test_solenoidal_excitation_forward_term_restated_in_numpy():
    """The oracle's forward excitation term equals the reference formula
    restated with numpy (momentum f, energy u . f) on a random state."""
    from helpers import add_solenoidal_excitation, solenoidal_forcing_numpy
    P0 = small_monopole(n=31, ny=29, sponge_points=5)
    P1 = small_monopole(n=31, ny=29, sponge_points=5)
    patch = add_solenoidal_excitation(P1, extent=(4, 26, 3, 25, 1, -1))
    q, _ = random_full_rhs_state(P0, 5)
    out = []
    for P in (P0, P1):
        o = oracle_lib.Oracle(P)
        o.set_field(1, capi.FIELD_CONSERVED, q)
        o.update_state()
        o.compute_rhs(capi.FORWARD, 1.7)
        out.append(o.get_field(1, capi.FIELD_RHS))
    d = out[1] - out[0]
    nx, ny = P0.blocks[0].grid_size[:2]
    x, y = P0.blocks[0].coordinates
    i, j = np.meshgrid(np.arange(nx), np.arange(ny), indexing="xy")
    inside = ((i >= 3) & (i <= 25) & (j >= 2) & (j <= 24)).ravel()
    fx, fy = solenoidal_forcing_numpy(patch, x[inside], y[inside], 1.7)
    u, v = q[1] / q[0], q[2] / q[0]
    expect = np.zeros_like(d)
    expect[1, inside] = fx
    expect[2, inside] = fy
    expect[3, inside] = u[inside] * fx + v[inside] * fy
    scale = np.max(np.abs(expect))
    assert scale > 1e-3
    assert np.max(np.abs(d - expect)) < 1e-12 * np.max(np.abs(out[0]))


def test_full_rhs_dual_consistency_2d_solenoidal_excitation():
    from helpers import add_solenoidal_excitation
    P = small_monopole(n=31, ny=29, sponge_points=5)
    add_solenoidal_excitation(P, extent=(4, 26, 3, 25, 1, -1))
    assert _dual_consistency(P, 4) >= 0.9


def test_gradient_finite_difference_sweep_with_solenoidal_excitation():
    """The adjoint of a run with a solenoidal excitation (evaluated at each
    forward stage's time) matches the J(eps) finite-difference sweep."""
    from helpers import add_solenoidal_excitation
    P = small_monopole(n=33, ny=33, n_steps=24, save_interval=6)
    add_solenoidal_excitation(P, extent=(3, 31, 3, 31, 1, -1), amplitude=0.05, velocity=(1.0, 0.5), frequency=0.5)
    o = oracle_lib.Oracle(P)
    J0 = o.run_forward(P.n_steps)
    G0 = o.run_adjoint()
    grad = o.gradient(4 * P.n_steps)
    assert J0 > 0 and G0 > 0
    P.options.controller_switch = True
    best = 1.0
    for k in (0, 2, 4):
        eps = 10 ** (-2 - 0.25 * k)
        o2 = oracle_lib.Oracle(P)
        o2.set_control_forcing(eps * grad)
        J1 = o2.run_forward(P.n_steps, keep_stages=False)
        best = min(best, abs((J1 - J0) / eps - G0) / G0)
    assert best < 1e-5


def _small_jet(**kw):
    kw.setdefault("nx", 28)
    kw.setdefault("ny_core", 25)
    kw.setdefault("ny_side", 26)
    kw.setdefault("nz", 25)
    kw.setdefault("length", 4.0)
    kw.setdefault("n_steps", 8)
    kw.setdefault("save_interval", 3)
    kw.setdefault("target", (0.5, 0.6, 0.3, 0.5))
    return configs.jet_3block_3d(**kw)


def test_jet_3block_gradient_finite_difference_sweep():
    """Three curvilinear 3D blocks with block interfaces, a solenoidal
    excitation and an actuator: the adjoint gradient matches J(eps)."""
    P = _small_jet()
    o = oracle_lib.Oracle(P)
    J0 = o.run_forward(P.n_steps)
    G0 = o.run_adjoint()
    grad = o.gradient(4 * P.n_steps)
    assert J0 > 0 and G0 > 0
    P.options.controller_switch = True
    best = 1.0
    for k in (0, 2, 4):
        eps = 10 ** (-2 - 0.25 * k)
        o2 = oracle_lib.Oracle(P)
        o2.set_control_forcing(eps * grad)
        J1 = o2.run_forward(P.n_steps, keep_stages=False)
        best = min(best, abs((J1 - J0) / eps - G0) / G0)
    assert best < 1e-5


def _linearized_case(P, seed):
    from magudi_gb300.configs import smooth_perturbed_state
    rng = np.random.default_rng(seed)
    q0 = smooth_perturbed_state(P.blocks[0], P.options.n_dimensions, P.options.ratio_of_specific_heats, rng,
                                amplitude=0.05)
    dq = rng.uniform(-1.0, 1.0, q0.shape) * np.abs(q0).mean(axis=1, keepdims=True)
    lam = rng.uniform(-1.0, 1.0, q0.shape)
    return q0, dq, lam


@pytest.mark.parametrize("viscous", [True, False])
def test_linearized_rhs_matches_central_difference(viscous):
    """computeRhsLinearized (src/RhsHelperImpl.f90:598-829) with the far-field
    and sponge linearizations is the derivative of the forward RHS."""
    P = small_monopole(n=31, ny=29, sponge_points=5)
    P.options.viscous = viscous
    q0, dq, _ = _linearized_case(P, 7)
    o = oracle_lib.Oracle(P)
    o.set_field(1, capi.FIELD_CONSERVED, q0)
    o.update_state()
    o.set_field(1, capi.FIELD_ADJOINT, dq)
    o.compute_rhs(capi.LINEARIZED, 0.3, 0.0)
    L = o.get_field(1, capi.FIELD_RHS)
    errs = []
    for e in (1e-3, 1e-4, 1e-5):
        r = []
        for sgn in (1.0, -1.0):
            o.set_field(1, capi.FIELD_CONSERVED, q0 + sgn * e * dq)
            o.update_state()
            o.compute_rhs(capi.FORWARD, 0.3)
            r.append(o.get_field(1, capi.FIELD_RHS))
        errs.append(np.linalg.norm((r[0] - r[1]) / (2 * e) - L) / np.linalg.norm(L))
    assert min(errs) < 1e-7 and errs[1] < 0.05 * errs[0]


def test_linearized_rhs_is_the_transpose_of_the_adjoint_rhs():
    """<lambda, L dq>_H = -<R^dagger lambda, dq>_H to rounding: the linearized
    and the adjoint RHS are exact transposes of each other."""
    P = small_monopole(n=31, ny=29, sponge_points=5)
    q0, dq, lam = _linearized_case(P, 9)
    o = oracle_lib.Oracle(P)
    o.set_field(1, capi.FIELD_CONSERVED, q0)
    o.update_state()
    H = o.get_field(1, capi.FIELD_NORM)
    o.set_field(1, capi.FIELD_ADJOINT, dq)
    o.compute_rhs(capi.LINEARIZED, 0.3, 0.0)
    a = np.sum(lam * H * o.get_field(1, capi.FIELD_RHS))
    o.set_field(1, capi.FIELD_ADJOINT, lam)
    o.compute_rhs(capi.ADJOINT, 0.3, 0.0)
    b = np.sum(o.get_field(1, capi.FIELD_RHS) * H * dq)
    assert abs(a + b) <= 1e-11 * abs(a)


@pytest.mark.parametrize("wall", ["SAT_SLIP_WALL", "SAT_ISOTHERMAL_WALL", "SAT_ADIABATIC_WALL"])
def test_linearized_rhs_with_walls_is_derivative_and_transpose(wall):
    """Linearized wall penalties (src/ImpenetrableWallImpl.f90:187-191,
    src/IsothermalWallImpl.f90:309-322): central differences of the forward
    RHS, and exact transposition against the adjoint RHS."""
    P = configs.wall_channel_2d(wall=wall)
    q0, dq, lam = _linearized_case(P, 12)
    o = oracle_lib.Oracle(P)
    o.set_field(1, capi.FIELD_CONSERVED, q0)
    o.update_state()
    H = o.get_field(1, capi.FIELD_NORM)
    o.set_field(1, capi.FIELD_ADJOINT, dq)
    o.compute_rhs(capi.LINEARIZED, 0.3, 0.0)
    L = o.get_field(1, capi.FIELD_RHS)
    errs = []
    for e in (1e-4, 1e-5):
        r = []
        for sgn in (1.0, -1.0):
            o2 = oracle_lib.Oracle(P)
            o2.set_field(1, capi.FIELD_CONSERVED, q0 + sgn * e * dq)
            o2.update_state()
            o2.compute_rhs(capi.FORWARD, 0.3)
            r.append(o2.get_field(1, capi.FIELD_RHS))
        errs.append(np.linalg.norm((r[0] - r[1]) / (2 * e) - L) / np.linalg.norm(L))
    assert min(errs) < 1e-7
    a = np.sum(lam * H * L)
    o.set_field(1, capi.FIELD_ADJOINT, lam)
    o.compute_rhs(capi.ADJOINT, 0.3, 0.0)
    b = np.sum(o.get_field(1, capi.FIELD_RHS) * H * dq)
    assert abs(a + b) <= 1e-11 * abs(a)


@pytest.mark.parametrize("rotate", [False, True])
def test_linearized_rhs_with_block_interfaces_is_derivative_and_transpose(rotate):
    """Linearized block-interface penalty (src/BlockInterfacePatchImpl.f90:468-515)
    across two blocks: central differences of the forward RHS of both blocks
    and exact transposition against the adjoint RHS."""
    P = configs.two_block_2d(rotate_second=rotate)
    rng = np.random.default_rng(21)
    q0, dq, lam = [], [], []
    for b in P.blocks:
        q = configs.smooth_perturbed_state(b, 2, 1.4, rng, amplitude=0.05)
        q0.append(q)
        dq.append(rng.uniform(-1.0, 1.0, q.shape) * np.abs(q).mean(axis=1, keepdims=True))
        lam.append(rng.uniform(-1.0, 1.0, q.shape))
    def rhs(o, mode, states, field):
        for bi in (1, 2):
            o.set_field(bi, field, states[bi - 1])
        if mode == capi.FORWARD:
            o.update_state()
        o.compute_rhs(mode, 0.3, 0.0)
        return [o.get_field(bi, capi.FIELD_RHS) for bi in (1, 2)]
    o = oracle_lib.Oracle(P)
    for bi in (1, 2):
        o.set_field(bi, capi.FIELD_CONSERVED, q0[bi - 1])
    o.update_state()
    H = [o.get_field(bi, capi.FIELD_NORM) for bi in (1, 2)]
    L = rhs(o, capi.LINEARIZED, dq, capi.FIELD_ADJOINT)
    nrm = np.sqrt(sum(np.sum(x ** 2) for x in L))
    errs = []
    for e in (1e-4, 1e-5):
        rp = rhs(oracle_lib.Oracle(P), capi.FORWARD, [q + e * d for q, d in zip(q0, dq)], capi.FIELD_CONSERVED)
        rm = rhs(oracle_lib.Oracle(P), capi.FORWARD, [q - e * d for q, d in zip(q0, dq)], capi.FIELD_CONSERVED)
        errs.append(np.sqrt(sum(np.sum(((a - b) / (2 * e) - l) ** 2) for a, b, l in zip(rp, rm, L))) / nrm)
    assert min(errs) < 1e-7
    a = sum(np.sum(l_ * h * x) for l_, h, x in zip(lam, H, L))
    Ra = rhs(o, capi.ADJOINT, lam, capi.FIELD_ADJOINT)
    b = sum(np.sum(r * h * d) for r, h, d in zip(Ra, H, dq))
    assert abs(a + b) <= 1e-11 * abs(a)


def test_linearized_rhs_refuses_solenoidal_excitation():
    from helpers import add_solenoidal_excitation
    P = small_monopole(n=31, ny=29, sponge_points=5)
    add_solenoidal_excitation(P, extent=(4, 26, 3, 25, 1, -1))
    o = oracle_lib.Oracle(P)
    o.update_state()
    with pytest.raises(RuntimeError):
        o.compute_rhs(capi.LINEARIZED, 0.0, 0.0)


def test_linearized_run_matches_central_difference_of_forward_runs():
    """runLinearized's final perturbation is the derivative of the final state
    of the forward run along the initial perturbation."""
    P = small_monopole(n=29, ny=29, n_steps=12, save_interval=4)
    q0, dq, _ = _linearized_case(P, 4)
    o = oracle_lib.Oracle(P)
    o.set_field(1, capi.FIELD_CONSERVED, q0)
    o.run_forward(P.n_steps, 4)
    o.set_field(1, capi.FIELD_ADJOINT, dq)
    o.run_linearized()
    dT = o.get_field(1, capi.FIELD_ADJOINT)
    errs = []
    for e in (1e-3, 1e-4, 1e-5):
        qs = []
        for sgn in (1.0, -1.0):
            o2 = oracle_lib.Oracle(P)
            o2.set_field(1, capi.FIELD_CONSERVED, q0 + sgn * e * dq)
            o2.run_forward(P.n_steps, 4, keep_stages=False)
            qs.append(o2.get_field(1, capi.FIELD_CONSERVED))
        errs.append(np.linalg.norm((qs[0] - qs[1]) / (2 * e) - dT) / np.linalg.norm(dT))
    assert min(errs) < 1e-7


def test_linearized_and_adjoint_runs_are_dual():
    """<lambda(0), dq(0)>_H = <lambda(T), dq(T)>_H: the adjoint run from a given
    terminal condition (adjoint_nonzero_initial_condition, no functional
    forcing) transposes the tangent run exactly."""
    P = small_monopole(n=29, ny=29, n_steps=12, save_interval=4)
    P.options.adjoint_forcing_switch = False
    q0, dq, lamT = _linearized_case(P, 6)
    o = oracle_lib.Oracle(P)
    o.set_field(1, capi.FIELD_CONSERVED, q0)
    o.run_forward(P.n_steps, 4)
    H = o.get_field(1, capi.FIELD_NORM)
    o.set_field(1, capi.FIELD_ADJOINT, dq)
    o.run_linearized()
    b = np.sum(lamT * H * o.get_field(1, capi.FIELD_ADJOINT))
    o.set_field(1, capi.FIELD_ADJOINT, lamT)
    o.set_adjoint_nonzero_initial_condition(True)
    o.run_adjoint()
    a = np.sum(o.get_field(1, capi.FIELD_ADJOINT) * H * dq)
    assert abs(a - b) <= 1e-11 * abs(b)


def test_tangent_run_of_the_functional_matches_the_adjoint_and_central_differences():
    """Forward mode through the tangent run: along the adjoint gradient
    direction the tangent of J equals the adjoint's sensitivity to rounding
    (jvp = vjp), and along a random control perturbation it matches central
    differences of J."""
    P = small_monopole(n=29, ny=29, n_steps=12, save_interval=4)
    P.options.controller_switch = True
    o = oracle_lib.Oracle(P)
    N = P.blocks[0].n_points
    zeros = np.zeros((4, N))
    J0 = o.run_forward(P.n_steps, 4)
    G0 = o.run_adjoint()
    g = o.gradient(4 * P.n_steps)
    o.run_forward(P.n_steps, 4)
    o.set_field(1, capi.FIELD_ADJOINT, zeros)
    dJ = o.run_linearized(g)
    assert abs(dJ - G0) <= 1e-11 * abs(G0)
    rng = np.random.default_rng(2)
    df = rng.standard_normal(g.shape)
    o.set_field(1, capi.FIELD_ADJOINT, zeros)
    dJr = o.run_linearized(df)
    best = 1.0
    for e in (1e-1, 1e-2, 1e-3):
        Js = []
        for sgn in (1.0, -1.0):
            o2 = oracle_lib.Oracle(P)
            o2.set_control_forcing(sgn * e * df)
            Js.append(o2.run_forward(P.n_steps, keep_stages=False))
        best = min(best, abs((Js[0] - Js[1]) / (2 * e) - dJr) / abs(dJr))
    assert best < 1e-5


def test_per_call_control_flow_reproduces_the_runs():
    """The reference's solver loop over the per-call entry points
    (magudi_gb300.drivers) gives the J and gradient norm of the run entry
    points, on the oracle."""
    from magudi_gb300.drivers import per_call_gradient
    P = small_monopole(n=29, ny=29, n_steps=11, save_interval=4)
    o = oracle_lib.Oracle(P)
    J = o.run_forward(P.n_steps, 4)
    G = o.run_adjoint()
    Jp, Gp = per_call_gradient(oracle_lib.Oracle(P), P, P.n_steps, 4)
    assert abs(Jp - J) <= 1e-12 * abs(J)
    assert abs(Gp - G) <= 1e-12 * abs(G)


@pytest.mark.parametrize("rotate", [False, True])
def test_two_block_linearized_and_adjoint_runs_are_dual(rotate):
    """Across a block interface, the tangent run and the adjoint run from a
    given terminal condition transpose each other exactly:
    <lambda(0), dq(0)>_H = <lambda(T), dq(T)>_H summed over the blocks."""
    P = configs.two_block_2d(functional=True, rotate_second=rotate, n_steps=10, dt=0.05)
    P.options.adjoint_forcing_switch = False
    rng = np.random.default_rng(31)
    o = oracle_lib.Oracle(P)
    o.run_forward(P.n_steps, 4)
    H = [o.get_field(bi, capi.FIELD_NORM) for bi in (1, 2)]
    dq0 = [1e-3 * rng.standard_normal((4, b.n_points)) for b in P.blocks]
    lamT = [rng.standard_normal((4, b.n_points)) for b in P.blocks]
    for bi in (1, 2):
        o.set_field(bi, capi.FIELD_ADJOINT, dq0[bi - 1])
    o.run_linearized()
    b = sum(np.sum(lamT[bi - 1] * H[bi - 1] * o.get_field(bi, capi.FIELD_ADJOINT)) for bi in (1, 2))
    for bi in (1, 2):
        o.set_field(bi, capi.FIELD_ADJOINT, lamT[bi - 1])
    o.set_adjoint_nonzero_initial_condition(True)
    o.run_adjoint()
    a = sum(np.sum(o.get_field(bi, capi.FIELD_ADJOINT) * H[bi - 1] * dq0[bi - 1]) for bi in (1, 2))
    assert abs(a - b) <= 1e-11 * abs(b)


def test_per_call_control_flow_with_control_forcing_reproduces_the_runs():
    """With a control forcing handed to the actuators stage by stage (the
    controller's updateForcing), the per-call loop gives the controlled run's J."""
    from magudi_gb300.drivers import per_call_forward, per_call_gradient
    P = small_monopole(n=29, ny=29, n_steps=9, save_interval=4)
    P.options.controller_switch = True
    o = oracle_lib.Oracle(P)
    f = 1e-2 * np.random.default_rng(3).standard_normal((4 * P.n_steps, o.actuator_points()))
    o.set_control_forcing(f)
    J = o.run_forward(P.n_steps, 4)
    G = o.run_adjoint()
    o2 = oracle_lib.Oracle(P)
    assert abs(per_call_forward(o2, P, P.n_steps, f) - J) <= 1e-12 * abs(J)
    Jp, Gp = per_call_gradient(oracle_lib.Oracle(P), P, P.n_steps, 4, f)
    assert abs(Jp - J) <= 1e-12 * abs(J)
    assert abs(Gp - G) <= 1e-12 * abs(G)


@pytest.mark.parametrize("periodicity, n, ok", [(capi.PERIODIC_PLANE, 3, False), (capi.PERIODIC_PLANE, 4, True),
                                                (capi.PERIODIC_OVERLAP, 4, False), (capi.PERIODIC_OVERLAP, 5, True)])
def test_periodic_block_size_limits(periodicity, n, ok):
    """The ghost fill of a periodic direction copies 4 points from the other
    end: PLANE needs 4 points and OVERLAP 5; smaller blocks are refused.
    PLANE: a Taylor-Green box; OVERLAP: an O-grid around an annulus."""
    from helpers import annulus_o_grid
    P = annulus_o_grid(n_theta=n) if periodicity == capi.PERIODIC_OVERLAP else configs.taylor_green_3d(n=n, dt=0.01)
    if not ok:
        with pytest.raises(RuntimeError, match="periodic direction needs at least"):
            oracle_lib.Oracle(P)
        return
    o = oracle_lib.Oracle(P)
    o.update_state()
    o.compute_rhs(capi.FORWARD, 0.0)
    assert np.all(np.isfinite(o.get_field(1, capi.FIELD_RHS)))
