"""Shared helpers of the test suite: problem builders and error norms."""
import numpy as np

from magudi_gb300 import capi, configs


def rel_err(a, b):
    """Norm-wise relative error ||a - b|| / ||b|| (pointwise relative error is
    meaningless where the RHS vanishes, e.g. on a quiescent state)."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    nb = np.linalg.norm(b.ravel())
    if nb == 0.0:
        return float(np.linalg.norm(a.ravel()))
    return float(np.linalg.norm((a - b).ravel()) / nb)


def small_monopole(n=41, ny=37, **kw):
    """Monopole-type problem on a small grid: far-field SATs, sponges, target
    and actuator patches, one acoustic source, viscous, dissipation."""
    kw.setdefault("sponge_points", 6)
    kw.setdefault("half_width", 6.0)
    kw.setdefault("target_center", (0.0, 3.0))
    kw.setdefault("mollifier_sigma", 0.7)
    return configs.monopole_2d(n=n, ny=ny, **kw)


def random_full_rhs_state(problem, seed=7):
    rng = np.random.default_rng(seed)
    N = problem.blocks[0].n_points
    nD = problem.options.n_dimensions
    q = configs.random_state(N, nD, problem.options.ratio_of_specific_heats, rng)
    lam = rng.uniform(0.0, 1.0, (nD + 2, N))
    return q, lam


def fd_order(h, err):
    h = np.asarray(h)
    err = np.asarray(err)
    return np.log(err[1:] / err[:-1]) / np.log(h[1:] / h[:-1])


def add_solenoidal_excitation(problem, grid_index=1, extent=(1, -1, 1, -1, 1, -1), amplitude=0.5, n_modes=4,
                              origin=(0.5, -0.3), velocity=(0.7, 0.2), frequency=0.4, radius=3.0, seed=3):
    """Adds a SOLENOIDAL_EXCITATION patch (modes drawn by problem.solenoidal_modes)."""
    from magudi_gb300.problem import Patch
    p = Patch("excitation", "SOLENOIDAL_EXCITATION", grid_index, 0, extent, n_modes=n_modes, origin=origin,
              velocity=velocity, amplitude=amplitude, frequency=frequency, radius=radius, random_seed=seed)
    problem.patches.append(p)
    return p


def solenoidal_forcing_numpy(patch, x, y, t):
    """addSolenoidalExcitation's forcing (f_x, f_y) at time t restated with numpy
    from src/SolenoidalExcitationPatchImpl.f90:93-130 (spatial functions) and
    :193-250 (temporal functions and the two sums)."""
    w, ph = patch.excitation_modes()
    g = 9.0 / (2.0 * patch.radius ** 2)
    dx, dy = x - patch.origin[0], y - patch.origin[1]
    S = patch.amplitude * np.exp(-g * (dx ** 2 + dy ** 2))
    a = np.outer(dx, w) + ph[:, 0]
    c = np.outer(dy, w) + ph[:, 1]
    b1, b2 = w * patch.velocity[0] * t, w * patch.velocity[1] * t
    t1 = np.sin(a - b1)
    t2 = np.cos(a - b1)
    t3 = np.sin(c - b2)
    t4 = np.cos(c - b2)
    fx = S * np.sum(t1 * (w * t4 - 2.0 * g * dy[:, None] * t3), axis=1)
    fy = S * np.sum(t3 * (w * t2 - 2.0 * g * dx[:, None] * t1), axis=1)
    return fx, fy


def annulus_o_grid(n_theta=33, n_r=25, r0=1.0, r1=3.0, dt=0.01, n_steps=6, save_interval=3):
    """2D O-grid around an annulus: direction 1 runs clockwise around it with
    OVERLAP periodicity (the last point repeats the first), direction 2 runs
    outward. Curvilinear, viscous, dissipation, far-field SATs on both
    circles, a Gaussian pressure pulse in a quiescent gas and the terminal
    kinetic-energy functional."""
    from magudi_gb300.problem import Block, Options, Patch, Problem, quiescent_state
    gamma = 1.4
    th = -2.0 * np.pi * np.arange(n_theta) / (n_theta - 1)
    r = r0 + (r1 - r0) * np.arange(n_r) / (n_r - 1)
    R, TH = np.meshgrid(r, th, indexing="ij")  # (n_r, n_theta): theta fastest
    x, y = R * np.cos(TH), R * np.sin(TH)
    x[:, -1], y[:, -1] = x[:, 0], y[:, 0]  # the duplicated point is the same point
    N = n_theta * n_r
    q = quiescent_state(N, 2, gamma)
    xr, yr = x.ravel(), y.ravel()
    pulse = 0.01 * np.exp(-((xr - 2.0) ** 2 + yr ** 2) / 0.2)
    q[3] += pulse / (gamma - 1.0)
    opts = Options(
        n_dimensions=2, viscous=True, dissipation=True, composite_dissipation=True, curvilinear=True,
        use_constant_cfl=False, time_step_size=dt, enable_functional=True, functional_type=1,
        reynolds_number=200.0, dissipation_amount=0.01)
    block = Block(grid_size=(n_theta, n_r, 1), coordinates=np.ascontiguousarray(np.stack([xr, yr])),
                  periodicity_type=(2, 0, 0), initial_state=q, target_state=quiescent_state(N, 2, gamma),
                  mean_pressure=np.full(N, 1.0 / gamma))
    patches = [Patch("farField.inner", "SAT_FAR_FIELD", 1, 2, (1, -1, 1, 1, 1, -1)),
               Patch("farField.outer", "SAT_FAR_FIELD", 1, -2, (1, -1, -1, -1, 1, -1))]
    return Problem(options=opts, blocks=[block], patches=patches, n_steps=n_steps, save_interval=save_interval)
