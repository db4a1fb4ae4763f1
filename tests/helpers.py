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
