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
