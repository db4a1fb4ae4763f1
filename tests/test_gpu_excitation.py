"""Solenoidal excitation and the three-block curvilinear jet on the GPU
against the oracle (-m gpu). Tolerances as in test_gpu_parity: 1e-12 per RHS,
1e-10 for J and the gradient after a run."""
import numpy as np
import pytest

import oracle_lib
from helpers import add_solenoidal_excitation, random_full_rhs_state, rel_err, small_monopole
from magudi_gb300 import capi, configs
from magudi_gb300.solver import Solver

pytestmark = pytest.mark.gpu

RHS_TOL = 1e-12
RUN_TOL = 1e-10


def _excited_monopole(**kw):
    P = small_monopole(n=33, ny=33, **kw)
    add_solenoidal_excitation(P, extent=(3, 31, 3, 31, 1, -1), amplitude=0.05, velocity=(1.0, 0.5), frequency=0.5)
    return P


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


def test_excitation_rhs_matches_oracle():
    P = _excited_monopole()
    q, lam = random_full_rhs_state(P, 21)
    pair = Solver(P), oracle_lib.Oracle(P)
    for s in pair:
        s.set_field(1, capi.FIELD_CONSERVED, q)
        s.set_field(1, capi.FIELD_ADJOINT, lam)
        s.update_state()
        s.compute_rhs(capi.FORWARD, 2.3)
    assert rel_err(*(s.get_field(1, capi.FIELD_RHS) for s in pair)) < RHS_TOL
    for s in pair:
        s.compute_rhs(capi.ADJOINT, 2.3, 1.0)
    assert rel_err(*(s.get_field(1, capi.FIELD_RHS) for s in pair)) < RHS_TOL


def test_excitation_substeps_match_oracle():
    """Per-call RK4 substeps forward then adjoint (the adjoint evaluates the
    excitation at each matching forward stage's time)."""
    P = _excited_monopole()
    _, lam = random_full_rhs_state(P, 5)
    q = configs.smooth_perturbed_state(P.blocks[0], 2, 1.4, np.random.default_rng(5))
    pair = Solver(P), oracle_lib.Oracle(P)
    for s in pair:
        s.set_field(1, capi.FIELD_CONSERVED, q)
        s.set_field(1, capi.FIELD_ADJOINT, lam * 1e-3)
        s.update_state()
    times = []
    for s in pair:
        t = 1.1
        for stage in (1, 2, 3, 4):
            t = s.rk4_substep(capi.FORWARD, t, 0.01, stage)
        for stage in (4, 3, 2, 1):
            t = s.rk4_substep(capi.ADJOINT, t, 0.01, stage)
        times.append(t)
    assert times[0] == times[1]
    for f in (capi.FIELD_CONSERVED, capi.FIELD_ADJOINT):
        assert rel_err(*(s.get_field(1, f) for s in pair)) < 1e-12


@pytest.mark.parametrize("cfl", [False, True])
def test_excitation_runs_match_oracle(cfl):
    P = _excited_monopole(n_steps=30, save_interval=6, cfl=0.6 if cfl else None)
    g, o = Solver(P), oracle_lib.Oracle(P)
    Jg, Jo = g.run_forward(P.n_steps, P.save_interval), o.run_forward(P.n_steps, P.save_interval)
    assert abs(Jg - Jo) <= RUN_TOL * abs(Jo)
    assert rel_err(g.get_field(1, capi.FIELD_CONSERVED), o.get_field(1, capi.FIELD_CONSERVED)) < 1e-11
    Gg, Go = g.run_adjoint(), o.run_adjoint()
    assert abs(Gg - Go) <= RUN_TOL * abs(Go)
    n = 4 * P.n_steps
    assert rel_err(g.gradient(n), o.gradient(n)) < RUN_TOL


def test_jet_3block_rhs_matches_oracle():
    P = _small_jet()
    rng = np.random.default_rng(4)
    pair = Solver(P), oracle_lib.Oracle(P)
    states = []
    for bi, b in enumerate(P.blocks, start=1):
        q = b.initial_state * (1.0 + 0.01 * rng.standard_normal(b.initial_state.shape))
        lam = rng.uniform(0.0, 1.0, q.shape)
        states.append((bi, q, lam))
    for s in pair:
        for bi, q, lam in states:
            s.set_field(bi, capi.FIELD_CONSERVED, q)
            s.set_field(bi, capi.FIELD_ADJOINT, lam)
        s.update_state()
        s.compute_rhs(capi.FORWARD, 0.4)
    for bi, _, _ in states:
        assert rel_err(*(s.get_field(bi, capi.FIELD_RHS) for s in pair)) < RHS_TOL
    for s in pair:
        s.update_adjoint_forcing(False)
        s.compute_rhs(capi.ADJOINT, 0.4, 1.0)
    for bi, _, _ in states:
        assert rel_err(*(s.get_field(bi, capi.FIELD_RHS) for s in pair)) < RHS_TOL


def test_jet_3block_runs_match_oracle():
    """Checkpointed forward and adjoint runs of the three-block jet."""
    P = _small_jet()
    g, o = Solver(P), oracle_lib.Oracle(P)
    Jg, Jo = g.run_forward(P.n_steps, P.save_interval), o.run_forward(P.n_steps, P.save_interval)
    assert Jo > 0 and abs(Jg - Jo) <= RUN_TOL * abs(Jo)
    for bi in (1, 2, 3):
        assert rel_err(g.get_field(bi, capi.FIELD_CONSERVED), o.get_field(bi, capi.FIELD_CONSERVED)) < 1e-11
    Gg, Go = g.run_adjoint(), o.run_adjoint()
    assert Go > 0 and abs(Gg - Go) <= RUN_TOL * abs(Go)
    n = 4 * P.n_steps
    assert rel_err(g.gradient(n), o.gradient(n)) < RUN_TOL
