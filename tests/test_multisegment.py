"""Multi-segment (time-split) runs, bin/msforward.f90 + bin/msadjoint.f90, on
the oracle (CPU): the driver logic, its penalty and its gradient against J(eps)."""
import numpy as np
import pytest

import oracle_lib
from helpers import small_monopole
from magudi_gb300 import capi
from magudi_gb300.multisegment import MultiSegment, penalty_gradient_factor, penalty_norm

K, NTS = 3, 8


def _problem():
    P = small_monopole(n=29, ny=29, n_steps=K * NTS, save_interval=4)
    P.options.controller_switch = True
    return P


def _trajectory_ics(P, perturb=0.0, seed=0):
    """Segment initial conditions: states of one run at the segment boundaries, optionally perturbed."""
    o = oracle_lib.Oracle(P)
    rng = np.random.default_rng(seed)
    ics = [None]
    for k in range(1, K):
        o.set_field(1, capi.FIELD_CONSERVED, P.blocks[0].initial_state)
        o.run_forward(k * NTS, NTS, keep_stages=False)
        q = o.get_field(1, capi.FIELD_CONSERVED)
        ics.append([q * (1.0 + perturb * rng.standard_normal(q.shape))])
    return ics


def test_penalty_norms():
    assert penalty_norm("quadratic", 4.0, 1.0) == 2.0 and penalty_gradient_factor("quadratic", 4.0, 1.0) == 1.0
    assert penalty_norm("huber", 4.0, 1.0) == 1.5 and penalty_gradient_factor("huber", 4.0, 1.0) == 2.0
    assert penalty_norm("huber", 0.25, 1.0) == 0.125 and penalty_gradient_factor("huber", 0.25, 1.0) == 1.0


def test_segments_on_the_trajectory_reproduce_the_single_run():
    P = _problem()
    single = oracle_lib.Oracle(P)
    J = single.run_forward(K * NTS, NTS, keep_stages=False)
    ms = MultiSegment(P, K, NTS, penalty_weight=1.0, backend=oracle_lib.Oracle, concurrent=False)
    r = ms.forward(_trajectory_ics(P))
    assert abs(r.time_integral - J) <= 1e-12 * abs(J)
    assert r.penalty <= 1e-20 and max(r.segment_l2sq) <= 1e-20


@pytest.mark.parametrize("kind,mollified", [("quadratic", False), ("huber", False), ("quadratic", True)])
def test_multisegment_gradient_finite_difference(kind, mollified):
    """Directional derivative of J along (control gradient, initial-condition
    gradients) equals msadjoint's total inner product."""
    P = _problem()
    ics = _trajectory_ics(P, perturb=2e-4, seed=3)
    mol = None
    if mollified:
        x, y = P.blocks[0].coordinates
        mol = [0.5 + 0.5 * np.exp(-((x - 1.0) ** 2 + y ** 2) / 8.0)]
    kw = dict(penalty_weight=3.0, penalty_type=kind, huber_threshold=1e-3, state_mollifier=mol,
              backend=oracle_lib.Oracle, concurrent=False)
    ms = MultiSegment(P, K, NTS, **kw)
    ms.set_control_forcing(np.zeros((4 * K * NTS, ms.P)))
    r0 = ms.forward(ics)
    a = ms.adjoint()
    assert a.total > 0 and min(a.segment_ic_ip[1:]) > 0 and r0.penalty > 0
    # central differences: the penalty is quadratic in the initial conditions
    best = 1.0
    for e in (1e-4, 1e-5, 1e-6, 1e-7):
        Js = []
        for sgn in (1.0, -1.0):
            ms2 = MultiSegment(P, K, NTS, **kw)
            ms2.set_control_forcing(sgn * e * a.gradient)
            ics2 = [None] + [[ics[k][0] + sgn * e * a.ic_gradients[k][0]] for k in range(1, K)]
            Js.append(ms2.forward(ics2).J)
        best = min(best, abs((Js[0] - Js[1]) / (2 * e) - a.total) / a.total)
    assert best < 1e-6


def test_store_trajectory_option_reaches_every_segment_context():
    """store_trajectory asks every segment context to keep its trajectory; on
    the oracle (which always recomputes) the results are unchanged."""
    P = _problem()
    ics = _trajectory_ics(P, perturb=1e-4, seed=2)
    calls = []

    class Recording(oracle_lib.Oracle):
        def set_trajectory_storage(self, enable=True, max_bytes=0.0):
            calls.append(enable)

    out = []
    for store in (False, True):
        ms = MultiSegment(P, K, NTS, penalty_weight=2.0, backend=Recording, concurrent=False,
                          store_trajectory=store)
        out.append((ms.forward(ics).J, ms.adjoint().total))
    assert calls == [True] * K
    assert out[0] == out[1]
