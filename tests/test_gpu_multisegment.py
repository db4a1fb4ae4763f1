"""Multi-segment runs on the GPU (segments concurrently, one host thread per
segment context) against the same driver on the oracle (-m gpu)."""
import numpy as np
import pytest

import oracle_lib
from helpers import rel_err
from magudi_gb300.multisegment import MultiSegment
from magudi_gb300.solver import Solver
from test_multisegment import K, NTS, _problem, _trajectory_ics

pytestmark = pytest.mark.gpu

RUN_TOL = 1e-10


@pytest.mark.parametrize("kind,mollified", [("quadratic", False), ("huber", False), ("quadratic", True)])
def test_multisegment_matches_oracle(kind, mollified):
    P = _problem()
    ics = _trajectory_ics(P, perturb=2e-4, seed=5)
    mol = None
    if mollified:
        x, y = P.blocks[0].coordinates
        mol = [0.5 + 0.5 * np.exp(-((x - 1.0) ** 2 + y ** 2) / 8.0)]
    out = []
    for backend, conc in ((Solver, True), (oracle_lib.Oracle, False)):
        ms = MultiSegment(P, K, NTS, penalty_weight=3.0, penalty_type=kind, huber_threshold=1e-3,
                          state_mollifier=mol, backend=backend, concurrent=conc)
        rng = np.random.default_rng(1)
        ms.set_control_forcing(1e-3 * rng.standard_normal((4 * K * NTS, ms.P)))
        out.append((ms.forward(ics), ms.adjoint()))
    (fg, ag), (fo, ao) = out
    assert abs(fg.J - fo.J) <= RUN_TOL * abs(fo.J)
    assert abs(fg.time_integral - fo.time_integral) <= RUN_TOL * abs(fo.time_integral)
    assert abs(ag.total - ao.total) <= RUN_TOL * abs(ao.total)
    assert rel_err(ag.gradient, ao.gradient) < RUN_TOL
    for k in range(1, K):
        assert rel_err(ag.ic_gradients[k][0], ao.ic_gradients[k][0]) < RUN_TOL


def test_multisegment_with_resident_trajectories_is_bitwise_the_checkpointed_one():
    """Every segment context keeps its trajectory (store_trajectory): J, the
    control gradient and the initial-condition gradients are those of the
    segments that recompute checkpoints."""
    P = _problem()
    ics = _trajectory_ics(P, perturb=2e-4, seed=5)
    out = []
    for store in (False, True):
        ms = MultiSegment(P, K, NTS, penalty_weight=3.0, store_trajectory=store)
        rng = np.random.default_rng(1)
        ms.set_control_forcing(1e-3 * rng.standard_normal((4 * K * NTS, ms.P)))
        out.append((ms.forward(ics), ms.adjoint()))
    (f0, a0), (f1, a1) = out
    assert f0.J == f1.J and a0.total == a1.total
    assert np.array_equal(a0.gradient, a1.gradient)
    for k in range(1, K):
        assert np.array_equal(a0.ic_gradients[k][0], a1.ic_gradients[k][0])
