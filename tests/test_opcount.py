"""The algorithmic FP64 operation counts that bench.py's roofline uses,
against the operation-counting build of the oracle (oracle/build_opcount.sh:
the oracle, which restates the reference's operation list, with a counting
value type). The counts per grid point of the 201 x 201 monopole RHS are
frozen in bench.py; this test recounts them, so that a change to the
oracle's operation list or to the frozen numbers cannot go unnoticed."""
import numpy as np

import oracle_lib
from magudi_gb300 import capi, configs


def _flops(c):
    return c["add"] + c["mul"] + c["div"] + c["sqrt"]


def test_frozen_counts_match_the_counting_oracle():
    import bench
    P = configs.monopole_2d(n=201)
    o = oracle_lib.Oracle(P, variant="opcount")
    rng = np.random.default_rng(1)
    q = configs.smooth_perturbed_state(P.blocks[0], 2, 1.4, rng)
    N = P.blocks[0].n_points
    o.set_field(1, capi.FIELD_CONSERVED, q)
    o.set_field(1, capi.FIELD_ADJOINT, rng.uniform(-1.0, 1.0, q.shape))
    oracle_lib.opcounts(True)
    o.update_state()
    o.compute_rhs(capi.FORWARD, 1.0)
    fw = oracle_lib.opcounts(True)
    o.update_adjoint_forcing(False)
    oracle_lib.opcounts(True)
    o.compute_rhs(capi.ADJOINT, 1.0, 1.0)
    ad = oracle_lib.opcounts(True)
    counted = {
        "forward_rhs": sum(_flops(c) for c in fw.values()) / N,
        "adjoint_rhs": sum(_flops(c) for c in ad.values()) / N,
        "adjoint_core": _flops(ad["adjoint"]) / N,
        "dissipation": _flops(ad["dissipation"]) / N,
        "forward_gradient_flux": (_flops(fw["state_gradient"]) + _flops(fw["forward_flux"])) / N,
    }
    for k, v in counted.items():
        assert abs(bench.ALGORITHMIC_FLOPS[k] - v) <= 0.005 * v, (k, v)
    # one power law per point (the viscosity) in the state update
    assert round(fw["state"]["special"] / N) == 1
