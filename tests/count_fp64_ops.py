"""Algorithmic FP64 operations per grid point of one forward and one adjoint
RHS, counted by the operation-counting build of the oracle
(oracle/build_opcount.sh), for the bench workloads:

    python tests/count_fp64_ops.py [monopole|tgv|jet] ...

The counts are the operation list of the reference's routines as the oracle
restates them (adds, multiplies, divisions and square roots; the power law
counts once as a special function), per section of the RHS. The GPU kernels
execute fewer FP64 instructions than these lists where they skip zero metric
terms or fuse a multiply and an add."""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.dirname(HERE))

import oracle_lib  # noqa: E402
from magudi_gb300 import capi, configs  # noqa: E402

WORKLOADS = {
    "monopole": ("2D monopole 201x201", lambda: configs.monopole_2d(n=201)),
    "tgv": ("3D Taylor-Green 128^3", lambda: configs.taylor_green_3d(n=128, n_steps=4)),
    "jet": ("3D three-block jet, half linear size (4.9 M points)",
            lambda: configs.jet_3block_3d(nx=192, ny_core=96, ny_side=86, nz=96, n_steps=8, save_interval=4)),
}


def flops(c):
    return c["add"] + c["mul"] + c["div"] + c["sqrt"]


def count(P):
    """(forward, adjoint) flops per point and the per-section breakdowns."""
    o = oracle_lib.Oracle(P, variant="opcount")
    N = sum(b.n_points for b in P.blocks)
    rng = np.random.default_rng(1)
    for bi, b in enumerate(P.blocks, start=1):
        q = np.ascontiguousarray(b.initial_state)
        o.set_field(bi, capi.FIELD_CONSERVED, q)
        o.set_field(bi, capi.FIELD_ADJOINT, rng.uniform(-1.0, 1.0, q.shape))
    oracle_lib.opcounts(True)
    o.update_state()
    o.compute_rhs(capi.FORWARD, 0.5)
    fw = oracle_lib.opcounts(True)
    o.update_adjoint_forcing(False)
    oracle_lib.opcounts(True)
    o.compute_rhs(capi.ADJOINT, 0.5, 1.0)
    ad = oracle_lib.opcounts(True)
    per = lambda d: {k: round(flops(v) / N, 1) for k, v in d.items()}  # noqa: E731
    return sum(flops(c) for c in fw.values()) / N, sum(flops(c) for c in ad.values()) / N, per(fw), per(ad), N


if __name__ == "__main__":
    for name in sys.argv[1:] or list(WORKLOADS):
        label, make = WORKLOADS[name]
        f, a, pf, pa, N = count(make())
        print(f"{label}: {N} points; forward RHS {f:.1f}, adjoint RHS {a:.1f} flops per point")
        print(f"  forward sections {pf}")
        print(f"  adjoint sections {pa}")
