"""Gradient-check sweep (the reference's finite-difference loop,
README.md:118-165 with bin/ZAXPY.f90) over many independent forward solves,
and its split over ranks.

cases()    the instances: grid sizes drawn with a seed from SIZES and the
           control amplitude 10^(-2-0.25k), k = i mod 20.
shard()    deterministic split of the instances over ranks, balanced by grid
           points (largest first onto the least-loaded rank). Instances are
           independent, so the ranks need no exchange until the costs are
           gathered.
gather_costs()  all costs on every rank, in instance order (one all_gather).
fd_errors()     the reference's table: amplitude, J, FD gradient, relative error.
"""
import numpy as np

SIZES = (129, 161, 201, 257, 321, 385)


def cases(n_instances=64, seed=0, sizes=SIZES):
    rng = np.random.default_rng(seed)
    drawn = rng.choice(np.asarray(sizes), n_instances)
    return [(int(drawn[i]), 10.0 ** (-2.0 - 0.25 * (i % 20))) for i in range(n_instances)]


def shard(case_list, rank, world):
    """Indices of the instances that rank `rank` of `world` runs."""
    load = [0] * world
    owner = {}
    order = sorted(range(len(case_list)), key=lambda i: (-case_list[i][0] ** 2, i))
    for i in order:
        r = min(range(world), key=lambda k: (load[k], k))
        owner[i] = r
        load[r] += case_list[i][0] ** 2
    return [i for i in range(len(case_list)) if owner[i] == rank]


def gather_costs(local_indices, local_costs, n_total):
    """Every rank's (index, cost) pairs gathered into one vector on all ranks."""
    import torch.distributed as dist
    mine = list(zip(local_indices, [float(c) for c in local_costs]))
    if not dist.is_available() or not dist.is_initialized() or dist.get_world_size() == 1:
        parts = [mine]
    else:
        parts = [None] * dist.get_world_size()
        dist.all_gather_object(parts, mine)
    out = np.full(n_total, np.nan)
    for part in parts:
        for i, c in part:
            out[i] = c
    return out


def fd_errors(J0, grad0, amplitudes, costs):
    """(A_k, J_k, (J_k - J0)/A_k, |(FD - Grad0)/Grad0|) rows of the sweep."""
    rows = []
    for a, J in zip(amplitudes, costs):
        g = (J - J0) / a
        rows.append((a, J, g, abs((g - grad0) / grad0)))
    return rows
