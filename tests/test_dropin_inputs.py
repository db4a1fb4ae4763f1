"""The reference's own AcousticMonopole example as a drop-in input
(tests/golden/acoustic_monopole: magudi.inp and bc.dat copied unchanged, and
the fields of the example's config.py on its 201 x 201 grid, all written by
make_monopole_example_golden.py): the two files parse into the options,
patches and source the example names, and the oracle runs the problem."""
import os

import numpy as np
import pytest

import oracle_lib
from magudi_gb300 import capi
from magudi_gb300.inputs import problem_from_inputs
from magudi_gb300.problem import Block

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "acoustic_monopole")


def example_problem():
    f = np.load(os.path.join(HERE, "fields.npz"))
    blk = Block(grid_size=tuple(int(x) for x in f["grid_size"]), coordinates=np.ascontiguousarray(f["coordinates"]),
                initial_state=np.ascontiguousarray(f["initial_state"]),
                control_mollifier=np.ascontiguousarray(f["control_mollifier"]),
                target_mollifier=np.ascontiguousarray(f["target_mollifier"]),
                mean_pressure=np.ascontiguousarray(f["mean_pressure"]))
    return problem_from_inputs(os.path.join(HERE, "magudi.inp"), os.path.join(HERE, "bc.dat"), [blk])


def test_example_files_parse_unchanged():
    P = example_problem()
    o = P.options
    assert o.discretization_scheme == capi.SBP_36
    assert o.viscous and not o.use_constant_cfl and not o.curvilinear
    assert o.reynolds_number == 200.0 and o.prandtl_number == 0.7
    assert o.viscosity_power_law_exponent == 0.0 and o.bulk_viscosity_ratio == 0.0
    assert o.dissipation and not o.composite_dissipation and o.dissipation_amount == 1e-4
    assert o.enable_solution_limits and (o.minimum_density, o.maximum_density) == (0.1, 5.0)
    assert (o.minimum_temperature, o.maximum_temperature) == (0.05, 4.0)
    assert o.time_step_size == 0.05 and P.n_steps == 800 and P.save_interval == 200
    assert [p.name for p in P.patches][:4] == ["farField.E", "farField.W", "farField.S", "farField.N"]
    sponge = [p for p in P.patches if p.type == "SPONGE"]
    assert len(sponge) == 4 and all(p.sponge_amount == 0.2 for p in sponge)
    assert all(p.viscous_penalty_amount == 0.0 for p in P.patches if p.type == "SAT_FAR_FIELD")
    (src,) = P.sources
    assert src.location[0] == -3.0 and src.amplitude == 0.01 and abs(src.radius - 2.1213203435596424) < 1e-15


def test_oracle_runs_the_example_inside_its_solution_limits():
    P = example_problem()
    o = oracle_lib.Oracle(P)
    J = o.run_forward(4, 2)
    assert o.run_status == 0 and np.isfinite(J) and J > 0.0
    G = o.run_adjoint()
    assert o.run_status == 0 and np.isfinite(G)
