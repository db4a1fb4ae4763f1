"""Solution limits in the CPU oracle (checkSolutionLimits,
src/SolverImpl.f90:189-304, restated in oracle/oracle.cpp): J = HUGE and
status MGD_SOLUTION_LIMITS on a NaN or out-of-range state, unchanged J
inside the limits, and the magudi.inp keys that switch them on."""
import sys

import numpy as np

import oracle_lib
from helpers import small_monopole
from magudi_gb300 import capi
from magudi_gb300.inputs import InputError, options_from_inputs

HUGE = sys.float_info.max


def _limited(rho=(0.5, 2.0), T=(1.0, 5.0)):
    P = small_monopole(n=25, ny=23, n_steps=6, save_interval=3)
    o = P.options
    o.enable_solution_limits = True
    o.minimum_density, o.maximum_density = rho
    o.minimum_temperature, o.maximum_temperature = T
    return P


def test_inside_the_limits_the_run_is_unchanged():
    P = _limited()
    ref = small_monopole(n=25, ny=23, n_steps=6, save_interval=3)
    a, b = oracle_lib.Oracle(P), oracle_lib.Oracle(ref)
    assert a.run_forward(6, 3) == b.run_forward(6, 3)
    assert a.run_status == 0
    assert a.run_adjoint() == b.run_adjoint()


def test_nan_and_out_of_range_states_give_huge():
    for bad in ("nan", "rho"):
        P = _limited()
        q = P.blocks[0].initial_state.copy()
        if bad == "nan":
            q[1, 40] = np.nan
        else:
            q[0, 40] = 2.5
        o = oracle_lib.Oracle(P)
        o.set_field(1, capi.FIELD_CONSERVED, q)
        assert o.run_forward(6, 3) == HUGE and o.run_status == capi.SOLUTION_LIMITS
        assert o.run_adjoint() == HUGE and o.run_status == capi.SOLUTION_LIMITS


class _Inputs(dict):
    def get_bool(self, k, d):
        return self.get(k, d)

    def get_float(self, k, d):
        return float(self.get(k, d))

    def get_str(self, k, d):
        return self.get(k, d)


def test_magudi_inp_keys_switch_the_limits_on():
    d = _Inputs({"enable_solution_limits": True, "minimum_density": 0.1, "maximum_density": 5.0,
                 "minimum_temperature": 0.2, "maximum_temperature": 9.0, "use_constant_CFL_mode": False,
                 "time_step_size": 0.01})
    o = options_from_inputs(d, 2)
    assert o.enable_solution_limits and o.maximum_temperature == 9.0
    del d["maximum_temperature"]
    try:
        options_from_inputs(d, 2)
    except InputError as e:
        assert "maximum_temperature" in str(e)
    else:
        raise AssertionError("a missing limit must be refused")
