"""ctypes front end of the CPU oracle (oracle/oracle.cpp) for the tests.

Tests compare the CUDA library against the oracle. It is
built by oracle/build.sh into oracle/_build/liboracle.so.
"""
import ctypes as C
import os
import subprocess

import numpy as np

from magudi_gb300 import capi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_PATH = os.path.join(ROOT, "oracle", "_build", "liboracle.so")
# The same source built with the reference's release flags (-O3 -ffast-math
# -funroll-loops): the timed CPU leg of the bench, never the parity checker.
TUNED_LIB_PATH = os.path.join(ROOT, "oracle", "_build", "liboracle_tuned.so")
# The operation-counting build (oracle/build_opcount.sh): counts the FP64
# operations of the reference's operation list per section of the RHS.
OPCOUNT_LIB_PATH = os.path.join(ROOT, "oracle", "_build", "liboracle_opcount.so")

_libs = {}


def build():
    subprocess.check_call(["bash", os.path.join(ROOT, "oracle", "build.sh")])


def lib(variant="strict"):
    """The oracle library: "strict" (IEEE arithmetic, the checker) or
    "tuned" (fast-math release build, for CPU timing)."""
    if variant not in _libs:
        path = {"strict": LIB_PATH, "tuned": TUNED_LIB_PATH, "opcount": OPCOUNT_LIB_PATH}[variant]
        if not os.path.exists(path):
            if variant == "opcount":
                subprocess.check_call(["bash", os.path.join(ROOT, "oracle", "build_opcount.sh")])
            else:
                build()
        L = C.CDLL(path)
        if variant == "opcount":
            L.orc_opcount.argtypes = [C.POINTER(C.c_longlong), C.c_int]
        L.orc_create.restype = C.c_void_p
        L.orc_create.argtypes = [C.POINTER(capi.Options)]
        L.orc_destroy.argtypes = [C.c_void_p]
        L.orc_last_error.restype = C.c_char_p
        L.orc_last_error.argtypes = [C.c_void_p]
        L.orc_add_block.argtypes = [C.c_void_p, C.POINTER(capi.BlockDesc), C.POINTER(C.c_double), C.POINTER(C.c_int)]
        L.orc_add_patch.argtypes = [C.c_void_p, C.POINTER(capi.PatchDesc)]
        L.orc_add_source.argtypes = [C.c_void_p, C.POINTER(capi.AcousticSource)]
        for f in ("orc_set_field", "orc_get_field"):
            getattr(L, f).argtypes = [C.c_void_p, C.c_int, C.c_int, C.POINTER(C.c_double)]
        L.orc_finalize_setup.argtypes = [C.c_void_p]
        L.orc_update_state.argtypes = [C.c_void_p]
        L.orc_compute_rhs.argtypes = [C.c_void_p, C.c_int, C.c_double, C.c_double]
        L.orc_update_adjoint_forcing.argtypes = [C.c_void_p, C.c_int]
        L.orc_compute_functional.argtypes = [C.c_void_p, C.POINTER(C.c_double)]
        L.orc_compute_sensitivity.argtypes = [C.c_void_p, C.POINTER(C.c_double)]
        L.orc_rk4_substep.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_double), C.c_double, C.c_int]
        L.orc_set_control_forcing.argtypes = [C.c_void_p, C.POINTER(C.c_double), C.c_longlong]
        L.orc_actuator_patch_size.argtypes = [C.c_void_p, C.POINTER(C.c_longlong)]
        L.orc_run_forward.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_double, C.POINTER(C.c_double)]
        L.orc_run_forward_nostore.argtypes = [C.c_void_p, C.c_int, C.c_double, C.POINTER(C.c_double)]
        L.orc_run_adjoint.argtypes = [C.c_void_p, C.POINTER(C.c_double)]
        L.orc_set_adjoint_nonzero_initial_condition.argtypes = [C.c_void_p, C.c_int]
        L.orc_set_patch_control_forcing.argtypes = [C.c_void_p, C.POINTER(C.c_double)]
        L.orc_run_linearized.argtypes = [C.c_void_p, C.POINTER(C.c_double), C.c_longlong, C.POINTER(C.c_double)]
        L.orc_time_step_size.argtypes = [C.c_void_p, C.POINTER(C.c_double)]
        L.orc_step_sizes.argtypes = [C.c_void_p, C.POINTER(C.c_double)]
        L.orc_get_gradient.argtypes = [C.c_void_p, C.POINTER(C.c_double), C.c_longlong]
        L.orc_operator_info.argtypes = [C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_double),
                                        C.POINTER(C.c_double), C.POINTER(C.c_double)]
        L.orc_apply_operator.argtypes = [C.c_int, C.c_int, C.POINTER(C.c_double), C.c_int,
                                         C.POINTER(C.c_int), C.c_int]
        L.orc_set_threads.argtypes = [C.c_int]
        _libs[variant] = L
    return _libs[variant]


def set_threads(n, variant="strict"):
    return lib(variant).orc_set_threads(n)


SECTIONS = {0: "other", 1: "state", 2: "forward", 3: "dissipation", 4: "adjoint", 5: "farfield_adjoint",
            6: "patches", 7: "region", 9: "adjoint_diffusion", 10: "state_gradient", 11: "forward_flux"}
OP_KINDS = ("add", "mul", "div", "sqrt", "special")


def opcounts(reset=True):
    """{section: {kind: count}} of the operation-counting build since the last reset."""
    buf = (C.c_longlong * (16 * 5))()
    lib("opcount").orc_opcount(buf, int(reset))
    return {SECTIONS.get(sec, str(sec)): {k: buf[sec * 5 + i] for i, k in enumerate(OP_KINDS)}
            for sec in range(16) if any(buf[sec * 5 + i] for i in range(5))}


def operator(which, scheme=capi.SBP_48):
    """(symmetry, interior, rhsBoundary1 (width, depth) array, normBoundary) of
    operator `which` of the SBP scheme (capi.SBP_*)."""
    L = lib()
    dims = (C.c_int * 4)()
    which = which + 8 * scheme
    L.orc_operator_info(which, dims, None, None, None)
    sym, iw, bw, bd = list(dims)
    interior = np.zeros(iw)
    rb1 = np.zeros(bw * bd)
    norm = np.zeros(max(bd, 12))
    nn = L.orc_operator_info(which, dims, capi.dptr(interior), capi.dptr(rb1), capi.dptr(norm))
    return sym, interior, rb1.reshape(bd, bw).T, norm[:nn]


def apply_operator(which, x, grid_size, direction, periodicity=0, scheme=capi.SBP_48):
    """Applies operator `which` (0 D, 1 D-adjoint, 2 dissipation, 3 its
    transpose, 4 composite dissipation) of the SBP scheme (capi.SBP_*) along
    `direction` (0-based) to x of shape (nc, N); returns a new array."""
    y = np.ascontiguousarray(x, dtype=np.float64).copy()
    gs = (C.c_int * 3)(*grid_size)
    nc = y.shape[0] if y.ndim == 2 else 1
    lib().orc_apply_operator(which + 8 * scheme, periodicity, capi.dptr(y), nc, gs, direction)
    return y


class Oracle:
    """One oracle region built from a magudi_gb300.problem.Problem."""

    def __init__(self, problem, finalize=True, variant="strict"):
        L = lib(variant)
        self.L = L
        self.problem = problem
        self._opts = problem.options.to_c()
        self.h = L.orc_create(C.byref(self._opts))
        self.nU = problem.n_unknowns
        for blk in problem.blocks:
            coords = np.ascontiguousarray(blk.coordinates, dtype=np.float64)
            ib = blk.iblank_array()
            d = blk.desc()
            rc = L.orc_add_block(self.h, C.byref(d), capi.dptr(coords), capi.iptr(ib))
            if rc:
                raise RuntimeError(L.orc_last_error(self.h).decode())
        for p in problem.patches:
            pd = p.to_c()
            L.orc_add_patch(self.h, C.byref(pd))
        for s in problem.sources:
            sd = s.to_c()
            L.orc_add_source(self.h, C.byref(sd))
        for bi, blk in enumerate(problem.blocks, start=1):
            if blk.target_state is not None:
                self.set_field(bi, capi.FIELD_TARGET, blk.target_state)
            if blk.control_mollifier is not None:
                self.set_field(bi, capi.FIELD_CONTROL_MOLLIFIER, blk.control_mollifier)
            if blk.target_mollifier is not None:
                self.set_field(bi, capi.FIELD_TARGET_MOLLIFIER, blk.target_mollifier)
            if blk.mean_pressure is not None:
                self.set_field(bi, capi.FIELD_MEAN_PRESSURE, blk.mean_pressure)
            if blk.initial_state is not None:
                self.set_field(bi, capi.FIELD_CONSERVED, blk.initial_state)
        if finalize:
            if L.orc_finalize_setup(self.h):
                raise RuntimeError(L.orc_last_error(self.h).decode())

    def __del__(self):
        if getattr(self, "h", None):
            self.L.orc_destroy(self.h)
            self.h = None

    def _ncomp(self, field):
        nD = self.problem.options.n_dimensions
        return {capi.FIELD_CONSERVED: self.nU, capi.FIELD_ADJOINT: self.nU, capi.FIELD_TARGET: self.nU,
                capi.FIELD_RHS: self.nU, capi.FIELD_METRICS: nD * nD,
                capi.FIELD_ARC_LENGTHS: nD}.get(field, 1)

    def set_field(self, block, field, arr):
        a = np.ascontiguousarray(arr, dtype=np.float64)
        self.L.orc_set_field(self.h, block, field, capi.dptr(a))

    def get_field(self, block, field):
        n = self.problem.blocks[block - 1].n_points
        nc = self._ncomp(field)
        out = np.zeros((nc, n)) if nc > 1 else np.zeros(n)
        self.L.orc_get_field(self.h, block, field, capi.dptr(out))
        return out

    def update_state(self):
        self.L.orc_update_state(self.h)

    def compute_rhs(self, mode, time=0.0, adjoint_forcing_factor=1.0):
        if self.L.orc_compute_rhs(self.h, mode, time, adjoint_forcing_factor) != 0:
            raise RuntimeError(self.L.orc_last_error(self.h).decode())

    def update_adjoint_forcing(self, no_forcing=False):
        self.L.orc_update_adjoint_forcing(self.h, int(no_forcing))

    def functional(self):
        v = C.c_double()
        self.L.orc_compute_functional(self.h, C.byref(v))
        return v.value

    def sensitivity(self):
        v = C.c_double()
        self.L.orc_compute_sensitivity(self.h, C.byref(v))
        return v.value

    def rk4_substep(self, mode, time, dt, stage):
        t = C.c_double(time)
        self.L.orc_rk4_substep(self.h, mode, C.byref(t), dt, stage)
        return t.value

    def actuator_points(self):
        n = C.c_longlong()
        self.L.orc_actuator_patch_size(self.h, C.byref(n))
        return n.value

    def set_control_forcing(self, entries):
        a = np.ascontiguousarray(entries, dtype=np.float64)
        n = a.size // max(1, self.actuator_points())
        self.L.orc_set_control_forcing(self.h, capi.dptr(a), n)

    # status of the last run: capi.SOLUTION_LIMITS when it stopped at a
    # solution-limit violation (value HUGE), else 0
    run_status = 0

    def run_forward(self, n_steps, save_interval=10, t0=0.0, keep_stages=True):
        v = C.c_double()
        if keep_stages:
            self.run_status = self.L.orc_run_forward(self.h, n_steps, save_interval, t0, C.byref(v))
        else:
            self.run_status = self.L.orc_run_forward_nostore(self.h, n_steps, t0, C.byref(v))
        return v.value

    def run_adjoint(self):
        v = C.c_double()
        self.run_status = self.L.orc_run_adjoint(self.h, C.byref(v))
        return v.value

    def set_patch_control_forcing(self, forcing):
        if forcing is None:
            self.L.orc_set_patch_control_forcing(self.h, None)
        else:
            a = np.ascontiguousarray(forcing, dtype=np.float64)
            self.L.orc_set_patch_control_forcing(self.h, capi.dptr(a))

    def set_adjoint_nonzero_initial_condition(self, enable):
        self.L.orc_set_adjoint_nonzero_initial_condition(self.h, int(bool(enable)))

    def set_trajectory_storage(self, enable=True, max_bytes=0.0):
        """The oracle always recomputes checkpoint segments, as the reference
        does; the setting only mirrors the library's API (same results)."""

    def run_linearized(self, delta_forcing=None):
        """Tangent run; returns the tangent of the functional."""
        v = C.c_double()
        if delta_forcing is None:
            rc = self.L.orc_run_linearized(self.h, None, 0, C.byref(v))
        else:
            a = np.ascontiguousarray(delta_forcing, dtype=np.float64)
            rc = self.L.orc_run_linearized(self.h, capi.dptr(a), a.size // max(1, self.actuator_points()), C.byref(v))
        if rc != 0:
            raise RuntimeError(self.L.orc_last_error(self.h).decode())
        return v.value

    def time_step_size(self):
        v = C.c_double()
        self.L.orc_time_step_size(self.h, C.byref(v))
        return v.value

    def step_sizes(self, n_steps):
        out = np.zeros(max(1, n_steps))
        n = self.L.orc_step_sizes(self.h, capi.dptr(out))
        return out[:n]

    def gradient(self, n_entries):
        P = self.actuator_points()
        out = np.zeros(n_entries * P)
        self.L.orc_get_gradient(self.h, capi.dptr(out), n_entries)
        return out.reshape(n_entries, P)
