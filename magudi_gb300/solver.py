"""Python front end of the CUDA library (the counterpart of magudi's
Region/Solver driving, for users and tests). Every call goes through the C
ABI of include/magudi_gb300.h; there is no CPU path. If the library cannot be
loaded the constructor raises.
"""
import ctypes as C
import os

import numpy as np

from . import capi

_lib = None


class MagudiError(RuntimeError):
    pass


def library_path():
    from .build import LIB_PATH
    return LIB_PATH


def load_library(build_if_missing=True):
    """Loads libmagudi_gb300.so (building it first if it is missing)."""
    global _lib
    if _lib is not None:
        return _lib
    path = library_path()
    if not os.path.exists(path):
        if not build_if_missing:
            raise MagudiError(f"{path} is missing; run magudi_gb300.build.build()")
        from .build import build
        build()
    L = C.CDLL(path)
    ctx = C.c_void_p
    L.mgd_last_error.restype = C.c_char_p
    L.mgd_last_error.argtypes = [ctx]
    L.mgd_create.argtypes = [C.POINTER(capi.Options), C.POINTER(ctx)]
    L.mgd_destroy.argtypes = [ctx]
    L.mgd_add_block.argtypes = [ctx, C.POINTER(capi.BlockDesc), C.POINTER(C.c_double), C.POINTER(C.c_int)]
    L.mgd_add_patch.argtypes = [ctx, C.POINTER(capi.PatchDesc)]
    L.mgd_add_acoustic_source.argtypes = [ctx, C.POINTER(capi.AcousticSource)]
    L.mgd_set_field.argtypes = [ctx, C.c_int, C.c_int, C.POINTER(C.c_double)]
    L.mgd_get_field.argtypes = [ctx, C.c_int, C.c_int, C.POINTER(C.c_double)]
    L.mgd_finalize_setup.argtypes = [ctx]
    L.mgd_update_state.argtypes = [ctx]
    L.mgd_compute_rhs.argtypes = [ctx, C.c_int, C.c_double, C.c_double]
    L.mgd_update_adjoint_forcing.argtypes = [ctx, C.c_int]
    L.mgd_compute_functional.argtypes = [ctx, C.POINTER(C.c_double)]
    L.mgd_compute_sensitivity.argtypes = [ctx, C.POINTER(C.c_double)]
    L.mgd_rk4_substep.argtypes = [ctx, C.c_int, C.POINTER(C.c_double), C.c_double, C.c_int]
    L.mgd_set_control_forcing.argtypes = [ctx, C.POINTER(C.c_double), C.c_longlong]
    L.mgd_actuator_patch_size.argtypes = [ctx, C.POINTER(C.c_longlong)]
    L.mgd_run_forward.argtypes = [ctx, C.c_int, C.c_int, C.c_double, C.POINTER(C.c_double)]
    L.mgd_run_adjoint.argtypes = [ctx, C.POINTER(C.c_double)]
    L.mgd_set_adjoint_nonzero_initial_condition.argtypes = [ctx, C.c_int]
    L.mgd_set_patch_control_forcing.argtypes = [ctx, C.POINTER(C.c_double)]
    L.mgd_run_linearized.argtypes = [ctx, C.POINTER(C.c_double), C.c_longlong, C.POINTER(C.c_double)]
    L.mgd_get_gradient.argtypes = [ctx, C.POINTER(C.c_double), C.c_longlong]
    L.mgd_time_step_size.argtypes = [ctx, C.POINTER(C.c_double)]
    L.mgd_actuator_weights.argtypes = [ctx, C.POINTER(C.c_double)]
    L.mgd_save_solution.argtypes = [ctx, C.c_char_p, C.c_int, C.c_int, C.c_double]
    L.mgd_wait_io.argtypes = [ctx]
    L.mgd_load_solution.argtypes = [ctx, C.c_char_p, C.c_int, C.POINTER(C.c_double)]
    L.mgd_save_grid.argtypes = [ctx, C.c_char_p]
    L.mgd_save_gradient.argtypes = [ctx, C.c_char_p, C.c_longlong]
    L.mgd_load_control_forcing.argtypes = [ctx, C.c_char_p, C.c_longlong]
    L.mgd_control_zaxpy.argtypes = [ctx, C.c_double, C.c_int]
    L.mgd_batch_create.argtypes = [C.POINTER(ctx), C.c_int, C.POINTER(C.c_void_p)]
    L.mgd_batch_run_forward.argtypes = [C.c_void_p, C.c_int, C.c_double, C.POINTER(C.c_double)]
    L.mgd_batch_destroy.argtypes = [C.c_void_p]
    L.mgd_batch_last_error.restype = C.c_char_p
    L.mgd_batch_last_error.argtypes = [C.c_void_p]
    L.mgd_batch_kernel_launches.restype = C.c_longlong
    L.mgd_batch_kernel_launches.argtypes = [C.c_void_p, C.c_int]
    L.mgd_get_step_sizes.argtypes = [ctx, C.POINTER(C.c_double), C.c_int]
    L.mgd_profile_stage_kernels.argtypes = [ctx, C.c_int, C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_int)]
    L.mgd_stream.restype = C.c_void_p
    L.mgd_stream.argtypes = [ctx]
    L.mgd_kernel_launches.restype = C.c_longlong
    L.mgd_kernel_launches.argtypes = [ctx, C.c_int]
    L.mgd_gradient_lanes.restype = C.c_int
    L.mgd_gradient_lanes.argtypes = [ctx, C.c_int]
    L.mgd_adjoint_core_lanes.restype = C.c_int
    L.mgd_adjoint_core_lanes.argtypes = [ctx, C.c_int]
    L.mgd_dissipation_tma.restype = C.c_int
    L.mgd_dissipation_tma.argtypes = [ctx, C.c_int]
    L.mgd_set_trajectory_storage.restype = C.c_int
    L.mgd_set_trajectory_storage.argtypes = [ctx, C.c_int, C.c_double]
    L.mgd_tune_run.restype = C.c_int
    L.mgd_tune_run.argtypes = [ctx, C.c_int, C.c_int, C.c_int, C.POINTER(C.c_double)]
    L.mgd_stage_tile.restype = C.c_int
    L.mgd_stage_tile.argtypes = [ctx, C.c_int, C.POINTER(C.c_int), C.c_int]
    L.mgd_check_solution_limits.argtypes = [ctx, C.POINTER(C.c_int)]
    L.mgd_batch_persistent.restype = C.c_int
    L.mgd_batch_persistent.argtypes = [C.c_void_p, C.c_int]
    L.mgd_batch_persistent_grid.restype = C.c_int
    L.mgd_batch_persistent_grid.argtypes = [C.c_void_p]
    L.mgd_selftest_fp64_rate.restype = C.c_int
    L.mgd_selftest_fp64_rate.argtypes = [C.c_int, C.POINTER(C.c_double)]
    L.mgd_selftest_grid_barrier.restype = C.c_int
    L.mgd_selftest_grid_barrier.argtypes = [C.c_int, C.c_int, C.c_int, C.c_longlong, C.POINTER(C.c_int),
                                            C.POINTER(C.c_longlong)]
    _lib = L
    return L


class Solver:
    """One region on the current CUDA device, built from a Problem."""

    def __init__(self, problem, finalize=True):
        self.L = load_library()
        self.problem = problem
        self.nU = problem.n_unknowns
        self._opts = problem.options.to_c()
        h = C.c_void_p()
        if self.L.mgd_create(C.byref(self._opts), C.byref(h)):
            raise MagudiError(self.L.mgd_last_error(None).decode())
        self.h = h
        for blk in problem.blocks:
            coords = np.ascontiguousarray(blk.coordinates, dtype=np.float64)
            ib = blk.iblank_array()
            d = blk.desc()
            self._check(self.L.mgd_add_block(self.h, C.byref(d), capi.dptr(coords), capi.iptr(ib)))
        for p in problem.patches:
            pd = p.to_c()
            self._check(self.L.mgd_add_patch(self.h, C.byref(pd)))
        for s in problem.sources:
            sd = s.to_c()
            self._check(self.L.mgd_add_acoustic_source(self.h, C.byref(sd)))
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
            self._check(self.L.mgd_finalize_setup(self.h))

    # the message of the last run that stopped at a solution-limit violation
    limit_violation = None

    def _check(self, rc):
        if rc:
            raise MagudiError(self.L.mgd_last_error(self.h).decode())

    def _run_status(self, rc):
        """Runs return HUGE (not an exception) when the solution left the
        limits, as Solver%runForward / runAdjoint do; the message is kept in
        limit_violation."""
        if rc == capi.SOLUTION_LIMITS:
            self.limit_violation = self.L.mgd_last_error(self.h).decode()
            return
        self.limit_violation = None
        self._check(rc)

    def close(self):
        if getattr(self, "h", None):
            self.L.mgd_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def _ncomp(self, field):
        nD = self.problem.options.n_dimensions
        return {capi.FIELD_CONSERVED: self.nU, capi.FIELD_ADJOINT: self.nU, capi.FIELD_TARGET: self.nU,
                capi.FIELD_RHS: self.nU, capi.FIELD_METRICS: nD * nD,
                capi.FIELD_ARC_LENGTHS: nD}.get(field, 1)

    def set_field(self, block, field, arr):
        a = np.ascontiguousarray(arr, dtype=np.float64)
        self._check(self.L.mgd_set_field(self.h, block, field, capi.dptr(a)))

    def get_field(self, block, field):
        n = self.problem.blocks[block - 1].n_points
        nc = self._ncomp(field)
        out = np.zeros((nc, n)) if nc > 1 else np.zeros(n)
        self._check(self.L.mgd_get_field(self.h, block, field, capi.dptr(out)))
        return out

    def update_state(self):
        self._check(self.L.mgd_update_state(self.h))

    def compute_rhs(self, mode, time=0.0, adjoint_forcing_factor=1.0):
        self._check(self.L.mgd_compute_rhs(self.h, mode, time, adjoint_forcing_factor))

    def update_adjoint_forcing(self, no_forcing=False):
        self._check(self.L.mgd_update_adjoint_forcing(self.h, int(no_forcing)))

    def functional(self):
        v = C.c_double()
        self._check(self.L.mgd_compute_functional(self.h, C.byref(v)))
        return v.value

    def sensitivity(self):
        v = C.c_double()
        self._check(self.L.mgd_compute_sensitivity(self.h, C.byref(v)))
        return v.value

    def rk4_substep(self, mode, time, dt, stage):
        t = C.c_double(time)
        self._check(self.L.mgd_rk4_substep(self.h, mode, C.byref(t), dt, stage))
        return t.value

    def actuator_points(self):
        n = C.c_longlong()
        self._check(self.L.mgd_actuator_patch_size(self.h, C.byref(n)))
        return n.value

    def set_control_forcing(self, entries):
        a = np.ascontiguousarray(entries, dtype=np.float64)
        n = a.size // max(1, self.actuator_points())
        self._check(self.L.mgd_set_control_forcing(self.h, capi.dptr(a), n))

    def run_forward(self, n_steps, save_interval=10, t0=0.0):
        v = C.c_double()
        self._run_status(self.L.mgd_run_forward(self.h, n_steps, save_interval, t0, C.byref(v)))
        return v.value

    def run_adjoint(self):
        v = C.c_double()
        self._run_status(self.L.mgd_run_adjoint(self.h, C.byref(v)))
        return v.value

    def check_solution_limits(self):
        """checkSolutionLimits of the current state: True when inside the
        limits, else False with the message in limit_violation."""
        w = C.c_int()
        self._check(self.L.mgd_check_solution_limits(self.h, C.byref(w)))
        self.limit_violation = None if w.value else self.L.mgd_last_error(self.h).decode()
        return bool(w.value)

    def run_linearized(self, delta_forcing=None):
        """Tangent run over the steps of the last run_forward: the perturbation
        in FIELD_ADJOINT advances along the checkpointed trajectory, the
        actuators adding the control perturbation delta_forcing (entries x
        actuator points, or None). Returns the tangent of the functional."""
        v = C.c_double()
        if delta_forcing is None:
            self._check(self.L.mgd_run_linearized(self.h, None, 0, C.byref(v)))
        else:
            a = np.ascontiguousarray(delta_forcing, dtype=np.float64)
            n = a.size // max(1, self.actuator_points())
            self._check(self.L.mgd_run_linearized(self.h, capi.dptr(a), n, C.byref(v)))
        return v.value

    def set_patch_control_forcing(self, forcing):
        """The actuator patches' forcing for the per-call forward RHS (P values), or None."""
        if forcing is None:
            self._check(self.L.mgd_set_patch_control_forcing(self.h, None))
        else:
            a = np.ascontiguousarray(forcing, dtype=np.float64)
            self._check(self.L.mgd_set_patch_control_forcing(self.h, capi.dptr(a)))

    def set_adjoint_nonzero_initial_condition(self, enable):
        """adjoint_nonzero_initial_condition: run_adjoint starts from the adjoint
        field held (set_field(..., FIELD_ADJOINT, ...)) instead of zero."""
        self._check(self.L.mgd_set_adjoint_nonzero_initial_condition(self.h, int(bool(enable))))

    def gradient(self, n_entries):
        P = self.actuator_points()
        out = np.zeros(n_entries * P)
        self._check(self.L.mgd_get_gradient(self.h, capi.dptr(out), n_entries))
        return out.reshape(n_entries, P)

    def time_step_size(self):
        """Region%getTimeStepSize of the current conserved variables."""
        v = C.c_double()
        self._check(self.L.mgd_time_step_size(self.h, C.byref(v)))
        return v.value

    def step_sizes(self, n_steps):
        """Step sizes of the steps of the last run_forward."""
        out = np.zeros(max(1, n_steps))
        self._check(self.L.mgd_get_step_sizes(self.h, capi.dptr(out), n_steps))
        return out[:n_steps]

    # files (PLOT3D solutions and grids, actuator-patch streams)
    def save_solution(self, filename, field=capi.FIELD_CONSERVED, timestep=0, time=0.0):
        """Asynchronous: the file is written by a host thread; wait_io() joins it."""
        self._check(self.L.mgd_save_solution(self.h, str(filename).encode(), field, timestep, time))

    def wait_io(self):
        self._check(self.L.mgd_wait_io(self.h))

    def load_solution(self, filename, field=capi.FIELD_CONSERVED):
        t = C.c_double()
        self._check(self.L.mgd_load_solution(self.h, str(filename).encode(), field, C.byref(t)))
        return t.value

    def save_grid(self, filename):
        self._check(self.L.mgd_save_grid(self.h, str(filename).encode()))

    def save_gradient(self, prefix, n_entries):
        self._check(self.L.mgd_save_gradient(self.h, str(prefix).encode(), n_entries))

    def load_control_forcing(self, prefix, n_entries):
        self._check(self.L.mgd_load_control_forcing(self.h, str(prefix).encode(), n_entries))

    def control_zaxpy(self, a, accumulate=False):
        """Control forcing = a * gradient (+ forcing) on the device."""
        self._check(self.L.mgd_control_zaxpy(self.h, a, int(accumulate)))

    def profile_stage_kernels(self, mode, reps=20):
        """Mean per-launch milliseconds of each kernel of one RK stage."""
        out = (C.c_double * 8)()
        n = C.c_int()
        self._check(self.L.mgd_profile_stage_kernels(self.h, mode, reps, out, C.byref(n)))
        return list(out)[: n.value]

    def stream_handle(self):
        return self.L.mgd_stream(self.h)

    def kernel_launches(self, reset=False):
        return self.L.mgd_kernel_launches(self.h, int(reset))

    def set_trajectory_storage(self, enable=True, max_bytes=0.0):
        """Store every RK stage of the forward run on the device (when it fits
        in max_bytes, <= 0: half the free device memory) so that run_adjoint
        reads the trajectory instead of recomputing checkpoint segments."""
        self._check(self.L.mgd_set_trajectory_storage(self.h, int(bool(enable)), float(max_bytes)))

    def tune_run(self, n_steps, save_interval, with_adjoint=True):
        """Run-level autotuning of the stage-kernel tiles on short checkpointed
        runs from the current state (which is restored). Returns the tuned
        run's wall time in ms."""
        v = C.c_double()
        self._check(self.L.mgd_tune_run(self.h, int(n_steps), int(save_interval), int(bool(with_adjoint)),
                                        C.byref(v)))
        return v.value

    def stage_tile(self, kernel, tile=None):
        """Tile (points per CTA along x, y, z) of stage kernel `kernel` (0..5):
        returns the current one, or sets `tile` first."""
        t = (C.c_int * 3)(*(tile or (0, 0, 0)))
        self._check(self.L.mgd_stage_tile(self.h, int(kernel), t, 1 if tile else 0))
        if tile:
            self._check(self.L.mgd_stage_tile(self.h, int(kernel), t, 0))
        return tuple(t)

    def dissipation_tma(self, mode=-1):
        """Composite dissipation of fully periodic 3D blocks staged by the
        tensor memory accelerator (1) or read through L1 (0); -1 reports."""
        r = self.L.mgd_dissipation_tma(self.h, int(mode))
        if r < 0:
            raise MagudiError(self.L.mgd_last_error(self.h).decode())
        return r

    def adjoint_core_lanes(self, lanes=0):
        """Form of the 2D adjoint core: 1 or 2 threads per point (lanes = 0
        reports it, 1 or 2 sets it)."""
        r = self.L.mgd_adjoint_core_lanes(self.h, int(lanes))
        if r < 0:
            raise MagudiError(self.L.mgd_last_error(self.h).decode())
        return r

    def gradient_lanes(self, lanes=0):
        """Form of the 2D gradient/flux kernel: 1 or 2 threads per point
        (lanes = 0 reports the autotuned form, 1 or 2 sets it)."""
        r = self.L.mgd_gradient_lanes(self.h, int(lanes))
        if r < 0:
            raise MagudiError(self.L.mgd_last_error(self.h).decode())
        return r


class Batch:
    """Forward runs of many Solvers at once (mgd_batch_*): by default all
    steps of every instance in one persistent cooperative launch (captured in
    a CUDA graph); persistent(0) switches to one graph of batched stage
    kernels per RK4 step. The solvers keep their own grids, states and
    control forcings."""

    def __init__(self, solvers):
        self.L = load_library()
        self.solvers = list(solvers)
        arr = (C.c_void_p * len(self.solvers))(*[s.h for s in self.solvers])
        h = C.c_void_p()
        if self.L.mgd_batch_create(C.cast(arr, C.POINTER(C.c_void_p)), len(self.solvers), C.byref(h)):
            raise MagudiError(self.L.mgd_batch_last_error(None).decode())
        self.h = h

    def run_forward(self, n_steps, t0=0.0):
        costs = np.zeros(len(self.solvers))
        if self.L.mgd_batch_run_forward(self.h, n_steps, t0, capi.dptr(costs)):
            raise MagudiError(self.L.mgd_batch_last_error(self.h).decode())
        return costs

    def kernel_launches(self, reset=False):
        return self.L.mgd_batch_kernel_launches(self.h, int(reset))

    def persistent(self, mode=None):
        """The run mode: 1 persistent single launch, 0 one graph per step
        (mode None only reports)."""
        return self.L.mgd_batch_persistent(self.h, -1 if mode is None else int(mode))

    def persistent_grid(self):
        return self.L.mgd_batch_persistent_grid(self.h)

    def close(self):
        if getattr(self, "h", None):
            self.L.mgd_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()
