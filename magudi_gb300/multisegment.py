"""Multi-segment (time-split) forward and adjoint runs: bin/msforward.f90 and
bin/msadjoint.f90 over one context per segment.

The horizon of n_segments * segment_length RK4 steps is split into segments
that each start from their own initial condition. Segment k runs
segment_length steps from ic_k (ic_0 is the problem's initial state) with the
slice of the global control-forcing stream that covers its steps. The cost is

    J = sum_k J_k + penalty_weight * penalty(sum_{k>=1} ||ic_k - end_{k-1}||^2_H)

with the quadratic norm 0.5 s or the Huber norm (src/MSPenaltyImpl.f90).
The adjoint runs every segment backward from its terminal condition
penalty_scale * (end_k - ic_{k+1}) (zero for the last segment). It uses
adjoint_nonzero_initial_condition and returns the segments' control
gradients and the initial-condition gradients
lambda_{k+1}(0) + penalty_scale * (ic_{k+1} - end_k). An optional state
mollifier w blends each initial condition with the previous segment's end
state, as the reference's time_splitting/state_mollifier does.

Segments are independent given their initial conditions, so their forward
runs, and later their adjoint runs, are issued from one host thread per
segment context. Each context has its own CUDA streams, so the segments run
concurrently on the GPU. Between the two passes the driver does the
reference's array algebra on the host: mismatches, inner products and
terminal conditions.
"""
from concurrent.futures import ThreadPoolExecutor
from dataclasses import dataclass, field
from typing import List, Optional

import numpy as np

from . import capi


def penalty_norm(kind, l2sq, threshold):
    """t_QuadraticPenalty%norm / t_HuberPenalty%norm (src/MSPenaltyImpl.f90)."""
    if kind == "quadratic":
        return 0.5 * l2sq
    l2 = np.sqrt(l2sq)
    return l2 - 0.5 * threshold if l2 >= threshold else 0.5 * l2sq / threshold


def penalty_gradient_factor(kind, l2sq, threshold):
    """gradientFactor of the quadratic (1) and Huber (max(||.||, threshold)) norms."""
    if kind == "quadratic":
        return 1.0
    l2 = np.sqrt(l2sq)
    return l2 if l2 >= threshold else threshold


@dataclass
class ForwardResult:
    J: float
    time_integral: float
    penalty: float
    segment_costs: List[float]
    segment_l2sq: List[float]


@dataclass
class AdjointResult:
    total: float                      # sum of the control and initial-condition inner products
    segment_control_ip: List[float]   # runAdjoint's value per segment
    segment_ic_ip: List[float]        # <dJ/d ic_k, dJ/d ic_k>_H (0 for segment 0)
    ic_gradients: list = field(default_factory=list)  # per segment: per-block arrays (None for segment 0)
    gradient: Optional[np.ndarray] = None  # control gradient entries of the whole horizon, file order


class MultiSegment:
    """msforward / msadjoint over per-segment contexts (Solver, or any object
    with the same methods)."""

    def __init__(self, problem, n_segments, segment_length, penalty_weight, penalty_type="quadratic",
                 huber_threshold=1e-12, state_mollifier=None, start_time=0.0, save_interval=None,
                 backend=None, concurrent=True, store_trajectory=False):
        if penalty_type not in ("quadratic", "huber"):
            raise ValueError(f"Unknown time_splitting/penalty_type '{penalty_type}': expected 'quadratic' or 'huber'.")
        if n_segments < 1 or segment_length < 1:
            raise ValueError("number_of_segments and segment_length must be >= 1")
        if problem.options.use_constant_cfl:
            raise ValueError("multi-segment runs use a constant time_step_size")
        if backend is None:
            from .solver import Solver
            backend = Solver
        self.problem = problem
        self.n_segments, self.nts = n_segments, segment_length
        self.weight, self.kind, self.threshold = penalty_weight, penalty_type, huber_threshold
        self.mollifier = state_mollifier  # per-block arrays (N,) or None
        self.t_start = start_time
        self.save_interval = save_interval or max(1, int(round(segment_length ** 0.5)))
        self.concurrent = concurrent
        self.ctx = [backend(problem) for _ in range(n_segments)]
        if store_trajectory:
            # each segment's forward run keeps its stages on the device for its adjoint run
            for c in self.ctx:
                c.set_trajectory_storage(True)
        self.n_blocks = len(problem.blocks)
        self.norms = [np.asarray(self.ctx[0].get_field(b, capi.FIELD_NORM)).reshape(-1)
                      for b in range(1, self.n_blocks + 1)]
        self.P = self.ctx[0].actuator_points()
        self._forcing = None
        self._ics = None
        self._ends = None

    # --- helpers ---------------------------------------------------------
    def _map(self, fn, items):
        if self.concurrent and len(items) > 1:
            with ThreadPoolExecutor(max_workers=len(items)) as ex:
                return list(ex.map(fn, items))
        return [fn(i) for i in items]

    def _inner(self, x, y, weighted):
        """Grid%computeInnerProduct over every block (src/GridImpl.f90:1118-1170)."""
        s = 0.0
        for b in range(self.n_blocks):
            w = self.norms[b] * (self.mollifier[b] if (weighted and self.mollifier is not None) else 1.0)
            s += float(np.sum(x[b] * w * y[b]))
        return s

    def _time(self, k):
        return self.t_start + k * self.nts * self.problem.options.time_step_size

    def _slice(self, k):
        """Entries of segment k in the global file-order stream (controlTimestepOffset = k * nts)."""
        total = self.n_segments * self.nts
        lo = 4 * (total - (k + 1) * self.nts)
        return slice(lo, lo + 4 * self.nts)

    def set_control_forcing(self, entries):
        """Control forcing of the whole horizon, 4 * n_segments * segment_length entries in file order."""
        a = np.asarray(entries, dtype=np.float64).reshape(4 * self.n_segments * self.nts, max(1, self.P))
        self._forcing = a

    # --- msforward -------------------------------------------------------
    def forward(self, ics=None):
        """ics[k] (k >= 1): per-block conserved states of segment k's initial
        condition; ics[0] and missing entries use the problem's initial state."""
        K = self.n_segments
        init = [b.initial_state for b in self.problem.blocks]
        self._ics = [init] + [list(ics[k]) if ics is not None and ics[k] is not None else init for k in range(1, K)]
        # every segment from its own initial condition: blending with the
        # previous end state needs that end state, so blended segments wait
        costs = [0.0] * K
        ends = [None] * K

        def run(k, start):
            c = self.ctx[k]
            for b in range(self.n_blocks):
                c.set_field(b + 1, capi.FIELD_CONSERVED, start[b])
            if self._forcing is not None:
                c.set_control_forcing(self._forcing[self._slice(k)])
            costs[k] = c.run_forward(self.nts, self.save_interval, self._time(k))
            ends[k] = [np.asarray(c.get_field(b + 1, capi.FIELD_CONSERVED)) for b in range(self.n_blocks)]

        if self.mollifier is None:
            self._map(lambda k: run(k, self._ics[k]), list(range(K)))
        else:
            run(0, self._ics[0])
            for k in range(1, K):
                run(k, self._blended(k, ends[k - 1]))
        l2 = [0.0] * K
        for k in range(1, K):
            d = [self._ics[k][b] - ends[k - 1][b] for b in range(self.n_blocks)]
            l2[k] = self._inner(d, d, weighted=True)
        self._ends = ends
        self._l2sum = sum(l2)
        ti = sum(costs)
        pen = self.weight * penalty_norm(self.kind, self._l2sum, self.threshold)
        return ForwardResult(ti + pen, ti, pen, costs, l2)

    def _blended(self, k, end_prev):
        """ic_k - (1 - w) (ic_k - end_{k-1}) (msforward's state-mollifier blend)."""
        out = []
        for b in range(self.n_blocks):
            w = self.mollifier[b]
            out.append(self._ics[k][b] - (1.0 - w) * (self._ics[k][b] - end_prev[b]))
        return out

    # --- msadjoint -------------------------------------------------------
    def adjoint(self):
        """Adjoint of the last forward(): every segment backward from its
        terminal condition, on the checkpoints its context kept from forward()."""
        if self._ends is None:
            raise RuntimeError("adjoint() needs a preceding forward()")
        K = self.n_segments
        scale = self.weight / penalty_gradient_factor(self.kind, self._l2sum, self.threshold)
        ctrl = [0.0] * K
        lam0 = [None] * K
        ic_grad = [None] * K
        icip = [0.0] * K
        grads = [None] * K

        def run(k, terminal):
            c = self.ctx[k]
            if terminal is None:
                c.set_adjoint_nonzero_initial_condition(False)
            else:
                for b in range(self.n_blocks):
                    c.set_field(b + 1, capi.FIELD_ADJOINT, terminal[b])
                c.set_adjoint_nonzero_initial_condition(True)
            ctrl[k] = c.run_adjoint()
            c.set_adjoint_nonzero_initial_condition(False)
            lam0[k] = [np.asarray(c.get_field(b + 1, capi.FIELD_ADJOINT)) for b in range(self.n_blocks)]
            if self.P > 0:
                grads[k] = c.gradient(4 * self.nts)

        def terminal_of(k):
            # terminal_k = scale (end_k - ic_{k+1}); with the mollifier
            # w scale (end_k - ic_{k+1}) + (1 - w) lambda_{k+1}(0)
            t = []
            for b in range(self.n_blocks):
                x = scale * (self._ends[k][b] - self._ics[k + 1][b])
                if self.mollifier is not None:
                    w = self.mollifier[b]
                    x = w * x + (1.0 - w) * lam0[k + 1][b]
                t.append(x)
            return t

        if self.mollifier is None:
            # terminal conditions need only the forward results: all segments at once
            self._map(lambda k: run(k, None if k == K - 1 else terminal_of(k)), list(range(K)))
        else:
            run(K - 1, None)
            for k in range(K - 2, -1, -1):
                run(k, terminal_of(k))
        for k in range(1, K):
            g = []
            for b in range(self.n_blocks):
                x = lam0[k][b] + scale * (self._ics[k][b] - self._ends[k - 1][b])
                if self.mollifier is not None:
                    x = self.mollifier[b] * x
                g.append(x)
            ic_grad[k] = g
            icip[k] = self._inner(g, g, weighted=False)
        gradient = None
        if self.P > 0:
            gradient = np.zeros((4 * K * self.nts, self.P))
            for k in range(K):
                gradient[self._slice(k)] = grads[k]
        return AdjointResult(sum(ctrl) + sum(icip), ctrl, icip, ic_grad, gradient)
