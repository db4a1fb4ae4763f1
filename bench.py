"""Benchmark of the magudi hot path on one GB300.

Workload (one "step"): the 2D acoustic monopole, 201x201 grid on [-14,14]^2,
FP64 viscous Navier-Stokes with SBP 4-8 derivatives and dissipation,
far-field SATs, 20-point sponges, a Gaussian cost target and control
mollifier; 960 RK4 steps forward (dt = 0.05) with a snapshot every 10 steps,
then the discrete adjoint over the same horizon with uniform checkpointing
(each 10-step segment's forward states recomputed on the device from its
snapshot, beside the adjoint) -- one complete forward + adjoint gradient
evaluation. The same gradient with the whole trajectory kept resident on the
device (no recomputation) is timed after it and reported as a secondary
figure (`resident_trajectory`).

Metric: FP64 Mpt-RHS/s = grid points x (forward + adjoint RHS evaluations)
/ seconds / 1e6 (the forward recomputation of checkpointing is not counted).
`value` is device-timed (CUDA events on the library's stream) with the
initial state already in HBM; `e2e` is the same metric through the C ABI
with the initial state uploaded from pinned host memory and the gradient
vector, J and Grad0 read back each step.

The CPU baseline and --impl reference run the CPU restatement of the
reference (oracle/; the Fortran reference cannot be built: it needs an MPI
Fortran toolchain and CMake-generated headers) on the host cores over the
complete workload: every timed step is the whole 960-step forward + adjoint
gradient. The bench line's `parity` compares the GPU's J, Grad0 and gradient
vector with that CPU run.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

GRID = 201
N_STEPS = 960
SAVE_INTERVAL = 10
WORKLOAD = ("2D acoustic monopole 201x201, FP64 viscous NS, SBP 4-8 + dissipation 0.01, far-field SAT + "
            "20-pt sponge, forward 960 RK4 steps (dt 0.05) + discrete adjoint gradient, checkpoints every 10 steps")


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cpu-warmup-rk-steps", type=int, default=20,
                    help="RK4 steps of each warm-up sample of the CPU legs (--impl reference)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-other-workloads", action="store_true",
                    help="skip the Taylor-Green and jet samples of the default line")
    ap.add_argument("--rk-steps", type=int, default=N_STEPS,
                    help="RK4 steps per gradient evaluation (profiling runs use a few)")
    ap.add_argument("--workload", default="gradient",
                    choices=["gradient", "sweep", "tgv", "jet", "msgrad", "tangent", "fdcheck"],
                    help="gradient: the forward + adjoint gradient evaluation (default); sweep: the batched "
                         "gradient-check sweep of 64 monopole instances of mixed grid sizes; tgv: the 3D "
                         "Taylor-Green vortex forward + adjoint (terminal kinetic energy, constant CFL); jet: "
                         "the three-block curvilinear 3D jet forward + adjoint; msgrad: the monopole gradient with "
                         "the 960 steps split into --ms-segments time segments run concurrently; tangent: the "
                         "monopole forward run followed by the linearized (tangent) run along it; fdcheck: the "
                         "reference's gradient-accuracy table at 201x201 x 960 steps, the 20 amplitudes as one batch")
    ap.add_argument("--ms-segments", type=int, default=8)
    ap.add_argument("--tgv-n", type=int, default=256)
    ap.add_argument("--tgv-steps", type=int, default=10, help="RK4 steps of the Taylor-Green sample (of the 2000-step run)")
    ap.add_argument("--dissipation-tma", type=int, default=-1, choices=[-1, 0, 1],
                    help="tgv workload: composite dissipation staged by the tensor memory accelerator (1) or read "
                         "through L1 (0); -1 keeps the library's default")
    ap.add_argument("--jet-steps", type=int, default=8, help="RK4 steps of the jet sample (of the 1000-step run)")
    ap.add_argument("--jet-save-interval", type=int, default=4)
    ap.add_argument("--jet-scale", type=float, default=1.0, help="grid scale of the jet (1 = 39.4 M points)")
    ap.add_argument("--sweep-instances", type=int, default=64)
    ap.add_argument("--sweep-per-call-sample", type=int, default=4,
                    help="instances timed through the per-call entry points beside the batch")
    ap.add_argument("--tiles", default=None,
                    help="stage-kernel tiles instead of run-level tuning, e.g. 8x16x1,8x8x1,8x16x1,8x8x1,8x8x1,16x4x1 "
                         "(gradient/flux, dissipation, divergence, adjoint core, diffusion, assembly), as a bench "
                         "line's config.tile_tuning.tiles reports them")
    ap.add_argument("--grad-lanes", type=int, default=0, help="with --tiles: 2D gradient/flux threads per point")
    ap.add_argument("--core-lanes", type=int, default=0, help="with --tiles: 2D adjoint core threads per point")
    ap.add_argument("--checkpoint-only", action="store_true",
                    help="msgrad and tangent workloads: recompute checkpoint segments instead of keeping the "
                         "trajectory on the device")
    ap.add_argument("--resident", action="store_true",
                    help="gradient workload: time the resident trajectory (no recomputation) as the primary figure; "
                         "by default the checkpoint recomputation is primary and the resident trajectory secondary")
    ap.add_argument("--profile-only", action="store_true",
                    help="run the gradient evaluations and exit (for ncu captures; prints no bench line)")
    return ap.parse_args()


def progress(msg):
    """One line on stderr per phase, so that a run that stops part way shows where."""
    print(f"[bench {time.strftime('%H:%M:%S')}] {msg}", file=sys.stderr, flush=True)


def rank_info():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("LOCAL_RANK", "0"))


def problem(n_steps=N_STEPS):
    from magudi_gb300 import configs
    return configs.monopole_2d(n=GRID, n_steps=n_steps, save_interval=SAVE_INTERVAL)


def _tuned_flags():
    try:
        return open(os.path.join(ROOT, "oracle", "_build", "tuned_flags.txt")).read().strip()
    except OSError:
        return ""


CPU_LEGS = {
    "strict": "oracle/oracle.cpp built -O3 -fno-fast-math -ffp-contract=off -fopenmp (the parity checker)",
    "tuned": ("oracle/oracle.cpp built with the reference's release flags -O3 -ffast-math -funroll-loops "
              + (_tuned_flags() + " " if _tuned_flags() else "") + "-fopenmp"),
}


def cpu_model():
    try:
        for line in open("/proc/cpuinfo"):
            if line.lower().startswith(("model name", "cpu part")):
                return line.split(":", 1)[1].strip()
    except OSError:
        pass
    import platform
    return platform.machine()


def cpu_gradient(variant="strict", steps=N_STEPS, threads=None, want_vector=False):
    """Runs the CPU oracle over `steps` RK4 steps forward + adjoint of the
    201x201 monopole (the full workload at steps = 960) on all host cores;
    returns seconds, Mpt-RHS/s, J, Grad0 and (optionally) the gradient vector."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import oracle_lib
    cores = threads or os.cpu_count()
    oracle_lib.set_threads(cores, variant)
    P = problem(steps)
    o = oracle_lib.Oracle(P, variant=variant)
    t = time.perf_counter()
    J = o.run_forward(steps, SAVE_INTERVAL)
    G = o.run_adjoint()
    dt = time.perf_counter() - t
    out = {"seconds": dt, "value": P.blocks[0].n_points * 8 * steps / dt / 1e6, "J": J, "grad0": G,
           "cores": cores, "variant": variant}
    if want_vector:
        out["gradient"] = o.gradient(4 * steps)
    del o
    return out


def parity_of(J, G, grad, ref):
    """Relative differences of the GPU's J, Grad0 and gradient vector from the
    strict oracle's complete run of the same workload."""
    import numpy as np
    return {"J_rel": abs(J - ref["J"]) / abs(ref["J"]), "grad0_rel": abs(G - ref["grad0"]) / abs(ref["grad0"]),
            "gradient_vector_rel": float(np.linalg.norm(grad - ref["gradient"]) / np.linalg.norm(ref["gradient"])),
            "tolerance": 1e-10, "against": "strict CPU oracle, complete 960-step forward + adjoint run"}


class ClockSampler:
    """nvidia-smi clock and throttle sampling during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self):
        self.proc = None
        # raw samples; the JSON line carries their summary (MGD_CLOCKS_CSV keeps a copy elsewhere)
        self.path = os.environ.get("MGD_CLOCKS_CSV", os.path.join(tempfile.gettempdir(), "mgd_clocks.csv"))

    def start(self):
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.QUERY}", "--format=csv,noheader,nounits",
                                          "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        self.proc.wait()
        self.f.close()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def fp64_peak(torch, clocks):
    """FP64 roof of this GPU: a cuBLAS DGEMM 6144^3 (best of 8 after a
    warm-up), and beside it the nominal rate of the SMs' FP64 pipes (4 flops
    per clock per SM: 2 DFMA lane-operations) at the sampled maximum clock."""
    n = 6144
    a = torch.randn(n, n, dtype=torch.float64, device="cuda")
    b = torch.randn(n, n, dtype=torch.float64, device="cuda")
    torch.matmul(a, b)
    best = 1e30
    for _ in range(8):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        torch.matmul(a, b)
        e1.record()
        torch.cuda.synchronize()
        best = min(best, e0.elapsed_time(e1) / 1e3)
    sms = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
    mhz = (clocks or {}).get("sm_max_mhz") or 2070.0
    return {"peak_tflops": 2.0 * n ** 3 / best / 1e12, "source": "measured: cuBLAS DGEMM 6144^3, best of 8",
            "nominal_tflops": sms * 4 * mhz * 1e6 / 1e12, "pipe_probe": fp64_pipe_probe()}


def fp64_pipe_probe():
    """DFMA lane-operations per clock per SM with 1, 2, 3, 4 and 8 warps on
    every SM (mgd_selftest_fp64_rate): how the FP64 rate splits over the
    SM's sub-partitions, which sets the floor of a kernel with few warps."""
    import ctypes as C
    from magudi_gb300.solver import load_library
    L = load_library()
    rates = {}
    for w in (1, 2, 3, 4, 8):
        r = C.c_double()
        if L.mgd_selftest_fp64_rate(w, C.byref(r)) == 0:
            rates[str(w)] = round(r.value, 3)
    return {"dfma_lane_ops_per_clock_per_sm_by_warps_per_sm": rates,
            "source": "mgd_selftest_fp64_rate: one CTA per SM, 4 independent DFMA chains per thread"}


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        return json.load(open(path)), "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


# Algorithmic traffic and FP64 operations per grid point of each stage kernel
# on the 2D viscous Cartesian workload (each array element that the kernel
# needs read or written once; stencil neighbours are re-reads, not counted).
# bytes: doubles x 8 plus int32 index words x 4. flops: the FP64 operations
# the kernel executes per point on the 201x201 grid, counted by ncu
# (2 x DFMA + DADD + DMUL over the launch, divided by the points; the kernels
# evaluate each term of their operation list once, boundary closure rows
# included).
KERNEL_UNITS = {
    # q 4, prim (u 2, p, T, mu, la, k) 7, metric diagonal 2, jac 1; writes fhat 8; ffOfPoint 3 ints
    "forward_gradient_flux": {"bytes": 8 * (4 + 7 + 2 + 1 + 8) + 4 * 3, "flops": 122},
    # q 4 read, dq 4 written
    "forward_dissipation": {"bytes": 8 * (4 + 4), "flops": 122},
    # fhat 8, dq 4, jac 1, q 4, qt 4, sponge 1, srcG 1, b1 4, b2 4 read; b2 4, q 4 written; ffOfPoint 3 + iblank 1 ints
    "forward_divergence_rk": {"bytes": 8 * (8 + 4 + 1 + 4 + 4 + 1 + 1 + 4 + 4 + 4 + 4) + 4 * 4, "flops": 118},
    # q 4 read, prim 8 written
    "forward_primitives": {"bytes": 8 * (4 + 8), "flops": 69},
    # lambda 4, metric diagonal 2, prim (u 2, v, T, mu, la, k) 7, tau 4, hf 2, jac 1 read; rcore 4, ad 6 written
    "adjoint_core": {"bytes": 8 * (4 + 2 + 7 + 4 + 2 + 1 + 4 + 6) + 4 * 3, "flops": 469},
    # lambda 4 read, dq 4 written
    "adjoint_dissipation": {"bytes": 8 * (4 + 4), "flops": 122},
    # ad 6 read, t2 3 written
    "adjoint_diffusion": {"bytes": 8 * (6 + 3), "flops": 84},
    # rcore 4, prim (v, u 2) 3, q_E 1, t2 3, dq 4, jac 1, lambda 4, sponge 1, tgtCount 1, b1 4, b2 4 read;
    # b2 4, lambda 4 written; ffOfPoint 3 + iblank 1 ints
    "adjoint_assemble_rk": {"bytes": 8 * (4 + 3 + 1 + 3 + 4 + 1 + 4 + 1 + 1 + 4 + 4 + 4 + 4) + 4 * 4, "flops": 47},
}
# Algorithmic FP64 operations per grid point of the 201x201 monopole RHS:
# the reference's operation list as the oracle restates it, counted by the
# operation-counting build of the oracle (oracle/build_opcount.sh; adds,
# multiplies, divides and square roots; tests/test_opcount.py recounts them).
# adjoint_core is the part of computeRhsAdjoint that the adjoint-core kernel
# performs (adjoint derivatives of lambda, the (A - B1)^T and B2^T products);
# the GPU kernels evaluate the same terms with fewer operations (the
# executed counts are in KERNEL_UNITS), so a rate over these counts is the
# reference-equivalent FP64 rate. forward_gradient_flux is the part of
# updateState after the transport variables (velocity and temperature
# gradients, stress, heat flux: 95.7) plus the part of computeRhsForward
# before the derivatives (Cartesian fluxes and their transform: 34.0), which
# the gradient/flux kernel performs.
ALGORITHMIC_FLOPS = {"forward_rhs": 406.8, "adjoint_rhs": 1073.2, "adjoint_core": 725.1, "dissipation": 126.4,
                     "forward_gradient_flux": 129.7}

# DRAM bytes (read + write) per launch from an ncu capture of the 201x201
# gradient workload (dram__bytes_read.sum + dram__bytes_write.sum of one
# launch of the tuned two-threads-per-point adjoint core, cold L2 between the
# profiler's passes); kernels not captured are reported as null. The capture
# and its command are summarised under profiles/.
MEASURED_TRAFFIC = {"adjoint_core": 7101696 + 0}
FORWARD_KERNELS = ["forward_gradient_flux", "forward_dissipation", "forward_divergence_rk", "forward_primitives",
                   "forward_functional"]
ADJOINT_KERNELS = ["adjoint_core", "adjoint_dissipation", "adjoint_diffusion", "adjoint_assemble_rk",
                   "adjoint_gradient_sensitivity", "adjoint_sat_vectors"]


def run_reference(args):
    """The reference arm: the CPU restatement of the reference on all host
    cores, every timed step the complete workload (960 RK4 steps forward +
    adjoint of the 201x201 monopole). The warm-up steps run a short sample of
    each CPU build (the CPU code has nothing to warm but caches and pages)
    and pick the faster build for the timed steps."""
    rank, world, _ = rank_info()
    if rank != 0:
        return
    sample = max(1, args.cpu_warmup_rk_steps)
    warm = {}
    for v in ("strict", "tuned"):
        for _ in range(max(1, args.warmup)):
            warm[v] = cpu_gradient(v, sample)["seconds"]
    variant = min(warm, key=warm.get)
    per_step, runs = [], []
    n_steps = args.rk_steps
    for _ in range(args.steps):
        r = cpu_gradient(variant, n_steps)
        runs.append(r)
        per_step.append(r["seconds"])
    sec = statistics.mean(per_step)
    pts = GRID * GRID
    value = pts * 8 * n_steps / sec / 1e6
    cores = runs[-1]["cores"]
    desc = (f"{CPU_LEGS[variant]}, OpenMP on {cores} threads of {cpu_model()}; every timed step the complete "
            f"{n_steps}-step forward + adjoint gradient; warm-up steps: {sample}-step samples of both builds "
            f"({', '.join(f'{k} {warm[k]:.2f} s' for k in warm)}), the faster build timed")
    line = {
        "impl": "reference", "metric": "FP64 Mpt-RHS/s", "value": value, "unit": "Mpt-RHS/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "ms_per_step": sec * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": WORKLOAD, "grid": "201x201", "rk4_steps": n_steps, "save_interval": SAVE_INTERVAL,
                   "sample": "the complete workload in every timed step"},
        "adjoint_gradient_s": sec, "J": runs[-1]["J"], "grad0": runs[-1]["grad0"],
        "cpu_baseline": {"value": value, "unit": "Mpt-RHS/s", "cores": cores, "kind": "port", "build": variant,
                         "cpu": cpu_model(), "sample": desc},
        "e2e": {"value": value, "unit": "Mpt-RHS/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def other_workloads(torch, steps=2, warmup=1):
    """Configs 3 and 5 beside the headline line, each as a bounded sample:
    the 256^3 Taylor-Green vortex (10 of its 2000 constant-CFL steps,
    forward + adjoint of the terminal kinetic energy) and the three-block
    curvilinear jet at half its linear size (4.9 M points, 8 of its 1000
    steps, forward + adjoint). Each reports its device-timed Mpt-RHS/s (RHS
    evaluations of the forward and adjoint passes), the strict oracle's rate
    and the GPU-vs-oracle parity of J and the adjoint state on a reduced grid
    of the same problem (the oracle on the full grids would take hours)."""
    import numpy as np
    from magudi_gb300 import capi, configs
    from magudi_gb300.solver import Solver
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import oracle_lib
    oracle_lib.set_threads(os.cpu_count())
    out = {}

    def rel(a, b):
        return float(np.linalg.norm(np.ravel(a) - np.ravel(b)) / np.linalg.norm(np.ravel(b)))

    def timed(P, n_steps, S):
        s = Solver(P)
        q0 = [b.initial_state for b in P.blocks]

        def step():
            for bi, q in enumerate(q0, start=1):
                s.set_field(bi, capi.FIELD_CONSERVED, q)
            J = s.run_forward(n_steps, S)
            G = s.run_adjoint()
            return J, G

        for _ in range(warmup):
            step()
        torch.cuda.synchronize()
        ts = []
        for _ in range(steps):
            torch.cuda.synchronize()
            t = time.perf_counter()
            J, G = step()
            torch.cuda.synchronize()
            ts.append(time.perf_counter() - t)
        pts = sum(b.n_points for b in P.blocks)
        sec = statistics.mean(ts)
        s.close()
        return {"value": pts * 8 * n_steps / sec / 1e6, "unit": "Mpt-RHS/s", "seconds_per_sample": sec,
                "grid_points": pts, "rk4_steps": n_steps, "save_interval": S, "J": J}

    def parity_and_cpu(Pg, Po, n_steps, S, adjoint_field=True):
        g, o = Solver(Pg), oracle_lib.Oracle(Po)
        Jg = g.run_forward(n_steps, S)
        t = time.perf_counter()
        Jo = o.run_forward(n_steps, S)
        o.run_adjoint()
        sec = time.perf_counter() - t
        g.run_adjoint()
        lam = rel(np.concatenate([g.get_field(b, capi.FIELD_ADJOINT).ravel() for b in range(1, len(Pg.blocks) + 1)]),
                  np.concatenate([o.get_field(b, capi.FIELD_ADJOINT).ravel() for b in range(1, len(Po.blocks) + 1)]))
        pts = sum(b.n_points for b in Po.blocks)
        g.close()
        return ({"J_rel": abs(Jg - Jo) / abs(Jo), "adjoint_state_rel": lam, "grid_points": pts, "rk4_steps": n_steps,
                 "tolerance": 1e-10},
                {"value": pts * 8 * n_steps / sec / 1e6, "unit": "Mpt-RHS/s", "cores": os.cpu_count(), "kind": "port",
                 "build": "strict", "sample": f"oracle on {pts} points, {n_steps} RK4 steps forward + adjoint "
                                              f"({sec:.1f} s)"})

    progress("config 3: Taylor-Green 256^3 sample")
    tgv = timed(configs.taylor_green_3d(n=256, n_steps=10, save_interval=5), 10, 5)
    small = configs.taylor_green_3d(n=32, n_steps=10, save_interval=5)
    par, cpu = parity_and_cpu(small, configs.taylor_green_3d(n=32, n_steps=10, save_interval=5), 10, 5)
    tgv.update({"workload": "3D Taylor-Green vortex 256^3, PLANE-periodic, Re 1600, M 0.1, constant CFL 0.5, "
                            "forward + adjoint of the terminal kinetic energy: 10 of the 2000 steps",
                "parity_reduced": par, "cpu_baseline_reduced": cpu})
    out["taylor_green_256"] = tgv
    progress("config 5: three-block jet sample")
    dims = dict(nx=192, ny_core=96, ny_side=86, nz=96)
    jet = timed(configs.jet_3block_3d(n_steps=8, save_interval=4, **dims), 8, 4)
    tiny = dict(nx=40, ny_core=25, ny_side=25, nz=25)
    par, cpu = parity_and_cpu(configs.jet_3block_3d(n_steps=4, save_interval=2, **tiny),
                              configs.jet_3block_3d(n_steps=4, save_interval=2, **tiny), 4, 2)
    jet.update({"workload": "3D three-block curvilinear jet at half the linear size of the 39.4 M-point case "
                            "(192x96x96 + 2 x 192x86x96), Mach 1.3, Re 2500, solenoidal inflow excitation, "
                            "block-interface SATs: 8 of the 1000 steps, forward + adjoint",
                "parity_reduced": par, "cpu_baseline_reduced": cpu})
    out["jet_three_block_half"] = jet
    return out


def run_ours(args):
    import numpy as np
    import torch

    rank, world, local = rank_info()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    from magudi_gb300 import capi
    from magudi_gb300.solver import Solver

    n_steps = args.rk_steps
    P = problem(n_steps)
    blk = P.blocks[0]
    pts = blk.n_points
    nU = P.n_unknowns
    s = Solver(P)
    # the workload as configured: snapshots every 10 steps, each segment's
    # forward states recomputed on the device beside the adjoint (--resident
    # times the resident trajectory instead; the other mode is measured after
    # the timed steps as a secondary figure)
    resident = bool(args.resident)
    s.set_trajectory_storage(resident)
    stream = torch.cuda.ExternalStream(s.stream_handle())
    n_entries = 4 * n_steps
    Pact = s.actuator_points()
    # device-resident initial state for the device-timed metric
    q0_dev = torch.from_numpy(np.ascontiguousarray(blk.initial_state)).cuda()
    # pinned host buffers for the end-to-end metric
    q0_host = torch.from_numpy(np.ascontiguousarray(blk.initial_state)).pin_memory()
    grad_host = torch.empty(n_entries * Pact, dtype=torch.float64).pin_memory()
    flush = torch.empty(512 * 1024 * 1024 // 8, dtype=torch.float64, device="cuda")

    def set_q(ptr):
        s._check(s.L.mgd_set_field(s.h, 1, capi.FIELD_CONSERVED, capi.C.cast(ptr, capi.C.POINTER(capi.C.c_double))))

    def gradient_step(ptr_q):
        set_q(ptr_q)
        J = s.run_forward(n_steps, SAVE_INTERVAL)
        G = s.run_adjoint()
        return J, G

    def timed_gradients(k):
        times, J, G = [], None, None
        for _ in range(k):
            flush.zero_()
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            if world > 1:
                torch.distributed.barrier()
            e0.record(stream)
            J, G = gradient_step(q0_dev.data_ptr())
            e1.record(stream)
            torch.cuda.synchronize()
            times.append(e0.elapsed_time(e1))
        return times, J, G

    # run-level tile tuning on short gradient runs (setup, outside the timed region)
    progress("tile tuning")
    set_q(q0_dev.data_ptr())
    t_tune = time.perf_counter()
    if args.tiles:
        for k, t in enumerate(args.tiles.split(",")):
            s.stage_tile(k, tuple(int(x) for x in t.split("x")))
        if args.grad_lanes:
            s.gradient_lanes(args.grad_lanes)
        if args.core_lanes:
            s.adjoint_core_lanes(args.core_lanes)
        tuned_ms = None
    else:
        tuned_ms = s.tune_run(4 * SAVE_INTERVAL, SAVE_INTERVAL)
    tuning = {"seconds": time.perf_counter() - t_tune, "run_steps": 4 * SAVE_INTERVAL, "tuned_run_ms": tuned_ms,
              "tiles": [list(s.stage_tile(k)) for k in range(6)], "gradient_flux_threads_per_point": s.gradient_lanes(),
              "adjoint_core_threads_per_point": s.adjoint_core_lanes(),
              "source": "--tiles" if args.tiles else "mgd_tune_run"}
    for _ in range(args.warmup):
        gradient_step(q0_dev.data_ptr())
    torch.cuda.synchronize()
    if args.profile_only:
        # the timed-equivalent evaluations in an NVTX range (ncu --nvtx --nvtx-include "gradient/")
        torch.cuda.nvtx.range_push("gradient")
        for _ in range(args.steps):
            J, G = gradient_step(q0_dev.data_ptr())
        torch.cuda.synchronize()
        torch.cuda.nvtx.range_pop()
        # one forward and one adjoint RHS of the final state through the
        # per-call entry points, in an NVTX range for filtered ncu captures
        # (ncu --nvtx --nvtx-include "stage_rhs/")
        s.compute_rhs(capi.FORWARD, 0.0)
        s.compute_rhs(capi.ADJOINT, 0.0, 1.0)
        torch.cuda.synchronize()
        torch.cuda.nvtx.range_push("stage_rhs")
        s.compute_rhs(capi.FORWARD, 0.0)
        s.compute_rhs(capi.ADJOINT, 0.0, 1.0)
        torch.cuda.nvtx.range_pop()
        torch.cuda.synchronize()
        print(json.dumps({"profile_only": True, "rk_steps": n_steps, "J": J, "grad0": G}), flush=True)
        return
    s.kernel_launches(reset=True)
    progress("timed gradients")
    clocks = ClockSampler()
    clocks.start()
    times, J, G = timed_gradients(args.steps)
    launches = s.kernel_launches(reset=True) // args.steps
    grad_vec = s.gradient(n_entries)
    # end to end through the C ABI with host buffers
    e2e_times = []
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        t = time.perf_counter()
        gradient_step(q0_host.data_ptr())
        s._check(s.L.mgd_get_gradient(s.h, capi.C.cast(grad_host.data_ptr(), capi.C.POINTER(capi.C.c_double)), n_entries))
        torch.cuda.synchronize()
        e2e_times.append((time.perf_counter() - t) * 1e3)
    clk = clocks.stop()
    # secondary figure: the same gradient in the other storage mode (same tiles)
    progress("secondary storage mode")
    s.set_trajectory_storage(not resident)
    gradient_step(q0_dev.data_ptr())
    torch.cuda.synchronize()
    alt_times, J_alt, G_alt = timed_gradients(args.steps)
    alt_ms = statistics.mean(alt_times)
    s.set_trajectory_storage(resident)
    ms = statistics.mean(times)
    if world > 1:
        t = torch.tensor([ms], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms = float(t.item())
    rhs_evals = 8 * n_steps
    value = world * pts * rhs_evals / (ms / 1e3) / 1e6
    e2e_ms = statistics.mean(e2e_times)
    e2e = world * pts * rhs_evals / (e2e_ms / 1e3) / 1e6
    # per-kernel timing for the roofline (separate short loops on the same stream)
    progress("per-kernel timing and FP64 peak")
    fwd = s.profile_stage_kernels(capi.FORWARD, 30)
    adj = s.profile_stage_kernels(capi.ADJOINT, 30)
    kern = dict(zip(FORWARD_KERNELS, fwd))
    kern.update(zip(ADJOINT_KERNELS, adj))
    # launches per gradient evaluation: forward stage kernels run in the forward
    # pass (and again in the checkpoint recomputation unless the trajectory is
    # resident), the functional only in the forward pass, adjoint kernels once
    per_grad = {k: (4 if resident else 8) * n_steps for k in FORWARD_KERNELS}
    per_grad["forward_functional"] = 4 * n_steps
    per_grad.update({k: 4 * n_steps for k in ADJOINT_KERNELS})
    share = {k: kern[k] * per_grad[k] for k in kern}
    dominant = max((k for k in share if k in KERNEL_UNITS), key=share.get)
    peaks, peak_kind = measured_peaks()
    units = KERNEL_UNITS[dominant]
    t_launch = kern[dominant] / 1e3
    achieved_gbs = units["bytes"] * pts / t_launch / 1e9
    alg_flops = ALGORITHMIC_FLOPS.get(dominant, units["flops"])
    achieved_tf = alg_flops * pts / t_launch / 1e12
    executed_tf = units["flops"] * pts / t_launch / 1e12
    fp64 = fp64_peak(torch, clk)
    # whole RHS: the reference's operation count over the stage kernels' time
    t_fwd = sum(kern[k] for k in FORWARD_KERNELS if k != "forward_functional") / 1e3
    t_adj = sum(kern[k] for k in ADJOINT_KERNELS if k != "adjoint_gradient_sensitivity") / 1e3
    mode_text = {False: "checkpoints every %d steps, each segment's forward states recomputed on the device beside "
                        "the adjoint (UniformCheckpointer)" % SAVE_INTERVAL,
                 True: "resident trajectory: every stage's state, primitives, stress and heat flux kept on the device "
                       "by the forward run, no recomputation"}
    line = {
        "metric": "FP64 Mpt-RHS/s", "value": value, "unit": "Mpt-RHS/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (quiescent monopole initial state generated in-process)",
        "config": {"workload": WORKLOAD, "grid": "201x201", "rk4_steps": N_STEPS, "save_interval": SAVE_INTERVAL,
                   "l2": "512 MB buffer written between timed steps (working set fits in L2)",
                   "parallelism": "replicas" if world > 1 else "single GPU",
                   "tile_tuning": tuning,
                   "adjoint_forward_states": mode_text[resident]},
        "adjoint_gradient_s": ms / 1e3,
        "J": J, "grad0": G,
        "e2e": {"value": e2e, "unit": "Mpt-RHS/s", "ms_per_step": e2e_ms,
                "h2d_bytes_per_step": pts * nU * 8, "d2h_bytes_per_step": n_entries * Pact * 8 + 16},
        "gpu_launches": launches,
        "clocks": clk,
        ("checkpoint_recompute" if resident else "resident_trajectory"): {
            "value": world * pts * rhs_evals / (alt_ms / 1e3) / 1e6, "unit": "Mpt-RHS/s", "ms_per_step": alt_ms,
            "steps": args.steps, "adjoint_forward_states": mode_text[not resident],
            "J_rel_diff": abs(J_alt - J) / abs(J), "grad0_rel_diff": abs(G_alt - G) / abs(G)},
        "kernels_ms_per_launch": kern,
        "kernel_time_share": {k: share[k] / sum(share.values()) for k in share},
        "roofline": {"bound": "fp64", "kernel": dominant, "achieved": achieved_tf, "peak": fp64["peak_tflops"],
                     "unit": "TFLOP/s", "frac": achieved_tf / fp64["peak_tflops"],
                     "traffic": MEASURED_TRAFFIC.get(dominant), "peak_source": fp64["source"],
                     "peak_nominal_tflops": fp64["nominal_tflops"], "fp64_pipe_probe": fp64["pipe_probe"],
                     "flops_per_point": alg_flops,
                     "flops_source": ("reference operation list, counted by the operation-counting oracle build"
                                      if dominant in ALGORITHMIC_FLOPS else
                                      "FP64 operations the kernel executes: the operation list has no separate count "
                                      "for this kernel's share of the RHS"),
                     "executed": {"flops_per_point": units["flops"], "achieved_tflops": executed_tf,
                                  "frac": executed_tf / fp64["peak_tflops"],
                                  "source": "FP64 instructions the kernel executes (ncu, 2 x DFMA + DADD + DMUL), "
                                            "counted for the one-thread-per-point form of the 2D kernels"},
                     "rhs": {"forward": {"flops_per_point": ALGORITHMIC_FLOPS["forward_rhs"],
                                         "achieved_tflops": ALGORITHMIC_FLOPS["forward_rhs"] * pts / t_fwd / 1e12,
                                         "stage_kernels_ms": t_fwd * 1e3},
                             "adjoint": {"flops_per_point": ALGORITHMIC_FLOPS["adjoint_rhs"],
                                         "achieved_tflops": ALGORITHMIC_FLOPS["adjoint_rhs"] * pts / t_adj / 1e12,
                                         "stage_kernels_ms": t_adj * 1e3}},
                     "hbm": {"achieved_gbs": achieved_gbs, "peak_gbs": peaks["hbm_gbs"],
                             "frac": achieved_gbs / peaks["hbm_gbs"], "bytes_per_point": units["bytes"],
                             "peak_source": peak_kind},
                     "note": "FP64 path with no tensor-core work: the binding roof is the FP64 pipe; the 201x201 "
                             "working set stays in L2, so the HBM fraction is not the bound"},
    }
    if rank == 0 and world == 1:
        # the same gradient through the per-call entry points (the reference's own
        # control flow over the computeRhs seam), timed once beside the graph path
        from magudi_gb300.drivers import per_call_gradient
        progress("per-call gradient")
        t_start = time.perf_counter()
        Jp, Gp = per_call_gradient(s, P, n_steps, SAVE_INTERVAL)
        tp = time.perf_counter() - t_start
        line["plain_per_call"] = {
            "value": pts * 8 * n_steps / tp / 1e6, "unit": "Mpt-RHS/s", "seconds": tp,
            "speedup_of_graph_path": tp / (ms / 1e3),
            "J_rel_diff": abs(Jp - J) / abs(J), "grad0_rel_diff": abs(Gp - G) / abs(G),
            "path": "mgd_rk4_substep + functional/sensitivity calls per stage, checkpoints and segment "
                    "stage states in host memory (Solver%runForward / runAdjoint with UniformCheckpointer)"}
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        # the complete workload on the host cores: the strict build is the
        # parity reference of this run, the faster build the CPU baseline
        progress("CPU oracle, strict build")
        legs = {"strict": cpu_gradient("strict", n_steps, want_vector=True)}
        progress("CPU oracle, tuned build")
        legs["tuned"] = cpu_gradient("tuned", n_steps)
        line["parity"] = parity_of(J, G, grad_vec, legs["strict"])
        fast = min(legs, key=lambda k: legs[k]["seconds"])
        line["cpu_baseline"] = {
            "value": legs[fast]["value"], "unit": "Mpt-RHS/s", "cores": legs[fast]["cores"], "kind": "port",
            "build": fast, "cpu": cpu_model(),
            "sample": f"the complete workload ({n_steps} RK4 steps forward + adjoint, 201x201) on the host cores "
                      f"with {CPU_LEGS[fast]}: {legs[fast]['seconds']:.1f} s",
            "legs": {k: {"value": v["value"], "seconds": v["seconds"], "flags": CPU_LEGS[k],
                         "J_rel_vs_strict": abs(v["J"] - legs["strict"]["J"]) / abs(legs["strict"]["J"])}
                     for k, v in legs.items()}}
    if rank == 0 and world == 1 and not args.no_other_workloads:
        # release the 201x201 context (its trajectory holds about 22 GB) first
        s.close()
        del s
        torch.cuda.empty_cache()
        line["other_workloads"] = other_workloads(torch)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def run_sweep(args):
    """Batched gradient-check sweep: every instance runs the monopole forward
    with control forcing amplitude x (adjoint gradient of its grid size) and
    reports its J. One step = the whole sweep through mgd_batch_run_forward;
    the plain single-solve path (mgd_run_forward per instance) is timed once
    beside it on the same instances."""
    import numpy as np
    import torch
    from magudi_gb300 import capi, configs, sweep
    from magudi_gb300.solver import Batch, Solver

    rank, world, local = rank_info()
    if world > 1:
        torch.distributed.init_process_group("nccl")
    torch.cuda.set_device(local)
    n_steps = args.rk_steps
    cases = sweep.cases(args.sweep_instances)
    # instances split over ranks by grid points (independent solves, no collective)
    mine_idx = sweep.shard(cases, rank, world)
    mine = [cases[i] for i in mine_idx]
    grads = {}
    for n in sorted({n for n, _ in mine}):
        s = Solver(configs.monopole_2d(n=n, n_steps=n_steps, save_interval=SAVE_INTERVAL))
        s.run_forward(n_steps, SAVE_INTERVAL)
        s.run_adjoint()
        grads[n] = s.gradient(4 * n_steps)
        s.close()
    solvers, q0, forcings = [], [], []
    for n, a in mine:
        P = configs.monopole_2d(n=n, n_steps=n_steps, save_interval=SAVE_INTERVAL, controller_switch=True)
        s = Solver(P)
        forcings.append(a * grads[n])
        s.set_control_forcing(forcings[-1])
        solvers.append(s)
        q0.append(np.ascontiguousarray(P.blocks[0].initial_state))
    batch = Batch(solvers)

    def reset():
        for s, q in zip(solvers, q0):
            s.set_field(1, capi.FIELD_CONSERVED, q)

    # the per-step graph path of the same batch, timed once beside the
    # persistent single launch (the default)
    batch.persistent(0)
    reset()
    batch.run_forward(n_steps)
    reset()
    torch.cuda.synchronize()
    t = time.perf_counter()
    graph_costs = batch.run_forward(n_steps)
    torch.cuda.synchronize()
    t_graph = time.perf_counter() - t
    batch.persistent(1)
    for _ in range(args.warmup):
        reset()
        batch.run_forward(n_steps)
    batch.kernel_launches(reset=True)
    clocks = ClockSampler()
    clocks.start()
    times = []
    costs = None
    for _ in range(args.steps):
        reset()
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
        t = time.perf_counter()
        costs = batch.run_forward(n_steps)
        torch.cuda.synchronize()
        times.append(time.perf_counter() - t)
    clk = clocks.stop()
    launches = batch.kernel_launches(reset=True) // args.steps
    # plain single-solve path on the same instances, once
    reset()
    torch.cuda.synchronize()
    t = time.perf_counter()
    plain_costs = [s.run_forward(n_steps, SAVE_INTERVAL) for s in solvers]
    torch.cuda.synchronize()
    t_plain = time.perf_counter() - t
    # the reference's control flow over the per-call entry points (one
    # mgd_rk4_substep per stage, the stage's forcing handed to the actuators),
    # timed on a sample of the instances
    from magudi_gb300.drivers import per_call_forward
    K = min(len(solvers), args.sweep_per_call_sample)
    t = time.perf_counter()
    pc_costs = [per_call_forward(solvers[i], solvers[i].problem, n_steps, forcings[i]) for i in range(K)]
    t_pc = time.perf_counter() - t
    pc_rel = max(abs(a - b) / abs(b) for a, b in zip(pc_costs, costs[:K])) if K else 0.0
    sec = statistics.mean(times)
    if world > 1:
        tt = torch.tensor([sec, t_plain], device="cuda")
        torch.distributed.all_reduce(tt, op=torch.distributed.ReduceOp.MAX)
        sec, t_plain = float(tt[0]), float(tt[1])
    pts = sum(n * n for n, _ in cases)
    max_rel = max(abs(a - b) / abs(b) for a, b in zip(costs, plain_costs))
    all_costs = sweep.gather_costs(mine_idx, costs, len(cases))
    line = {
        "metric": "batched FD-sweep solves/s", "value": len(cases) / sec, "unit": "solves/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": sec * 1e3, "higher_is_better": True,
        "scaling": "strong", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (quiescent monopole states, gradient-direction control forcing computed in-process)",
        "config": {"workload": f"{len(cases)} 2D monopole instances, sizes drawn with seed 0 from "
                               f"{list(sweep.SIZES)} (squared), control amplitude 10^(-2-0.25k), k = i mod 20, "
                               f"{n_steps} RK4 steps forward each, all steps of all instances in one persistent "
                               f"launch",
                   "instances": len(cases), "rk4_steps": n_steps, "total_points": pts,
                   "l2": "working set (all instances) larger than L2",
                   "parallelism": f"instances sharded round-robin over {world} GPU(s)" if world > 1 else "single GPU"},
        "mpt_rhs_per_s": pts * 4 * n_steps / sec / 1e6,
        "launch": {"mode": "one persistent cooperative launch for all steps, captured in a CUDA graph",
                   "ctas": batch.persistent_grid()},
        "per_step_graphs": {"value": len(cases) / t_graph, "unit": "solves/s", "seconds": t_graph,
                            "max_rel_diff_J": max(abs(a - b) / abs(b) for a, b in zip(graph_costs, costs)),
                            "path": "one CUDA graph of batched stage kernels per RK4 step"},
        "plain_single_solve": {"value": len(cases) / t_plain, "unit": "solves/s", "seconds": t_plain,
                               "path": "mgd_run_forward per instance, one after another"},
        "speedup_vs_plain": t_plain / sec,
        "max_rel_diff_vs_plain_J": max_rel,
        "per_call_sample": {"instances": K, "seconds": t_pc, "value": K / t_pc if K else None, "unit": "solves/s",
                            "batch_speedup": (len(cases) / sec) / (K / t_pc) if K else None,
                            "max_rel_diff_vs_batch_J": pc_rel,
                            "path": "mgd_rk4_substep + functional per stage with the stage's forcing handed to the "
                                    "actuators (Solver%runForward over the computeRhs seam), the first instances"},
        "J_first": float(all_costs[0]), "J_last": float(all_costs[-1]),
        "gpu_launches": launches,
        "clocks": clk,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def run_fdcheck(args):
    """The reference's gradient-accuracy procedure (README.md:118-165) at the
    headline configuration: the 201x201 monopole, 960 RK4 steps, checkpoints
    every 10 steps. One forward + adjoint run gives J0, Grad0 and the control
    gradient g; then one batch runs the forward with the control forcing
    A_k g for A_k = 10^(-2-0.25k), k = 0..19 (bin/ZAXPY.f90 on the device),
    plus A = 0, and the line reports the reference's table: A_k, J_k,
    (J_k - J0)/A_k and its relative error against Grad0."""
    import torch
    from magudi_gb300 import configs, sweep
    from magudi_gb300.solver import Batch, Solver

    rank, world, local = rank_info()
    torch.cuda.set_device(local)
    n_steps = args.rk_steps
    P = configs.monopole_2d(n=GRID, n_steps=n_steps, save_interval=SAVE_INTERVAL)
    base = Solver(P)
    t = time.perf_counter()
    J0 = base.run_forward(n_steps, SAVE_INTERVAL)
    G0 = base.run_adjoint()
    g = base.gradient(4 * n_steps)
    t_grad = time.perf_counter() - t
    amps = [0.0] + [10.0 ** (-2.0 - 0.25 * k) for k in range(20)]
    solvers = []
    for a in amps:
        Pc = configs.monopole_2d(n=GRID, n_steps=n_steps, save_interval=SAVE_INTERVAL, controller_switch=True)
        s = Solver(Pc)
        s.set_control_forcing(a * g)
        solvers.append(s)
    batch = Batch(solvers)
    torch.cuda.synchronize()
    t = time.perf_counter()
    costs = batch.run_forward(n_steps)
    torch.cuda.synchronize()
    t_batch = time.perf_counter() - t
    J0b = costs[0]
    rows = sweep.fd_errors(J0b, G0, amps[1:], costs[1:])
    best = min(r[3] for r in rows)
    line = {
        "metric": "gradient accuracy (FD sweep)", "value": best, "unit": "min relative error",
        "n_gpus": 1, "steps": 1, "warmup": 0, "ms_per_step": (t_grad + t_batch) * 1e3, "higher_is_better": False,
        "dtype": "f64", "data": "synthetic (quiescent monopole)",
        "config": {"workload": f"2D acoustic monopole {GRID}x{GRID}, {n_steps} RK4 steps, checkpoints every "
                               f"{SAVE_INTERVAL}: adjoint gradient, then the forward with control forcing A_k g, "
                               f"A_k = 10^(-2-0.25k), k = 0..19, as one batch of {len(amps)} instances"},
        "J0": J0, "J0_batch": J0b, "grad0": G0, "gradient_seconds": t_grad, "batch_seconds": t_batch,
        "table": [{"A": a, "J": J, "fd_gradient": fdg, "rel_error": e} for a, J, fdg, e in rows],
    }
    if rank == 0:
        print(json.dumps(line), flush=True)


def run_tgv(args):
    """3D Taylor-Green vortex on n^3 points, PLANE-periodic, Re 1600, Mach 0.1,
    constant CFL 0.5: forward run plus the discrete adjoint of the terminal
    kinetic energy, with checkpoints held on the device. The configured run
    has 2000 steps; one bench step is a bounded sample of --tgv-steps steps
    (forward + adjoint) of it, and the metric counts grid points x RHS
    evaluations per second like the default workload."""
    import torch
    from magudi_gb300 import configs
    from magudi_gb300.solver import Solver

    rank, world, local = rank_info()
    torch.cuda.set_device(local)
    n_steps = args.tgv_steps
    P = configs.taylor_green_3d(n=args.tgv_n, n_steps=n_steps)
    S = P.save_interval
    s = Solver(P)
    if args.dissipation_tma >= 0:
        s.dissipation_tma(args.dissipation_tma)
    q0 = P.blocks[0].initial_state
    from magudi_gb300 import capi

    def step():
        s.set_field(1, capi.FIELD_CONSERVED, q0)
        J = s.run_forward(n_steps, S)
        s.run_adjoint()
        return J

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    s.kernel_launches(reset=True)
    clocks = ClockSampler()
    clocks.start()
    times = []
    J = None
    # the timed steps in an NVTX range (ncu --nvtx --nvtx-include "gradient/")
    torch.cuda.nvtx.range_push("gradient")
    for _ in range(args.steps):
        torch.cuda.synchronize()
        t = time.perf_counter()
        J = step()
        torch.cuda.synchronize()
        times.append(time.perf_counter() - t)
    torch.cuda.nvtx.range_pop()
    clk = clocks.stop()
    sec = statistics.mean(times)
    pts = args.tgv_n ** 3
    dts = s.step_sizes(n_steps)
    line = {
        "metric": "FP64 Mpt-RHS/s", "value": pts * 8 * n_steps / sec / 1e6, "unit": "Mpt-RHS/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": sec * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (Taylor-Green initial field)",
        "config": {"workload": f"3D Taylor-Green vortex {args.tgv_n}^3 PLANE-periodic, Re 1600, M 0.1, SBP 4-8 + "
                               f"dissipation, constant CFL 0.5, forward + discrete adjoint of the terminal "
                               f"kinetic energy; sample of {n_steps} of the 2000 steps, checkpoint every {S}",
                   "grid": f"{args.tgv_n}^3", "rk4_steps": n_steps, "save_interval": S,
                   "dissipation_form": "tensor-memory-accelerator staging" if s.dissipation_tma() else "L1",
                   "l2": "working set larger than L2", "parallelism": "single GPU"},
        "J": J, "dt_first": float(dts[0]), "dt_last": float(dts[-1]),
        "projected_2000_step_gradient_s": sec / n_steps * 2000,
        "gpu_launches": s.kernel_launches(reset=True) // max(1, args.steps), "clocks": clk,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)


def run_jet(args):
    """Three-block curvilinear 3D jet (core 384 x 192 x 192 and two 384 x 171 x
    192 shear-layer blocks, 39.4 M points), Mach 1.3, Re 2500, solenoidal inflow
    excitation, block-interface SATs on the device: forward run plus the
    discrete adjoint of the squared-pressure functional with checkpoints held
    on the device. The configured run has 1000 steps; one bench step is a
    bounded sample of --jet-steps steps (forward + adjoint). The metric counts
    grid points x RHS evaluations per second like the default workload."""
    import torch
    from magudi_gb300 import capi, configs
    from magudi_gb300.solver import Solver

    rank, world, local = rank_info()
    torch.cuda.set_device(local)
    n_steps, S = args.jet_steps, args.jet_save_interval
    f = args.jet_scale
    dims = dict(nx=max(28, int(round(384 * f))), ny_core=max(25, int(round(192 * f))),
                ny_side=max(25, int(round(171 * f))), nz=max(25, int(round(192 * f))))
    P = configs.jet_3block_3d(n_steps=n_steps, save_interval=S, **dims)
    free0, total = torch.cuda.mem_get_info()
    s = Solver(P)
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    pts = sum(b.n_points for b in P.blocks)

    def step():
        for bi, b in enumerate(P.blocks, start=1):
            s.set_field(bi, capi.FIELD_CONSERVED, b.initial_state)
        J = s.run_forward(n_steps, S)
        G = s.run_adjoint()
        return J, G

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    free2, _ = torch.cuda.mem_get_info()
    s.kernel_launches(reset=True)
    clocks = ClockSampler()
    clocks.start()
    times = []
    J = G = None
    for _ in range(args.steps):
        torch.cuda.synchronize()
        t = time.perf_counter()
        J, G = step()
        torch.cuda.synchronize()
        times.append(time.perf_counter() - t)
    clk = clocks.stop()
    sec = statistics.mean(times)
    # device memory of the full 1000-step run with checkpoints every S1 steps
    # (q snapshots every S1 steps + 4 S1 stage slots of q, the choice that
    # minimises T / S1 + 4 S1): the setup's resident arrays plus those states
    T, S1 = 1000, 16
    state = 5 * 8 * pts
    # (plus the per-stage gradient entries of the actuator points)
    full_run = (free0 - free1) + (T // S1 + 2 + 4 * S1) * state + 4 * T * 8 * s.actuator_points()
    line = {
        "metric": "FP64 Mpt-RHS/s", "value": pts * 8 * n_steps / sec / 1e6, "unit": "Mpt-RHS/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": sec * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (jet initial field)",
        "config": {"workload": f"3D three-block curvilinear jet, {pts / 1e6:.1f} M points "
                               f"({'+'.join('x'.join(str(v) for v in b.grid_size) for b in P.blocks)}), "
                               f"Mach 1.3, Re 2500, SBP 4-8 + dissipation, block-interface SATs, 8-mode "
                               f"solenoidal excitation, forward + discrete adjoint of the squared pressure on a "
                               f"cylindrical target; sample of {n_steps} of the 1000 steps, checkpoint every {S}",
                   "grid_points": pts, "rk4_steps": n_steps, "save_interval": S, "dt": P.options.time_step_size,
                   "l2": "working set larger than L2", "parallelism": "single GPU, all blocks on the device"},
        "J": J, "gradient_norm_sq": G,
        "projected_1000_step_gradient_s": sec / n_steps * T,
        "device_memory_gb": {"setup": (free0 - free1) / 1e9, "sample_run": (free0 - free2) / 1e9,
                             "projected_1000_step_run_q_slots_every_16": full_run / 1e9,
                             "device_total": total / 1e9},
        "gpu_launches": s.kernel_launches(reset=True) // max(1, args.steps), "clocks": clk,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)


def run_msgrad(args):
    """Multi-segment gradient of the 2D monopole (201^2, 960 steps): the steps
    split into --ms-segments segments whose initial conditions lie on the
    trajectory of one run (bin/msforward.f90 + bin/msadjoint.f90, quadratic
    penalty). The segments' forward and adjoint runs go concurrently, one host
    thread and one context per segment. Timed beside the single-run gradient
    of the same 960 steps. The metric counts forward and adjoint RHS
    evaluations per second like the default workload."""
    import torch
    from magudi_gb300 import capi, configs
    from magudi_gb300.multisegment import MultiSegment
    from magudi_gb300.solver import Solver

    rank, world, local = rank_info()
    torch.cuda.set_device(local)
    K = args.ms_segments
    T = args.rk_steps
    nts = T // K
    T = nts * K
    Pseg = configs.monopole_2d(n=GRID, n_steps=nts, save_interval=SAVE_INTERVAL)
    Pfull = configs.monopole_2d(n=GRID, n_steps=T, save_interval=SAVE_INTERVAL)
    single = Solver(Pfull)
    resident = not args.checkpoint_only
    q0 = Pfull.blocks[0].initial_state
    ics = [None]
    for k in range(1, K):
        single.set_field(1, capi.FIELD_CONSERVED, q0)
        single.run_forward(k * nts, SAVE_INTERVAL)
        ics.append([single.get_field(1, capi.FIELD_CONSERVED)])
    # both the segments and the single run keep their trajectories on the device
    single.set_trajectory_storage(resident)
    single.set_field(1, capi.FIELD_CONSERVED, q0)
    single.tune_run(4 * SAVE_INTERVAL, SAVE_INTERVAL)
    ms = MultiSegment(Pseg, K, nts, penalty_weight=1.0, save_interval=SAVE_INTERVAL, store_trajectory=resident)

    def ms_step():
        r = ms.forward(ics)
        a = ms.adjoint()
        return r.J, a.total

    def single_step():
        single.set_field(1, capi.FIELD_CONSERVED, q0)
        J = single.run_forward(T, SAVE_INTERVAL)
        return J, single.run_adjoint()

    for _ in range(args.warmup):
        ms_step()
        single_step()
    torch.cuda.synchronize()
    clocks = ClockSampler()
    clocks.start()
    t_ms, t_single = [], []
    for _ in range(args.steps):
        torch.cuda.synchronize()
        t = time.perf_counter()
        J, G = ms_step()
        torch.cuda.synchronize()
        t_ms.append(time.perf_counter() - t)
        t = time.perf_counter()
        J1, G1 = single_step()
        torch.cuda.synchronize()
        t_single.append(time.perf_counter() - t)
    clk = clocks.stop()
    sec, sec1 = statistics.mean(t_ms), statistics.mean(t_single)
    pts = GRID * GRID
    line = {
        "metric": "FP64 Mpt-RHS/s", "value": pts * 8 * T / sec / 1e6, "unit": "Mpt-RHS/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": sec * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (monopole)",
        "config": {"workload": f"2D acoustic monopole {GRID}x{GRID}, {T} RK4 steps as {K} time segments of {nts} "
                               f"(initial conditions on the trajectory, quadratic matching penalty), forward + "
                               f"discrete adjoint of every segment, segments concurrent; checkpoint every "
                               f"{SAVE_INTERVAL} steps",
                   "trajectory": "recomputed from checkpoints" if args.checkpoint_only else
                                 "resident in every segment's context and in the single run",
                   "segments": K, "segment_steps": nts, "l2": "working set fits in L2 (no flush)",
                   "parallelism": "single GPU, one context and host thread per segment"},
        "J": J, "gradient_inner_product": G,
        "single_run": {"value": pts * 8 * T / sec1 / 1e6, "unit": "Mpt-RHS/s", "seconds": sec1, "J": J1,
                       "gradient_norm_sq": G1},
        "speedup_vs_single_run": sec1 / sec,
        "clocks": clk,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)


def run_tangent(args):
    """Tangent (linearized) run of the 2D monopole (201^2, 960 steps):
    Solver%runLinearized along the forward trajectory, kept on the device by
    the forward run (with --checkpoint-only: checkpoints every 10 steps, each
    segment's stage states recomputed before its linearized steps). One bench
    step is the forward run plus the tangent run; the metric counts forward
    and linearized RHS evaluations per second, and the tangent run alone is
    reported beside it."""
    import numpy as np
    import torch
    from magudi_gb300 import capi
    from magudi_gb300.solver import Solver

    rank, world, local = rank_info()
    torch.cuda.set_device(local)
    T = args.rk_steps
    P = problem(T)
    s = Solver(P)
    # the forward run keeps every stage on the device; the tangent run reads it
    s.set_trajectory_storage(not args.checkpoint_only)
    q0 = P.blocks[0].initial_state
    rng = np.random.default_rng(0)
    dq0 = 1e-3 * rng.standard_normal(q0.shape) * np.abs(q0).mean(axis=1, keepdims=True)
    s.set_field(1, capi.FIELD_CONSERVED, q0)
    s.tune_run(4 * SAVE_INTERVAL, SAVE_INTERVAL)

    def step():
        # each library call returns after its work completed on the device
        s.set_field(1, capi.FIELD_CONSERVED, q0)
        t0 = time.perf_counter()
        s.run_forward(T, SAVE_INTERVAL)
        t1 = time.perf_counter()
        s.set_field(1, capi.FIELD_ADJOINT, dq0)
        s.run_linearized()
        t2 = time.perf_counter()
        return t2 - t0, t2 - t1

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    s.kernel_launches(reset=True)
    clocks = ClockSampler()
    clocks.start()
    times, tan = [], []
    for _ in range(args.steps):
        a, b = step()
        times.append(a)
        tan.append(b)
    clk = clocks.stop()
    sec = statistics.mean(times)
    sec_tan = statistics.mean(tan)
    pts = GRID * GRID
    dT = s.get_field(1, capi.FIELD_ADJOINT)
    line = {
        "metric": "FP64 Mpt-RHS/s", "value": pts * 8 * T / sec / 1e6, "unit": "Mpt-RHS/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": sec * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (monopole)",
        "config": {"workload": f"2D acoustic monopole {GRID}x{GRID}, {T} RK4 steps forward, then the linearized "
                               f"(tangent) run along the forward trajectory (checkpoint every {SAVE_INTERVAL})",
                   "trajectory": "recomputed from checkpoints" if args.checkpoint_only else
                                 "resident: every stage's state, primitives, stress and heat flux kept on the device",
                   "l2": "working set fits in L2 (no flush)", "parallelism": "single GPU"},
        "tangent_run": {"value": pts * 4 * T / sec_tan / 1e6, "unit": "Mpt-RHS/s (linearized RHS)",
                        "seconds": sec_tan},
        "final_perturbation_norm": float(np.linalg.norm(dT)),
        "gpu_launches": s.kernel_launches(reset=True) // max(1, args.steps), "clocks": clk,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "sweep":
        run_sweep(args)
    elif args.workload == "tgv":
        run_tgv(args)
    elif args.workload == "jet":
        run_jet(args)
    elif args.workload == "msgrad":
        run_msgrad(args)
    elif args.workload == "tangent":
        run_tangent(args)
    elif args.workload == "fdcheck":
        run_fdcheck(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
