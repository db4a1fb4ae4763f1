"""The bench line contract on the CPU (no GPU): the reference arm (the oracle
timed on the host cores) prints one JSON line with the keys the bench contract
names, on a 2-step sample of the 201x201 workload, and the command line takes
the contract's options."""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _run(*args, timeout=300):
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), *args], cwd=ROOT, capture_output=True,
                       text=True, timeout=timeout)
    assert r.returncode == 0, r.stderr[-2000:]
    return r.stdout


def test_command_line_takes_the_contract_options():
    out = _run("--help", timeout=120)
    for opt in ("--gpus", "--steps", "--warmup", "--impl", "--workload", "--resident", "--tiles"):
        assert opt in out


def test_reference_arm_prints_one_contract_line():
    # a 4-step gradient instead of the 960-step one keeps the CPU suite short
    out = _run("--impl", "reference", "--steps", "1", "--warmup", "1", "--rk-steps", "4", "--cpu-warmup-rk-steps", "2")
    lines = [l for l in out.splitlines() if l.strip().startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for key in ("impl", "metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "scaling", "vs_baseline", "dtype", "config", "cpu_baseline", "e2e"):
        assert key in d, key
    assert d["impl"] == "reference" and d["metric"] == "FP64 Mpt-RHS/s" and d["value"] > 0.0
    assert d["e2e"]["value"] == d["value"] and d["e2e"]["h2d_bytes_per_step"] == 0
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["cores"] >= 1
    assert d["cpu_baseline"]["build"] in ("strict", "tuned")
    assert d["config"]["rk4_steps"] == 4 and abs(d["ms_per_step"] / 1e3 - d["adjoint_gradient_s"]) < 1e-9
    assert "workload" in d["config"]
