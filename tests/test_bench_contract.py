"""bench.py's JSON line.  The reference arm on the host cores (no GPU): the bench contract
(keys, impl, e2e equal to the line's value with no host copies, cpu_baseline describing
the run), and under a two-rank launch rank 0 alone prints it.  The main arm (GPU) on a
small case: the contract keys plus roofline, e2e with host copies, launches and clocks."""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
KEYS = {"impl", "metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
        "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"}
ARGS = ["bench.py", "--impl", "reference", "--side", "400", "--tracks", "2000", "--steps", "3", "--warmup", "3"]


def _lines(stdout):
    return [json.loads(l) for l in stdout.splitlines() if l.startswith("{")]


def _check(d, n_gpus):
    assert KEYS <= set(d), KEYS - set(d)
    assert d["impl"] == "reference" and d["n_gpus"] == n_gpus
    assert d["steps"] == 3 and d["warmup"] == 3 and d["value"] > 0 and d["higher_is_better"] is True
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    cb = d["cpu_baseline"]
    assert cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["value"] == d["value"] and cb["sample"]
    assert d["config"]["workload"] and d["config"]["n"] == 400
    assert len(d["step_ms"]) == 3 and abs(sum(d["step_ms"]) / 3 - d["ms_per_step"]) < 1e-6 * d["ms_per_step"]


def test_reference_arm_prints_one_contract_line():
    r = subprocess.run([sys.executable, *ARGS], cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = _lines(r.stdout)
    assert len(lines) == 1
    _check(lines[0], 1)


def test_reference_arm_two_ranks_rank0_alone_prints():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), *ARGS, "--gpus", "2"]
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = _lines(r.stdout)
    assert len(lines) == 1
    _check(lines[0], 2)


@pytest.mark.gpu
def test_gpu_arm_prints_one_contract_line():
    """The main arm on a small case: the contract keys, the roofline object of the dominant
    kernel, an e2e number with host copies, a positive launch count and the clock record."""
    cmd = [sys.executable, "bench.py", "--small", "--steps", "3", "--warmup", "3", "--no-cpu", "--no-plain",
           "--no-pair", "--no-c5"]
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = _lines(r.stdout)
    assert len(lines) == 1
    d = lines[0]
    assert (KEYS - {"impl"}) | {"roofline", "gpu_launches", "clocks"} <= set(d)
    assert d["n_gpus"] == 1 and d["steps"] == 3 and d["warmup"] == 3 and d["value"] > 0
    roof = d["roofline"]
    assert roof["bound"] in ("hbm", "tensor") and roof["achieved"] > 0 and roof["peak"] > 0
    assert abs(roof["frac"] - roof["achieved"] / roof["peak"]) < 1e-9
    e2e = d["e2e"]
    assert e2e["value"] > 0 and e2e["h2d_bytes_per_step"] > 0 and e2e["d2h_bytes_per_step"] > 0
    assert d["gpu_launches"] > 0
    clk = d["clocks"]
    assert {"sm_mhz", "sm_max_mhz", "reasons"} <= set(clk)
    assert clk["sm_max_mhz"] is None or clk["sm_max_mhz"] > 0  # None: no sample in a short run
