"""The bench's reference arm, run on the CPU as it runs on a GPU host: one JSON line with the contract's keys, the
same workload description as the GPU arm, no host copies, and none of the engine's native code loaded (the arm times
the oracle's C restatement of the reference's serial path on the host cores)."""
import json
import os
import socket
import subprocess
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

# Runs bench.py in-process, then reports which shared objects the process mapped.
PROBE = """
import json, runpy, sys
sys.argv = ['bench.py', '--impl', 'reference', '--steps', '1', '--warmup', '0']
runpy.run_path('bench.py', run_name='__main__')
maps = open('/proc/self/maps').read()
print(json.dumps({'mapped': sorted({l.split()[-1] for l in maps.splitlines() if l.split()[-1].endswith('.so')})}))
"""


def _json_lines(text):
    return [json.loads(line) for line in text.splitlines() if line.startswith("{")]


def _check_line(line, n_gpus):
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
                "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert key in line, key
    assert line["impl"] == "reference"
    assert line["n_gpus"] == n_gpus and line["steps"] == 1 and line["warmup"] == 0
    assert line["value"] > 0 and line["ms_per_step"] > 0 and line["higher_is_better"] is True
    baseline = line["cpu_baseline"]
    assert baseline["kind"] in ("port", "reference") and baseline["cores"] >= 1 and baseline["sample"]
    assert baseline["value"] == pytest.approx(line["value"])
    e2e = line["e2e"]
    assert e2e["value"] == pytest.approx(line["value"]) and e2e["unit"] == line["unit"]
    assert e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0
    config = line["config"]
    for key in ("workload", "pairs", "cells_per_step", "input_bytes_per_step"):
        assert key in config, key
    assert config["pairs"] == 1 << 20 and config["cells_per_step"] > 4e10


def test_reference_arm_line_and_libraries():
    run = subprocess.run([sys.executable, "-c", PROBE], cwd=REPO, capture_output=True, text=True, timeout=600)
    assert run.returncode == 0, run.stderr[-2000:]
    lines = _json_lines(run.stdout)
    assert len(lines) == 2, run.stdout[-2000:]
    _check_line(lines[0], 1)
    mapped = lines[1]["mapped"]
    assert not any("libszs_gb300" in path for path in mapped), mapped
    assert any(path.endswith("liboracle_port.so") for path in mapped), mapped


def test_reference_arm_under_torchrun_prints_one_line():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    command = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
               "--master-addr", "127.0.0.1", "--master-port", str(port), "bench.py", "--impl", "reference",
               "--gpus", "2", "--steps", "1", "--warmup", "0"]
    run = subprocess.run(command, cwd=REPO, capture_output=True, text=True, timeout=600)
    assert run.returncode == 0, run.stderr[-2000:]
    lines = _json_lines(run.stdout)
    assert len(lines) == 1, run.stdout[-2000:]
    _check_line(lines[0], 2)
