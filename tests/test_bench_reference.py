"""bench.py's reference arm (`--impl reference`: the oracle's float
restatement of the reference solver loop on the host cores) on the CPU: the
JSON line it prints carries the keys the benchmark contract names, the same
metric and workload as the GPU arm, and under a two-rank launch only rank 0
prints while the other exits 0 without work."""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def last_json(out):
    lines = [l for l in out.strip().splitlines() if l.startswith("{")]
    return [json.loads(l) for l in lines]


def run(cmd, env=None):
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True,
                       timeout=600, env=env)
    assert r.returncode == 0, r.stderr[-2000:]
    return r.stdout


def test_reference_arm_line():
    sys.path.insert(0, ROOT)
    import bench
    out = run([sys.executable, "bench.py", "--impl", "reference",
               "--steps", "1", "--warmup", "1"])
    lines = last_json(out)
    assert len(lines) == 1
    d = lines[0]
    assert d["impl"] == "reference"
    assert d["metric"] == bench.METRIC
    assert d["unit"] == "cell-updates/s" and d["higher_is_better"] is True
    assert d["value"] > 0 and d["n_gpus"] == 1 and d["steps"] == 1
    assert d["warmup"] >= 3          # at least 3 warm-up steps, always
    p, gap, _ = bench.workload_params()
    assert d["config"]["workload"] == \
        bench.config_dict(p, gap, "")["workload"]
    cb = d["cpu_baseline"]
    assert cb["kind"] in ("port", "reference") and cb["cores"] >= 1
    assert cb["value"] == d["value"]
    e = d["e2e"]
    assert e["value"] == d["value"] and e["unit"] == d["unit"]
    assert e["h2d_bytes_per_step"] == 0 and e["d2h_bytes_per_step"] == 0


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_reference_arm_two_ranks():
    pytest.importorskip("torch")
    out = run([sys.executable, "-m", "torch.distributed.run", "--nnodes=1",
               "--nproc-per-node", "2", "--master-addr", "127.0.0.1",
               "--master-port", str(free_port()), "bench.py", "--impl",
               "reference", "--gpus", "2", "--steps", "1", "--warmup", "1"])
    lines = last_json(out)
    assert len(lines) == 1
    assert lines[0]["impl"] == "reference" and lines[0]["n_gpus"] == 2
