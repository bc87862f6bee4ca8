"""Host-side checks of bench.py that need no GPU: the reference arm (the
oracle timed on the host cores) prints one JSON line with the contract's
keys, also when launched as two gloo ranks, and the timing rules are
enforced on the command line."""

import json
import os
import socket
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _json_lines(text):
    out = []
    for line in text.splitlines():
        line = line.strip()
        if line.startswith("{"):
            out.append(json.loads(line))
    return out


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


ARGS = ["--impl", "reference", "--steps", "1", "--warmup", "3", "--cpu-sample-edge", "12"]


def test_reference_arm_prints_contract_line():
    r = subprocess.run([sys.executable, "bench.py"] + ARGS, cwd=ROOT, capture_output=True,
                       text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = _json_lines(r.stdout)
    assert len(lines) == 1
    d = lines[0]
    assert d["impl"] == "reference" and d["unit"] == "ms" and d["higher_is_better"] is False
    assert d["value"] > 0 and d["steps"] == 1 and d["warmup"] == 3 and d["n_gpus"] == 1
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["cores"] >= 1
    assert d["cpu_baseline"]["value"] == d["value"] and d["cpu_baseline"]["sample"]
    assert d["e2e"] == {"value": d["value"], "unit": "ms", "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}


def test_reference_arm_two_gloo_ranks_print_one_line():
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(_free_port()), "bench.py",
           "--gpus", "2"] + ARGS
    env = dict(os.environ, OMP_NUM_THREADS="2")
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=900, env=env)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = _json_lines(r.stdout)
    assert len(lines) == 1
    assert lines[0]["n_gpus"] == 2 and lines[0]["impl"] == "reference"


def test_warmup_below_three_is_rejected():
    r = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--warmup", "2"],
                       cwd=ROOT, capture_output=True, text=True, timeout=120)
    assert r.returncode != 0
    assert "warmup" in r.stderr


def test_cpu_baseline_entry_all_threads_and_one_core():
    code = ("import argparse, json, bench; a = argparse.Namespace(cpu_sample_edge=12, grid=256); "
            "print(json.dumps(bench.cpu_baseline_entry(a, (3 * 256 - 2) ** 3, 61)))")
    r = subprocess.run([sys.executable, "-c", code], cwd=ROOT, capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    d = _json_lines(r.stdout)[-1]
    assert d["kind"] == "port" and d["unit"] == "ms" and d["value"] > 0
    assert d["cores"] == (os.cpu_count() or 1) and d["sample"]
    one = d["single_core"]
    assert one["cores"] == 1 and one["unit"] == "ms" and one["value"] > 0 and one["sample"]
