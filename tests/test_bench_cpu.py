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


ARGS = ["--impl", "reference", "--steps", "2", "--warmup", "3", "--grid", "16"]


def test_reference_arm_prints_contract_line():
    r = subprocess.run([sys.executable, "bench.py"] + ARGS, cwd=ROOT, capture_output=True,
                       text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = _json_lines(r.stdout)
    assert len(lines) == 1
    d = lines[0]
    assert d["impl"] == "reference" and d["unit"] == "ms" and d["higher_is_better"] is False
    assert d["value"] > 0 and d["steps"] == 2 and d["warmup"] == 3 and d["n_gpus"] == 1
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["cores"] >= 1
    assert d["cpu_baseline"]["value"] == d["value"] and d["cpu_baseline"]["sample"]
    assert d["e2e"] == {"value": d["value"], "unit": "ms", "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}
    # the workload itself: 16^3 27-point rows and non-zeros, each step one
    # full solve to 1e-8
    n, nnz = 16 ** 3, (3 * 16 - 2) ** 3
    assert d["config"]["rows"] == n and d["config"]["nnz"] == nnz
    assert d["oracle_iterations"] > 1 and d["final_rel_residual"] <= 1e-8
    assert d["value"] == d["ms_per_step"]
    import bench

    args = bench.argparse.Namespace(grid=16)
    assert d["config"] == bench.workload_config(args, n, nnz, 1)


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


def test_oracle_legs_parity_and_cpu_baseline():
    """The GPU line's CPU legs on a 16^3 case: the oracle with the GPU
    hierarchy's parameters reports its levels and iterations beside the
    given GPU figures; the CPU baseline is one full solve with lineal's
    partitions, the one-core figure explicitly omitted."""
    code = ("import argparse, json, bench; a = argparse.Namespace(grid=16, partition_size=512, "
            "partition_growth=4.0, min_partitions=8, coarse_smallest_last=False); "
            "p, c = bench.oracle_legs(a, [4096, 1], 7); print(json.dumps([p, c]))")
    r = subprocess.run([sys.executable, "-c", code], cwd=ROOT, capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    par, cpu = json.loads(r.stdout.strip().splitlines()[-1])
    assert par["gpu_iterations"] == 7 and par["oracle_iterations"] > 0
    assert par["oracle_levels"][0] == 4096 and par["levels_equal"] is False
    assert par["oracle_rel_residual"] <= 1e-8
    assert cpu["kind"] == "port" and cpu["unit"] == "ms" and cpu["value"] > 0
    assert cpu["cores"] == (os.cpu_count() or 1) and cpu["iterations"] > 0
    assert "omitted" in cpu["single_core"]
