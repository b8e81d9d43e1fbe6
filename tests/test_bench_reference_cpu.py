"""The benchmark's reference arm (the oracle on the host cores) runs without a GPU: one JSON line
with the contract's keys, `impl: reference`, the same `config` as the GPU arm's line, a
cpu_baseline describing the run and an e2e object with no transfers; under torchrun with two
ranks only rank 0 prints, and both exit 0."""

import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ARGS = ["bench.py", "--impl", "reference", "--steps", "3", "--warmup", "3"]


def reference_lines(cmd):
    out = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    return [json.loads(ln) for ln in out.stdout.splitlines() if ln.startswith("{")]


def check_line(d, n_gpus):
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "higher_is_better", "scaling", "vs_baseline",
              "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert k in d, k
    assert d["impl"] == "reference"
    assert d["value"] > 0 and d["n_gpus"] == n_gpus and d["steps"] == 3 and d["warmup"] == 3
    assert d["higher_is_better"] is True
    assert "workload" in d["config"]
    cb = d["cpu_baseline"]
    assert cb["value"] == d["value"] and cb["unit"] == d["unit"] and cb["cores"] >= 1
    assert cb["kind"] in ("port", "reference") and cb["sample"]
    assert d["e2e"]["value"] == d["value"] and d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["d2h_bytes_per_step"] == 0


def test_reference_arm_single_process():
    """The default workload: whole frames of the batched configuration, as the GPU arm renders."""
    import bench

    lines = reference_lines([sys.executable] + ARGS)
    assert len(lines) == 1
    check_line(lines[0], 1)
    assert lines[0]["config"] == json.loads(json.dumps(bench.workloads()["batched"].config()))
    assert lines[0]["fragments_per_step"] == 45935231  # the full frame: 64 targets, 256 draws


def test_reference_arm_under_torchrun_two_ranks():
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2", "--master-addr",
           "127.0.0.1", "--master-port", "29573"] + ARGS + ["--gpus", "2", "--workload", "colored"]
    lines = reference_lines(cmd)
    assert len(lines) == 1  # rank 0 alone
    check_line(lines[0], 2)
