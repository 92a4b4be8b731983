"""The benchmark's command-line contract, on a machine without a GPU: the reference arm
(the CPU implementation of the loop, timed on the host cores) prints one JSON line
with the keys the contract names, and our arm fails loudly instead of falling back to
a CPU path."""
import json
import os
import subprocess
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def run(*args, timeout=600):
    return subprocess.run([sys.executable, os.path.join(REPO, "bench.py"), *args], capture_output=True, text=True,
                          timeout=timeout, cwd=REPO)


def test_reference_arm_prints_the_contract_line():
    r = run("--impl", "reference", "--steps", "1", "--warmup", "3", "--ref-seconds", "0.5")
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads(r.stdout.strip().splitlines()[-1])
    if "unavailable" in line:
        pytest.skip(line["unavailable"])
    metric = json.load(open(os.path.join(REPO, "BASELINE.json")))["metric"]
    assert line["impl"] == "reference" and line["metric"] == metric
    assert line["unit"] == "samples/s" and line["higher_is_better"] is True
    assert line["value"] > 0 and line["steps"] == 1 and line["warmup"] == 3
    cb = line["cpu_baseline"]
    assert cb["kind"] in ("reference", "port") and cb["cores"] >= 1 and cb["value"] == line["value"] and cb["sample"]
    e2e = line["e2e"]
    assert e2e["value"] == line["value"] and e2e["unit"] == line["unit"]
    assert e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0
    assert "workload" in line["config"]


def test_our_arm_needs_a_gpu():
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    r = run("--steps", "1", "--warmup", "3", "--no-configs", "--batched", "none", timeout=300)
    assert r.returncode != 0
    assert not any(l.startswith("{") and '"value"' in l for l in r.stdout.splitlines())
