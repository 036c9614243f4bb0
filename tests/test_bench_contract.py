"""CPU: the reference arm of bench.py runs on the host cores and prints the
one-line JSON contract (impl, metric, unit, value, cpu_baseline, e2e with
zero transfer bytes) that the device arm's line is compared with."""
from __future__ import annotations

import json
import subprocess
import sys

from conftest import ROOT


def test_reference_arm_prints_the_contract_line():
    out = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--steps", "1",
                          "--warmup", "3", "--equil", "5", "--cpu-systems", "3"], cwd=ROOT, capture_output=True,
                         text=True, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [l for l in out.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["unit"] == "atom-steps/s" and d["higher_is_better"] is True
    assert d["metric"].startswith("aggregate atom-steps/s")
    assert d["value"] > 0 and d["steps"] == 1 and d["warmup"] == 3 and d["n_gpus"] == 1
    cb = d["cpu_baseline"]
    assert cb["value"] == d["value"] and cb["kind"] in ("port", "reference") and cb["cores"] >= 1
    assert d["e2e"]["value"] == d["value"] and d["e2e"]["unit"] == d["unit"]
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["d2h_bytes_per_step"] == 0
    assert d["config"]["workload"] == "batch256" and d["config"]["systems"] == 256
    assert d["ms_per_step"] > 0 and d["gpu_launches"] == 0
    assert "3 stratified systems" in cb["sample"]


def test_both_arms_describe_the_same_workload():
    import argparse

    import bench

    args = argparse.Namespace(workload="batch256", systems=256, seed=20261203, equil=400, gpus=1)
    specs = bench.workload_sizes("batch256", 256, 20261203)
    cfg = bench.workload_config(args, specs)
    assert cfg["atoms_total"] == sum(10 * c * r for c, r, _ in specs)
    # the reference arm prints workload_config(args, specs) for the same args
    assert cfg == bench.workload_config(args, bench.workload_sizes("batch256", 256, 20261203))
