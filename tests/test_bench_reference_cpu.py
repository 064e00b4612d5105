"""The benchmark's reference arm on CPU: `bench.py --impl reference` times
the reference's own CPU code (its ver-c/src, built from the staged sources;
the oracle, its restatement in C, where that build is absent) on the host
cores and prints the JSON line of the benchmark contract.  No GPU is
involved."""
from __future__ import annotations

import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_prints_the_contract_line():
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    if not os.path.exists(O.LIB_PATH):
        pytest.skip("oracle library not built")
    p = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--workload", "uniform",
                        "--n", "3000", "--steps", "2", "--warmup", "1", "--cpu-sample", "64"],
                       capture_output=True, text=True, timeout=300, cwd=ROOT)
    assert p.returncode == 0, p.stderr[-2000:]
    line = json.loads(p.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference"
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "higher_is_better", "config", "cpu_baseline",
              "e2e"):
        assert k in line, k
    kind = "reference" if O.reference_available() else "port"
    assert line["value"] > 0 and line["cpu_baseline"]["kind"] == kind and line["cpu_baseline"]["cores"] >= 1
    # a step is one timed batch of sampled targets
    assert 0 < line["ms_per_step"] < 300_000
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["value"] == line["value"]
    assert line["config"]["n_blobs"] == 3000


def test_roofline_traffic_figures_parse():
    """The per-launch DRAM bytes that `bench.py` puts in its roofline object
    come from the committed ncu summary: one figure per form at the headline
    workload, each a plausible per-launch byte count (more than the blobs'
    own 16 bytes each, less than 16 GB)."""
    sys.path.insert(0, ROOT)
    import bench
    t = bench.roofline_traffic()
    for mode in ("plain", "mixed", "learned"):
        key = f"{mode}:two_patch_sheet_4M"
        assert key in t, key
        assert 16 * 4_194_304 < t[key] < 16 << 30, (key, t[key])
