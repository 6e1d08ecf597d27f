"""bench.py's GPU arm prints one JSON line with every key of the bench
contract, on a small batched case (4 scenes), and its records are consistent."""
import json
import subprocess
import sys
from pathlib import Path

import pytest

pytestmark = pytest.mark.gpu

REPO = Path(__file__).resolve().parents[1]


def test_bench_line_keeps_the_contract():
    cmd = [sys.executable, str(REPO / "bench.py"), "--scenes", "4", "--fixed-config",
           "--block", "128", "--parts", "2", "--steps", "4", "--warmup", "3", "--no-adjoint",
           "--no-cpu", "--no-sub"]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=900, cwd=REPO)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, r.stdout[-2000:]
    d = json.loads(lines[0])
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step",
                "higher_is_better", "scaling", "vs_baseline", "dtype", "data", "config",
                "e2e", "gpu_launches", "roofline", "clocks", "cpu_baseline"):
        assert key in d, key
    assert d["n_gpus"] == 1 and d["steps"] == 4 and d["warmup"] == 3
    assert d["value"] > 0 and d["ms_per_step"] > 0
    assert d["e2e"]["h2d_bytes_per_step"] > 0 and d["e2e"]["d2h_bytes_per_step"] > 0
    assert d["e2e"]["identical_to_one_batch"] is True
    assert d["parts"]["count"] == 2 and d["parts"]["identical_to_one_batch"] is True
    assert d["identical_to_per_scene"]["equal"] is True
    assert d["identical_to_per_scene"]["other_form_equal"] is True
    rf = d["roofline"]
    assert rf["bound"] == "hbm" and rf["peak"] > 0 and 0 < rf["frac"] < 1.5
    assert d["gpu_launches"] == d["forms"]["separate"]["launches_per_step"] * 2 * 4
    assert "sm_mhz" in d["clocks"]


def test_brute_line_counts_the_pairs_it_filters():
    """The brute-force workload's line: agent-queries/s of the 65,536-agent
    call, with the pairs its distance filter ran on well below a full scan's
    (the bucketed scan skips chunks beyond every bound) and its issue rate."""
    cmd = [sys.executable, str(REPO / "bench.py"), "--workload", "brute", "--steps", "3",
           "--warmup", "3", "--no-cpu"]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=900, cwd=REPO)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, r.stdout[-2000:]
    d = json.loads(lines[0])
    assert d["metric"] == "agent-queries/s" and d["value"] > 0
    rf = d["roofline"]
    assert 0 < rf["pairs_evaluated"] < rf["pairs_all"] / 10
    assert rf["pairs_all"] == 65536.0 * 65535
    assert d["issue"] is not None and 0 < d["issue"]["frac"] < 1.5
    assert d["gpu_launches"] == 10 * 3  # ten launches per call
