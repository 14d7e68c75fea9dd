"""The benchmark's reference arm keeps the JSON-line contract (CPU only:
the reference arm runs the oracle's restatement of the reference algorithm
on the host cores)."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _run(*args):
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), *args], cwd=ROOT, capture_output=True,
                         text=True, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [l for l in out.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, out.stdout[-2000:]
    return json.loads(lines[0])


def test_reference_arm_line():
    d = _run("--impl", "reference", "--workload", "config1", "--steps", "1", "--warmup", "1")
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
              "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert k in d, k
    assert d["impl"] == "reference" and d["value"] > 0 and d["higher_is_better"] is True
    assert d["warmup"] >= 3  # at least three warm-up steps whatever is asked
    assert d["config"]["workload"]
    cb = d["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == d["value"] and cb["sample"]
    assert cb["extrapolated"] is False  # config 1 runs every point
    assert "reference_gpu_spread" in d  # timed on a GPU box, "unavailable" here
    e = d["e2e"]
    assert e["value"] == d["value"] and e["h2d_bytes_per_step"] == 0 and e["d2h_bytes_per_step"] == 0


def test_reference_arm_unavailable_workload():
    d = _run("--impl", "reference", "--workload", "batch", "--steps", "1")
    assert d["impl"] == "reference" and d["unavailable"]


def test_library_line_cpu_baseline_is_the_reference_arm_in_a_child():
    """The library line's cpu_baseline comes from the reference arm's code run
    in a child process without a CUDA context (both arms' CPU figures are
    then one measurement method)."""
    import argparse
    sys.path.insert(0, ROOT)
    import bench
    cb = bench.cpu_baseline_isolated(argparse.Namespace(workload="config1", K=None), steps=1)
    assert "unavailable" not in cb, cb
    assert cb["kind"] == "port" and cb["value"] > 0 and cb["cores"] >= 1 and cb["sample"]
    assert cb["extrapolated"] is False and "child process" in cb["process"]


def test_points_option_is_for_the_clustered_workload_only():
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--workload", "polar",
                          "--points", "1000"], cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert out.returncode == 2 and "--points" in out.stderr
