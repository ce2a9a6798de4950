"""The reference arm of bench.py on CPU: the CPU FP64 restatement timed on the same workload and
`config` as the GB300 arm, and the scaling of a bounded sample to a full solve."""
import argparse
import contextlib
import io
import json
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def _reference_line(workload):
    import bench
    args = argparse.Namespace(workload=workload, steps=1, warmup=0, gpus=1, cpu_iterations=2)
    buf = io.StringIO()
    with contextlib.redirect_stdout(buf):
        bench.run_reference(args, 0)
    return json.loads(buf.getvalue().strip().splitlines()[-1])


def test_reference_line_has_the_gb300_arms_config():
    import bench
    line = _reference_line("ring")
    _, _, cfg = bench.workload("ring")
    assert line["impl"] == "reference"
    assert line["config"] == bench.bench_config(cfg)
    assert line["metric"] == bench.METRIC and line["unit"] == "ms" and line["higher_is_better"] is False
    cb = line["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == line["value"]
    assert line["e2e"] == {"value": line["value"], "unit": "ms", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    assert "complete converged solve" in cb["sample"]


def test_sample_scaling_counts_the_finalisation_once():
    import bench
    prob, opts, _ = bench.workload("ring")
    ms, info = bench.cpu_sample(prob, opts, 2, 50)
    assert info["sample_iterations"] == 2
    assert info["fixed_ms"] >= 0.0
    assert abs(ms - (info["fixed_ms"] + 50 * info["per_iteration_ms"])) <= 1e-9 * ms
    # the loop's own clock lies inside the call's
    assert info["fixed_ms"] + 2 * info["per_iteration_ms"] <= info["sample_seconds"] * 1e3 * (1 + 1e-12)
