"""bench.py's reference arm on the CPU, for every workload: the bounded CPU
sample of each workload runs through the reference (or the oracle's port)
and the JSON line carries the contract's keys.  No GPU is needed."""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402

KEYS = {"impl", "metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step",
        "higher_is_better", "scaling", "vs_baseline", "dtype", "data", "config",
        "cpu_baseline", "e2e"}


@pytest.mark.parametrize("workload", sorted(bench.WORKLOADS))
def test_reference_arm_runs(workload):
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                        "--workload", workload, "--steps", "1", "--warmup", "0",
                        "--cpu-sample", "20000", "--ref-sample-only"],
                       cwd=ROOT, stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads(r.stdout.strip().splitlines()[-1])
    assert KEYS <= set(line), KEYS - set(line)
    assert line["impl"] == "reference" and line["value"] > 0
    assert line["dtype"] == bench.DTYPE_OF[workload]
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["cpu_baseline"]["cores"] >= 1
    assert line["config"]["workload"]


def test_published_baseline_only_for_its_workload():
    cls, n = bench.WORKLOADS["object_point3d"]
    wl = cls(None, None, n, None)
    assert n in wl.published and wl.published[n] == pytest.approx((1 << 20) / 51.58e-3 / 1e9)
    for name, (c, n_full) in bench.WORKLOADS.items():
        if name != "object_point3d":
            assert not getattr(c, "published", None), name


def test_reference_arm_times_the_full_workload_when_it_fits():
    """A workload that fits the budget is timed at its full size (same_config)."""
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                        "--workload", "qsort_f32_2e20", "--steps", "2", "--warmup", "1",
                        "--cpu-sample", "65536"],
                       cwd=ROOT, stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads(r.stdout.strip().splitlines()[-1])
    assert line["config"]["same_config"] is True
    assert line["cpu_baseline"]["sample"] == f"{1 << 20} keys per step"
    assert line["cpu_baseline"]["input_restore"] == "outside the timed region"
    assert line["reference_x86_host"]["value"] > 0
