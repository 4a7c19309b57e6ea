"""bench.py on the CPU: the reference arm (the reference's CPU algorithm timed
on the host cores) prints a line with every key of the benchmark contract, and
the command line offers every workload.  No GPU is touched."""
import argparse
import importlib.util
import json
import subprocess
import sys

import pytest

import helpers

BENCH = helpers.ROOT / "bench.py"


def load_bench():
    spec = importlib.util.spec_from_file_location("bench_under_test", BENCH)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_cli_lists_every_workload():
    out = subprocess.run([sys.executable, str(BENCH), "--help"], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stderr
    for w in ("lloyd", "bigk", "kkm", "kkm-panel", "batch"):
        assert w in out.stdout


def test_reference_arm_line():
    b = load_bench()
    args = argparse.Namespace(gpus=1, steps=1, warmup=0, impl="reference", workload="lloyd")
    line = b.reference_arm(args, 0)
    json.dumps(line)                                          # one JSON line
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "scaling", "vs_baseline", "dtype", "data", "config", "impl", "cpu_baseline", "e2e"):
        assert key in line, key
    assert line["impl"] == "reference" and line["metric"] == b.METRIC and line["unit"] == "iters/s"
    assert line["value"] > 0 and line["higher_is_better"] is True
    cb = line["cpu_baseline"]
    assert cb["value"] == line["value"] and cb["kind"] in ("reference", "port") and cb["cores"] >= 1
    assert line["e2e"] == {"value": line["value"], "unit": "iters/s", "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}
    assert line["config"]["workload"].startswith("lloyd n=1048576 d=128 k=256")
    assert b.reference_arm(args, 1) is None                   # other ranks do no work


def test_reference_arm_loads_no_product_library():
    """In a process of its own the reference arm maps only oracle libraries:
    its data come from the numpy twin of the product's generator."""
    out = subprocess.run([sys.executable, str(BENCH), "--impl", "reference", "--steps", "1", "--warmup", "0"],
                         capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr
    line = json.loads(out.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference"
    assert not [x for x in line["repo_libraries_loaded"] if x.startswith("matrix-centric-k-means_gb300")]
    assert any(x.startswith("oracle") for x in line["repo_libraries_loaded"])


@pytest.mark.parametrize("use_ref", [False, True])
def test_cpu_sample_scales_to_the_full_workload(km, use_ref):
    """A sample of the rows is timed and scaled by n / rows to full iterations/s."""
    if use_ref and helpers.reference_lib() is None:
        pytest.skip("the reference CPU build is not present")
    b = load_bench()
    X = km.synth_blobs(8192, b.D, b.BLOBS, b.LO, b.HI, b.SIGMA, b.DATA_SEED, nthreads=4)
    ips, secs, reps = b.run_cpu_sample(X, 2, 8192, 0.0, use_ref)
    assert reps == 1 and secs > 0
    assert ips == pytest.approx(1.0 / (secs * b.N / 8192))
