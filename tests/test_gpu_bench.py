"""bench.py's GPU workloads at small sizes: each prints one JSON line with the
fields the measurement contract needs (the full-size runs are what bench.py
reports; these keep every mode working)."""
import json
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def run(*args, timeout=600):
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), *args], capture_output=True,
                       text=True, timeout=timeout, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.strip()]
    assert len(lines) == 1, r.stdout[-2000:]
    return json.loads(lines[0])


def test_scale_mode_small():
    d = run("--n", "65536", "--k", "64", "--steps", "5", "--warmup", "3", "--no-sweep",
            "--no-host-build", "--no-autotune", "--no-extras")
    # per step the packing launch (a 16 MiB B at K = 64) and the SpMM
    assert d["value"] > 0 and d["ms_per_step"] > 0 and d["gpu_launches"] == 10
    for key in ("roofline", "cpu_baseline", "e2e", "clocks", "comparators"):
        assert d[key] is not None, key
    assert d["roofline"]["bound"] == "hbm" and 0 < d["roofline"]["frac"]
    assert d["e2e"]["h2d_bytes_per_step"] == 65536 * 64 * 4
    assert d["roofline"]["gather_model"]["floor_ms"] > 0
    assert d["accuracy"]["rel_fro_vs_fp64"] < 1e-3


def test_batch_mode_small():
    d = run("--workload", "batch", "--graphs", "12", "--rows-hi", "5000", "--steps", "2",
            "--warmup", "3")
    assert d["batch"]["bitwise_equal_to_separate"] is True
    assert d["batch"]["rel_fro_vs_fp64_max"] < 1e-3
    assert d["config"]["graphs"] == 12 and d["value"] > 0


def test_precision_mode_small():
    d = run("--workload", "precision", "--n", "131072")
    assert d["targets"]["tf32_rel_fro_le_1e-3"] and d["targets"]["3xtf32_rel_fro_le_1e-6"]


def test_serve_mode_small():
    d = run("--workload", "serve", "--rows-hi", "8000", timeout=900)
    cb = d["serve"]["continuous_batching"]
    assert all(v["achieved_rps"] > 0 and v["p99_ms"] >= v["p50_ms"] for v in cb.values())
    assert d["served_error"]["rel_fro_vs_fp64_max"] < 1e-3  # the TF32 tolerance


def test_small_mode():
    d = run("--workload", "small", "--steps", "20", "--warmup", "5")
    # one SpMM launch per step, after the launch that packs B when the tuned
    # shape packs it (a B of 8 MiB at K = 128)
    shape = d["run"]["launch_shape"]
    packs = shape["packed_b"] == 1 if isinstance(shape, dict) else True
    assert d["config"]["n_rows"] == 16384 and d["gpu_launches"] == 20 * (2 if packs else 1)
    assert d["ms_per_step"] > 0 and d["no_flush"]["ms_per_step"] > 0
    assert d["cpu_baseline"]["value"] > 0 and d["roofline"]["frac"] > 0


def test_reference_arm_gpu_kernels():
    from oracle import ref_gpu
    if not __import__("os").path.exists(ref_gpu.CUBIN):
        pytest.skip("reference kernels not built here")
    d = run("--impl", "reference", "--n", "65536", "--k", "64", "--steps", "2", "--warmup", "1")
    g = d["reference_gpu_kernels"]
    assert "unavailable" not in g, g
    assert g["by_k"]["64"]["ms"] > 0
    assert g["path"] == "plain" or g["plain_kernel_by_k"]["64"]["ms"] > 0
    assert d["value"] > 0 and d["impl"] == "reference"


def test_both_arms_print_the_same_config():
    """The reference arm and ours identify the workload with the same config
    dict (sizes, realised degrees, tiles, windows, groups, seed), so that a
    comparison of the two lines can check they measured the same thing."""
    ours = run("--n", "65536", "--k", "64", "--steps", "2", "--warmup", "3", "--no-sweep",
               "--no-host-build", "--no-autotune", "--no-extras", "--no-cpu-baseline", "--no-cusparse")
    ref = run("--impl", "reference", "--n", "65536", "--k", "64", "--steps", "2", "--warmup", "1",
              "--no-ref-gpu")
    assert ours["config"] == ref["config"]
    ours_s = run("--workload", "small", "--steps", "5", "--warmup", "3", "--no-cpu-baseline", "--no-autotune")
    ref_s = run("--impl", "reference", "--workload", "small", "--steps", "2", "--warmup", "1", "--no-ref-gpu")
    assert ours_s["config"] == ref_s["config"]


def test_profile_modes_run():
    """The commands the ncu summaries were made with keep running."""
    d = run("--profile", "1", "--n", "65536", "--k", "64")
    assert d["profile_launches"] == 1 and d["tiles"] > 0
    d = run("--profile-step", "2", "--n", "65536", "--k", "128", "--no-autotune")
    assert d["profile_steps"] == 2 and d["path"] in ("plain", "adaptive")
    d = run("--workload", "small", "--profile", "2")
    assert d["profile_launches"] == 2
