"""bench.py's host logic without a GPU: the compulsory-byte model, the
reference arm (the CPU CSR SpMM on a small workload), the replica
aggregation across ranks (two gloo processes on CPU), the DRAM-traffic
figure keyed by the kernel sources, and the clock summary."""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402


def test_algorithmic_bytes_of_the_1m_row_workload():
    # 4 nnz + 8T + 4(T+1) + 32T + 4(W+1) + 4 cols K + 32 W K at K = 128
    nnz, T, W, n = 32_179_233, 4_031_464, 131_072, 1 << 20
    b = bench.algorithmic_bytes(nnz, T, W, n, 128)
    assert b == 4 * nnz + 8 * T + 4 * (T + 1) + 32 * T + 4 * (W + 1) + 4 * n * 128 + 32 * W * 128
    assert 1.37e9 < b < 1.39e9
    assert bench.algorithmic_bytes(nnz, T, W, n, 128, G=253_000) == b + 4 * T + 4 * 253_001


def test_reference_arm_prints_one_json_line():
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                        "--steps", "2", "--warmup", "1", "--n", "16384", "--k", "32"],
                       capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr
    lines = [ln for ln in r.stdout.splitlines() if ln.strip()]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["unit"] == "GFLOP/s" and d["value"] > 0
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["cpu_baseline"]["cores"] >= 1
    assert d["higher_is_better"] is True


def _rank(rank, world, port, ms, out):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    got = bench.replica_throughput(ms, 2e9, world, "cpu")
    out.put((rank, got))
    dist.destroy_process_group()


def test_replica_throughput_takes_the_slowest_rank_over_gloo():
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + os.getpid() % 1000
    ps = [ctx.Process(target=_rank, args=(r, 2, port, [2.0, 4.0][r], q)) for r in range(2)]
    for p in ps:
        p.start()
    res = dict(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=60)
    for r in (0, 1):
        ms, gf = res[r]
        assert ms == pytest.approx(4.0)
        assert gf == pytest.approx(2e9 * 2 / 4e-3 / 1e9)
    assert bench.replica_throughput(2.0, 2e9, 1) == (2.0, pytest.approx(1000.0))


def test_reference_kernel_launch_config():
    """The reference's TF32Compute choices (include/tf32_comp.hpp:19-31,
    52-111; thresholds 512 plain and 128 adaptive, src/mma_tf32.cu:218)."""
    from oracle import ref_gpu
    assert ref_gpu.launch_config(128, False, 131072) == ("tf32_mma_kernel", 131072, (32, 4))
    assert ref_gpu.launch_config(256, False, 10) == ("tf32_mma_kernel", 10, (32, 8))
    assert ref_gpu.launch_config(1024, False, 10) == ("tf32_mma_g512_kernel", 10, (32, 16))
    assert ref_gpu.launch_config(32, True, 10, 7) == ("tf32_mma_balance_kernel", 7, (32, 1))
    assert ref_gpu.launch_config(128, True, 10, 7) == ("tf32_mma_balance_kernel", 7, (32, 4))
    assert ref_gpu.launch_config(256, True, 10, 7) == ("tf32_mma_balance_g128_kernel", 7, (32, 4))
    import torch
    if not torch.cuda.is_available():
        assert ref_gpu.available() is not None


def test_measured_traffic_is_keyed_by_the_kernel_sources(monkeypatch):
    """roofline.traffic is reported only while the kernel sources hash to the
    value its ncu capture was taken on; otherwise null with the reason."""
    got, src = bench.measured_traffic(128)
    assert got == bench.TRAFFIC[128]["bytes"] and bench.TRAFFIC[128]["src_sha"] in src
    monkeypatch.setattr(bench, "kernel_source_hash", lambda: "0000000000000000")
    got, src = bench.measured_traffic(128)
    assert got is None and src.startswith("stale")
    got, src = bench.measured_traffic(64)
    assert got is None and "no ncu capture" in src


def test_clock_summary_takes_the_median_and_every_reason():
    c = bench.ClockSampler(0)
    c.source = "test"
    assert c.summary()["samples"] == 0
    c.samples = [(2070.0, 2070.0, set()), (1900.0, 2070.0, {"sw_power_cap"}), (2070.0, 2070.0, set()),
                 (1500.0, 2070.0, {"hw_slowdown", "sw_power_cap"})]
    s = c.summary()
    assert s["sm_mhz"] == 1985.0 and s["sm_max_mhz"] == 2070.0 and s["samples"] == 4
    assert s["reasons"] == ["hw_slowdown", "sw_power_cap"]
