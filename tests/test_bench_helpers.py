"""The pure helpers behind bench.py's JSON line, on CPU: the reference's
algorithmic byte count (mttkrp_cuda_onekernel.cu:94-97), the workload both
arms report, the peak lookup, the ncu traffic figure read from the committed
summary, and the served request stream's distributions."""
import json
import math
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
import bench as B  # noqa: E402


def test_algorithmic_bytes_formula():
    # nnz * (4N + 4) + sum_m I_m * R * 4: 2.3712 GB per launch on the power-law workload
    assert B.algo_bytes(B.DIMS, 100_000_000, 32) == 100_000_000 * 16 + (4_000_000 + 2_000_000 + 25_000) * 128
    assert abs(B.algo_bytes(B.DIMS, 100_000_000, 32) / 1e9 - 2.3712) < 1e-4
    # order 4: 20 bytes per nonzero
    assert B.algo_bytes([10, 20, 30, 40], 1000, 16) == 1000 * 20 + 100 * 16 * 4


def test_workload_config_is_shared_and_json():
    c1 = B.workload_config(100_000_000, 1)
    c2 = B.workload_config(100_000_000, 4)
    assert c1["workload"] == c2["workload"] and c1["dims"] == B.DIMS and c1["rank"] == 32
    assert c1["parallelism"] == "single" and c2["parallelism"] == "replicas"
    json.dumps(c1)


def test_peak_lookup_and_traffic_figure():
    peak, kind = B.peaks()
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        assert kind == "measured" and peak == float(json.load(open(path))["hbm_gbs"])
    else:
        assert (peak, kind) == (6800.0, "fallback")
    traffic = B.traffic_per_launch()
    # the committed ncu summary: DRAM bytes per launch above the algorithmic count
    assert traffic is not None and traffic > B.algo_bytes(B.DIMS, 100_000_000, 32)


def test_serve_stream_distributions():
    reqs = B.serve_stream(4096)
    assert len(reqs) == 4096
    arr = np.array([r["arrival"] for r in reqs])
    assert np.all(np.diff(arr) > 0)
    assert abs(4096 / arr[-1] - B.SERVE_RATE) < 0.1 * B.SERVE_RATE       # Poisson at ~2,000/s
    orders = [len(r["dims"]) for r in reqs]
    assert abs(orders.count(3) / 4096 - 0.5) < 0.05
    assert all(64 <= d <= 100_000 for r in reqs for d in r["dims"])
    assert all(1 <= r["nnz"] <= 1_000_000 and r["nnz"] <= 0.5 * math.prod(r["dims"]) + 1 for r in reqs)
    assert {r["rank"] for r in reqs} == {8, 16, 32, 64}
    assert B.serve_stream(16) == B.serve_stream(16)                       # seeded
