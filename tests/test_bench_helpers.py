"""Host logic of the measurement (bench.py), on CPU: the roofline object's arithmetic, latency
grouping per kind and size class, and the serving entry's CPU baseline (the oracle on the same
requests), whose vertex count must equal the oracle's own counts for those requests."""

import os
import sys

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))

import bench  # noqa: E402
from lyon_gb300 import serving, workloads  # noqa: E402
from oracle import lyon_oracle as orc  # noqa: E402


def test_roofline_entry_arithmetic():
    r = bench.roofline_entry(2.0e9, 0.5, "k", traffic=3.0e9)
    assert r["bound"] == "hbm" and r["unit"] == "GB/s"
    assert abs(r["achieved"] - 4.0) < 1e-12
    assert abs(r["frac"] - r["achieved"] / r["peak"]) < 1e-15
    assert r["traffic"] == 3.0e9 and r["kernel_ms"] == 500.0


def test_latency_groups_split_kinds_and_sizes():
    sb, so = workloads.plain_stroke(200, seed=1)
    fb, fo = workloads.glyph_fill(50, seed=3)
    reqs = [serving.Request(serving.KIND_STROKE, sb, 0, 10, so),
            serving.Request(serving.KIND_FILL, fb, 0, 5, fo),
            serving.Request(serving.KIND_STROKE, sb, 0, 150, so)]
    # Latencies in arrival order; arrival k submitted request k % 3.
    lat = [1.0, 100.0, 2.0, 3.0, 200.0, 4.0]
    g = bench._latency_groups({"latencies_ms": lat}, reqs)
    assert g["stroke_all"]["requests"] == 4
    assert g["fill_all"]["requests"] == 2
    assert g["stroke_le_1000_paths"]["max_ms"] == 4.0
    assert g["fill_le_1000_paths"]["p50_ms"] == 150.0
    assert "stroke_gt_1000_paths" not in g


def test_serving_cpu_baseline_counts_the_oracles_vertices():
    sp, so = workloads.plain_stroke(400, seed=1)
    fp, fo = workloads.glyph_fill(120, seed=3)
    reqs = serving.mixed_requests(sp, so, fp, fo, 12, seed=5, max_paths=60)
    r = bench._serving_cpu_baseline(reqs, count=12)
    want = 0
    for q in reqs:
        sub = q.batch.subset(range(q.start, q.start + q.count))
        res = orc.batch("stroke" if q.kind == serving.KIND_STROKE else "fill", sub, q.options,
                        32, 2, want_output=False)
        want += int(np.asarray(res["vtx_counts"]).sum())
    assert f"{want} output vertices" in r["sample"]
    assert r["value"] > 0 and r["requests_per_s"] > 0 and r["kind"] == "port"
