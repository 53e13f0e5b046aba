"""Serving loop: requests of mixed kinds and sizes submitted together are coalesced into batched
launches; every request's result must equal the result of the same request run alone (the
batched entry point on just its paths, u32 indices in one id space per request)."""

import numpy as np
import pytest

from lyon_gb300 import serving, workloads
from lyon_gb300 import tessellation as T

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def pools():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    sb, so = workloads.plain_stroke(3000, seed=31)
    sb2, so2 = workloads.batched_stroke(2000, seed=32)
    fb, fo = workloads.glyph_fill(800, seed=33)
    return sb, so, sb2, so2, fb, fo


def _alone(ctx, req):
    """The request by itself through lyon_gpu_stroke_paths / lyon_gpu_fill_paths."""
    sub = req.batch.subset(range(req.start, req.start + req.count))
    db = T.DeviceBatch.upload(sub, 0)
    od = T.upload_options(req.options, 0)
    kind = "stroke" if req.kind == serving.KIND_STROKE else "fill"
    res = T.tessellate_paths(kind, db, od, len(req.options), 32, T.INDEX_GLOBAL, 0, ctx)
    ctx.synchronize()
    v = res.vertices().cpu().numpy() if res.total_vertices else np.zeros((0, 2), np.float32)
    i = res.indices().cpu().numpy().view(np.uint32) if res.total_indices else np.zeros(0, np.uint32)
    st = res.statuses().cpu().numpy()
    return v, i, st


@pytest.mark.parametrize("stroke_workers", [0, 2])
def test_mixed_requests_equal_alone(pools, stroke_workers):
    # With stroke workers, strokes run on their own high-priority streams with one stroke block
    # per SM while fill sweeps keep at most 8 blocks per SM: the results must not change.
    sb, so, sb2, so2, fb, fo = pools
    rng = np.random.default_rng(7)
    reqs = []
    for k in range(48):
        choice = k % 3
        pool, opts, kind = [(sb, so, serving.KIND_STROKE), (sb2, so2, serving.KIND_STROKE),
                            (fb, fo, serving.KIND_FILL)][choice]
        n = int(rng.choice([1, 2, 7, 40, 150, 600]))
        n = min(n, pool.num_paths)
        start = int(rng.integers(0, pool.num_paths - n + 1))
        o = opts if len(opts) == 1 else opts[start:start + n]
        reqs.append(serving.Request(kind, pool, start, n, o))
    srv = serving.Server(0, num_workers=2, max_batch_paths=1500,
                         num_stroke_workers=stroke_workers, max_stroke_batch_paths=1500)
    try:
        tickets = [srv.submit(r) for r in reqs]  # all queued at once: coalesced into batches
        ctx = T.Context(0)
        for r, t in zip(reqs, tickets):
            res = srv.wait(t)
            assert res.status == 0
            v, i, vo, st = res.host_copy()
            av, ai, ast = _alone(ctx, r)
            assert np.array_equal(st, ast)
            assert np.array_equal(i, ai)
            assert np.array_equal(v, av)
            assert res.latency_ms >= res.queue_ms >= 0.0
            srv.release(t)
    finally:
        srv.close()


def test_load_runner_completes_every_request(pools):
    sb, so, _, _, fb, fo = pools
    reqs = serving.mixed_requests(sb, so, fb, fo, 64, seed=3, max_paths=500)
    srv = serving.Server(0, num_workers=2)
    try:
        st = srv.run_load(reqs, rate_per_s=500.0, duration_s=0.5, seed=11, want_latencies=True)
    finally:
        srv.close()
    assert st["submitted"] > 0 and st["completed"] == st["submitted"]
    assert st["failed"] == 0
    assert st["p50_ms"] <= st["p99_ms"] <= st["max_ms"]
    assert len(st["latencies_ms"]) == st["completed"]


def test_lone_request_reaches_its_lane(pools):
    # One request at a time into a server with stroke and fill lanes: each must be taken by a
    # worker of its kind although nothing else is queued (a wake-up that reaches only a worker of
    # the other kind would leave it waiting). Polled with a deadline, so a lost wake-up fails the
    # test instead of blocking it.
    import time
    sb, so, _, _, fb, fo = pools
    srv = serving.Server(0, num_workers=2, num_stroke_workers=2)
    try:
        cfg = srv.config()
        assert cfg["num_workers"] == 2 and cfg["num_stroke_workers"] == 2
        assert cfg["fill_blocks_per_sm"] == 8
        for kind, pool, opts, n in ((serving.KIND_STROKE, sb, so, 1500),
                                    (serving.KIND_FILL, fb, fo, 300),
                                    (serving.KIND_STROKE, sb, so, 1)):
            t = srv.submit(serving.Request(kind, pool, 0, n, opts))
            deadline = time.monotonic() + 60.0
            res = srv.poll(t)
            while res is None and time.monotonic() < deadline:
                time.sleep(0.001)
                res = srv.poll(t)
            assert res is not None, f"request of kind {kind} not served within 60 s"
            assert res.status == 0 and res.num_paths == n
            srv.release(t)
    finally:
        srv.close()
