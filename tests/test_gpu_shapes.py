"""GPU parity of the basic shapes (crates/tessellation/src/basic_shapes.rs) and the path
builder's shapes (crates/path/src/builder.rs) against the oracle.

Rectangles are exact; circles match in topology exactly and in positions within `ATOL` of the
radius (their arc vertices come from f32 cos/sin, whose last bit differs between libms).
"""

import numpy as np
import pytest

from lyon_gb300 import tessellation as T
from lyon_gb300.options import FILL_OPTIONS_DTYPE, FillOptions, LineCap, LineJoin, StrokeOptions
from lyon_gb300.path import PathBuilder
from oracle import lyon_oracle as orc

pytestmark = pytest.mark.gpu

ATOL = 1e-5


@pytest.fixture(scope="module")
def gpu():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import gpu_helpers
    return gpu_helpers


def _batch(gpu, kind, params, tols, index_bits=32, index_mode=T.INDEX_GLOBAL, vertex_offset=0):
    import torch
    c = gpu.ctx()
    p = torch.tensor(np.asarray(params, np.float32).reshape(-1), device="cuda")
    o = np.zeros(len(tols), FILL_OPTIONS_DTYPE)
    o["tolerance"] = tols
    o["handle_intersections"] = 1
    od = T.upload_options(o, 0)
    res = T.fill_shapes(kind, p, len(params), od, len(tols), index_bits, index_mode,
                        vertex_offset, c)
    c.synchronize()
    v = res.vertices().cpu().numpy() if res.total_vertices else np.zeros((0, 2), np.float32)
    i = res.indices().cpu().numpy() if res.total_indices else np.zeros(0, np.int32)
    i = i.view(np.uint16) if index_bits == 16 else i.view(np.uint32)
    vo, io = res.offsets()
    return v, i, res.statuses().cpu().numpy(), vo.cpu().numpy(), io.cpu().numpy()


def test_rectangles_match_oracle_global_ids(gpu):
    rng = np.random.default_rng(61)
    lo = rng.uniform(-500, 500, size=(5000, 2)).astype(np.float32)
    rects = np.concatenate([lo, lo + rng.uniform(0, 100, size=(5000, 2)).astype(np.float32)], 1)
    v, i, st, vo, io = _batch(gpu, T.SHAPE_RECTANGLE, rects, [0.1], vertex_offset=7)
    assert (st == 0).all() and len(v) == 4 * len(rects) and len(i) == 6 * len(rects)
    # One BuffersBuilder appended shape after shape: ids continue from the vertex offset.
    out = orc.Output(32, 7)
    for r in rects:
        out.L.lyon_oracle_fill_rectangle(out.h, *[float(x) for x in r])
    ref = out.snapshot(0)
    assert np.array_equal(v, ref.vertices)
    assert np.array_equal(i, ref.indices)


def test_circles_match_oracle(gpu):
    # The lyon test's circle (radius 100 at the default tolerance: 64 vertices, 62 triangles)
    # and random ones, radii 0-500 (0 gives nothing), tolerances 0.001-1, u16 per shape.
    rng = np.random.default_rng(62)
    n = 3000
    circles = np.stack([rng.uniform(-1000, 1000, n), rng.uniform(-1000, 1000, n),
                        rng.uniform(-500, 500, n)], axis=1).astype(np.float32)
    circles[0] = (1.0, 2.0, 100.0)
    circles[1, 2] = 0.0
    tols = rng.choice(np.array([0.001, 0.01, 0.1, 1.0], np.float32), size=n)
    tols[0] = 0.1
    v, i, st, vo, io = _batch(gpu, T.SHAPE_CIRCLE, circles, tols, index_bits=16,
                              index_mode=T.INDEX_PER_PATH)
    assert int(vo[1] - vo[0]) == 64 and int(io[1] - io[0]) == 3 * 62
    assert int(vo[2] - vo[1]) == 0
    for k in range(n):
        ref = orc.fill_circle(circles[k, :2], circles[k, 2], tols[k], index_bits=16)
        assert int(st[k]) == ref.status, k
        if ref.status:
            continue
        gv = v[int(vo[k]):int(vo[k + 1])]
        gi = i[int(io[k]):int(io[k + 1])]
        assert np.array_equal(gi, ref.indices), k
        scale = max(1.0, float(np.abs(circles[k]).max()))
        assert np.allclose(gv, ref.vertices, rtol=0, atol=ATOL * scale), k


def test_single_shape_drop_ins(gpu):
    c = gpu.ctx()
    buffers = T.VertexBuffers(16)
    b = T.BuffersBuilder(buffers)
    fill = T.FillTessellator(c)
    fill.tessellate_rectangle((0.0, 1.0, 2.0, 4.0), FillOptions(), b)  # basic_shapes.rs test
    fill.tessellate_circle((1.0, 2.0), 100.0, FillOptions(), b)
    assert len(buffers.vertices) == 4 + 64 and len(buffers.indices) == 3 * (2 + 62)
    ref = orc.Output(16, 0)
    ref.L.lyon_oracle_fill_rectangle(ref.h, 0.0, 1.0, 2.0, 4.0)
    ref.L.lyon_oracle_fill_circle(ref.h, 1.0, 2.0, 100.0, 0.1)
    r = ref.snapshot(0)
    assert np.array_equal(buffers.indices, r.indices)
    assert np.allclose(buffers.vertices, r.vertices, rtol=0, atol=1e-3)


def test_builder_shapes_stroke_and_fill(gpu):
    # Rectangles, circles, rounded rectangles and polygons built as lyon's path builder builds
    # them, then stroked and filled through the batched entry points.
    b = PathBuilder()
    b.add_rectangle((0, 0, 10, 5), 1)
    b.add_rectangle((20, 0, 30, 5), -1)
    b.add_circle((50, 50), 20, 1)
    b.add_circle((100, 50), 7.5, -1)
    b.add_rounded_rectangle((0, 100, 60, 140), (5, 10, 0, 30), 1)
    b.add_rounded_rectangle((100, 100, 130, 120), (50, 50, 50, 50), -1)
    b.add_polygon([(200, 0), (230, 10), (215, 40)], True)
    path = b.build()
    from lyon_gb300.path import PathBatch
    batch = PathBatch.from_paths([path])
    for join in (LineJoin.Miter, LineJoin.Round):
        so = StrokeOptions(line_width=2.0, tolerance=0.05, line_join=join,
                           start_cap=LineCap.Butt, end_cap=LineCap.Butt)
        s = gpu.compare_per_path("stroke", batch, np.asarray(so.to_record()), index_bits=32)
        assert not s["mismatches"], s["mismatches"]
    fo = FillOptions(tolerance=0.05)
    s = gpu.compare_per_path("fill", batch, fo.to_record(), index_bits=32)
    assert not s["mismatches"], s["mismatches"]
