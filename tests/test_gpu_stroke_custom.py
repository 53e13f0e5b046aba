"""GPU parity of the custom-attribute stroke output against the oracle: every vertex's
VertexSource (StrokeVertex::source, crates/tessellation/src/stroke.rs:2719-2722) and its
interpolated attributes (StrokeVertex::interpolated_attributes, :2728-2747), for fixed and
variable line widths, through lyon_gpu_stroke_paths_custom / lyon_gpu_stroke_path_custom.

Per path: status, counts and index topology exactly; sources exactly (ids, and t bit for bit);
interpolated attributes bit for bit against the oracle's interpolation of the GPU's own sources;
positions within 1e-5 of the path's scale (NaN where lyon's variable-width stepper makes NaN).
The fixed-width sequential stepper must also reproduce the warp-per-path kernel's positions and
indices exactly.
"""

import numpy as np
import pytest

from lyon_gb300 import workloads
from lyon_gb300 import tessellation as T
from lyon_gb300.options import STROKE_OPTIONS_DTYPE, LineCap, LineJoin, StrokeOptions
from lyon_gb300.path import Path, Verb
from oracle import lyon_oracle as orc

pytestmark = pytest.mark.gpu

RTOL = 1e-5


@pytest.fixture(scope="module")
def gpu():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import gpu_helpers
    return gpu_helpers


def _options(n, seed):
    rng = np.random.default_rng(seed)
    o = np.zeros(n, dtype=STROKE_OPTIONS_DTYPE)
    o["line_join"] = rng.choice([LineJoin.Miter, LineJoin.MiterClip, LineJoin.Round,
                                 LineJoin.Bevel], size=n)
    caps = rng.choice([LineCap.Butt, LineCap.Square, LineCap.Round], size=(n, 2))
    o["start_cap"] = caps[:, 0]
    o["end_cap"] = caps[:, 1]
    o["line_width"] = rng.uniform(0.5, 8.0, size=n).astype(np.float32)
    o["miter_limit"] = rng.choice(np.array([1.0, 4.0, 10.0], np.float32), size=n)
    o["tolerance"] = rng.choice(np.array([0.01, 0.1, 1.0], np.float32), size=n)
    return o


def _gpu_custom(gpu, batch, opts, attrs, width_attribute=-1, index_bits=32, records=False):
    import torch
    c = gpu.ctx()
    db = T.DeviceBatch.upload(batch, 0)
    od = T.upload_options(opts, 0)
    a = torch.from_numpy(np.ascontiguousarray(attrs, np.float32)).cuda()
    res = T.tessellate_paths("stroke", db, od, len(opts), index_bits=index_bits,
                             index_mode=T.INDEX_PER_PATH, ctx=c, attributes=records,
                             custom_attributes=a, width_attribute=width_attribute)
    c.synchronize()
    nv = res.total_vertices
    if records:
        rec = (res.records().cpu().numpy().view(T.STROKE_VERTEX_DTYPE).reshape(-1)
               if nv else np.zeros(0, T.STROKE_VERTEX_DTYPE))
        v = np.stack([rec["x"], rec["y"]], axis=1) if nv else np.zeros((0, 2), np.float32)
    else:
        rec = None
        v = res.vertices().cpu().numpy() if nv else np.zeros((0, 2), np.float32)
    i = res.indices().cpu().numpy() if res.total_indices else np.zeros(0, np.int32)
    i = i.view(np.uint16) if index_bits == 16 else i.view(np.uint32)
    src = res.sources().cpu().numpy().view(np.uint32) if nv else np.zeros((0, 3), np.uint32)
    att = (res.custom_attributes().cpu().numpy() if nv and attrs.shape[1]
           else np.zeros((nv, attrs.shape[1]), np.float32))
    vo, io = res.offsets()
    return dict(vertices=v, records=rec, indices=i, sources=src, attributes=att,
                status=res.statuses().cpu().numpy(), vtx_offsets=vo.cpu().numpy(),
                idx_offsets=io.cpu().numpy())


def compare_custom(gpu, batch, opts, attrs, width_attribute=-1, index_bits=32, records=False):
    g = _gpu_custom(gpu, batch, opts, attrs, width_attribute, index_bits, records)
    widths = attrs[:, width_attribute] if width_attribute >= 0 else None
    r = orc.batch_stroke_sources(batch, opts, index_bits, 8, widths=widths,
                                 want_attributes=records)
    # The interpolation kernel against the oracle's, on the GPU's own sources: bit for bit.
    if len(g["sources"]):
        want = orc.interpolate_attributes(g["sources"], attrs)
        assert np.array_equal(g["attributes"], want, equal_nan=True)
    bad, exact = [], 0
    for p in range(batch.num_paths):
        if int(g["status"][p]) != int(r["status"][p]):
            bad.append((p, "status", int(g["status"][p]), int(r["status"][p])))
            continue
        if g["status"][p] != 0:
            continue
        g0, g1 = int(g["vtx_offsets"][p]), int(g["vtx_offsets"][p + 1])
        o0, o1 = int(r["vtx_offsets"][p]), int(r["vtx_offsets"][p + 1])
        gi0, gi1 = int(g["idx_offsets"][p]), int(g["idx_offsets"][p + 1])
        oi0, oi1 = int(r["idx_offsets"][p]), int(r["idx_offsets"][p + 1])
        oi = r["indices"][oi0:oi1].astype(np.uint64)
        if index_bits == 16:
            oi = oi & 0xFFFF
        if g1 - g0 != o1 - o0 or not np.array_equal(g["indices"][gi0:gi1].astype(np.uint64), oi):
            bad.append((p, "topology"))
            continue
        if not np.array_equal(g["sources"][g0:g1], r["sources"][o0:o1]):
            bad.append((p, "sources"))
            continue
        gv, ov = g["vertices"][g0:g1], r["vertices"][o0:o1]
        if np.array_equal(gv, ov, equal_nan=True):
            exact += 1
        else:
            pts = batch.points[batch.point_offsets[p]:batch.point_offsets[p + 1]]
            wmax = 1.0
            if widths is not None:
                wmax = max(1.0, float(np.max(widths[batch.point_offsets[p]:
                                                    batch.point_offsets[p + 1]])))
            lw = float(opts[p if len(opts) > 1 else 0]["line_width"]) * wmax
            scale = max(1.0, float(np.abs(pts).max()) if len(pts) else 1.0) + lw
            if not np.allclose(gv, ov, rtol=0, atol=RTOL * scale, equal_nan=True):
                bad.append((p, "positions"))
                continue
        if records:
            gr = g["records"][g0:g1]
            oa = r["attributes"][o0:o1]
            if not np.array_equal(gr["side"], oa[:, 3]):
                bad.append((p, "side"))
    return bad, exact, g


def test_custom_fixed_width_curves(gpu):
    # Lines, quadratics (with sharp-turn splits), cubics, every join and cap, three attributes.
    batch, _ = workloads.batched_stroke(1500, seed=91)
    opts = _options(batch.num_paths, 92)
    attrs = np.random.default_rng(93).normal(size=(len(batch.points), 3)).astype(np.float32)
    bad, exact, g = compare_custom(gpu, batch, opts, attrs)
    print(f"paths={batch.num_paths} exact={exact} bad={len(bad)}")
    assert len(bad) <= max(2, batch.num_paths // 500), bad[:10]


def test_custom_fixed_width_matches_warp_kernel(gpu):
    # The sequential stepper and the warp-per-path kernel are two restatements of lyon's
    # fixed-width stroker: identical positions and indices, path by path.
    batch, _ = workloads.batched_stroke(1000, seed=94)
    opts = _options(batch.num_paths, 95)
    attrs = np.zeros((len(batch.points), 0), np.float32)
    g = _gpu_custom(gpu, batch, opts, attrs)
    f = gpu.gpu_batch("stroke", batch, opts, index_bits=32, index_mode=T.INDEX_PER_PATH)
    assert np.array_equal(g["status"], f["status"])
    assert np.array_equal(g["vtx_offsets"], f["vtx_offsets"])
    assert np.array_equal(g["indices"], f["indices"])
    assert np.array_equal(g["vertices"], f["vertices"])


def test_custom_variable_width_records_u16(gpu):
    batch, _ = workloads.batched_stroke(1200, seed=96)
    opts = _options(batch.num_paths, 97)
    rng = np.random.default_rng(98)
    attrs = np.stack([rng.normal(size=len(batch.points)),
                      rng.uniform(0.2, 3.0, size=len(batch.points))], axis=1).astype(np.float32)
    bad, exact, _ = compare_custom(gpu, batch, opts, attrs, width_attribute=1, index_bits=16,
                                   records=True)
    print(f"paths={batch.num_paths} exact={exact} bad={len(bad)}")
    assert len(bad) <= max(2, batch.num_paths // 500), bad[:10]


def test_custom_polylines(gpu):
    poly, popts = workloads.map_polylines(3000, seed=99, max_len=300)
    attrs = np.random.default_rng(100).uniform(-5, 5, size=(len(poly.points), 4)).astype(
        np.float32)
    bad, exact, _ = compare_custom(gpu, poly, popts, attrs)
    assert len(bad) <= max(2, poly.num_paths // 500), bad[:10]


def test_stroke_vertex_source_01_single_path(gpu):
    # lyon's stroke_vertex_source_01 (stroke.rs:3039-3130) through the single-path drop-in with
    # a vertex constructor, the width read from attribute 0.
    path = Path.from_arrays([Verb.BEGIN, Verb.LINE_TO, Verb.QUADRATIC_TO, Verb.CLOSE],
                            [[0, 0], [10, 10], [10, 20], [0, 20], [0, 0]])
    attrs = np.array([[1.0], [2.0], [0.0], [3.0], [1.0]], np.float32)
    opts = StrokeOptions().with_variable_line_width(0)
    buffers = T.VertexBuffers(32)
    builder = T.BuffersBuilder(buffers, vertex_ctor=lambda v: v)
    T.StrokeTessellator(gpu.ctx()).tessellate_path(path, opts, builder, attributes=attrs)
    ref = orc.stroke(path, opts, 32, widths=attrs[:, 0], sources=True)
    v = buffers.vertices
    assert np.array_equal(buffers.indices, ref.indices)
    assert np.allclose(np.stack([v["x"], v["y"]], axis=1), ref.vertices, rtol=0, atol=1e-4)
    src = np.stack([v["src_from"], v["src_to"], v["src_t"].view(np.uint32)], axis=1)
    assert np.array_equal(src, ref.sources)
    from test_oracle_sources import check_vertex_source_01
    check_vertex_source_01(np.stack([v["x"], v["y"]], axis=1), src, v["attributes"],
                           4 * 1.5 + 1e-3)


def test_custom_single_path_positions_only_and_errors(gpu):
    path = Path.from_arrays([Verb.BEGIN, Verb.CUBIC_TO, Verb.END],
                            [[0, 0], [10, 30], [20, -30], [30, 0]])
    attrs = np.array([[1.0, 0.0], [9.0, 9.0], [9.0, 9.0], [3.0, 1.0]], np.float32)
    buffers = T.VertexBuffers(16)
    T.StrokeTessellator(gpu.ctx()).tessellate_path(path, StrokeOptions(line_width=2.0),
                                                   T.BuffersBuilder(buffers), attributes=attrs)
    ref = orc.stroke(path, StrokeOptions(line_width=2.0), 16)
    assert np.array_equal(buffers.indices, ref.indices)
    assert np.array_equal(buffers.vertices, ref.vertices)
    with pytest.raises(ValueError):
        T.StrokeTessellator(gpu.ctx()).tessellate_path(
            path, StrokeOptions().with_variable_line_width(0), T.BuffersBuilder(buffers))
    with pytest.raises(T.TessellationError):
        T.StrokeTessellator(gpu.ctx()).tessellate_path(
            path, StrokeOptions().with_variable_line_width(2), T.BuffersBuilder(buffers),
            attributes=attrs)


def test_interpolate_attributes_standalone(gpu):
    import torch
    c = gpu.ctx()
    attrs = np.random.default_rng(101).normal(size=(50, 3)).astype(np.float32)
    rng = np.random.default_rng(102)
    n = 4000
    src = np.zeros((n, 3), np.uint32)
    src[:, 0] = rng.integers(0, 52, size=n)  # a few ids out of range
    edge = rng.random(n) < 0.6
    src[:, 1] = np.where(edge, rng.integers(0, 50, size=n), orc.NO_ENDPOINT)
    src[:, 2] = rng.random(n).astype(np.float32).view(np.uint32)
    d_src = torch.from_numpy(src.view(np.int32)).cuda()
    d_att = torch.from_numpy(attrs).cuda()
    d_out = torch.empty((n, 3), dtype=torch.float32, device="cuda")
    r = c.lib.lyon_gpu_interpolate_attributes(c.h, d_src.data_ptr(), n, d_att.data_ptr(), 3, 50,
                                              d_out.data_ptr())
    assert r == 0
    c.synchronize()
    out = d_out.cpu().numpy()
    bad = src[:, 0] >= 50
    assert np.all(np.isnan(out[bad]))
    want = orc.interpolate_attributes(src[~bad], attrs)
    assert np.array_equal(out[~bad], want)


def test_path_buffer_with_attributes_feeds_the_custom_stroke(gpu):
    # PathBuffer (crates/path/src/path_buffer.rs) as the batched container: its batch and its
    # attribute table go to lyon_gpu_stroke_paths_custom unchanged.
    from lyon_gb300.path_buffer import PathBuffer
    buf = PathBuffer()
    rng = np.random.default_rng(141)
    for i in range(200):
        b = buf.builder().with_attributes(2)
        b.begin(rng.uniform(0, 100, 2), rng.uniform(0.5, 2, 2))
        for _ in range(int(rng.integers(1, 6))):
            if rng.random() < 0.5:
                b.line_to(rng.uniform(0, 100, 2), rng.uniform(0.5, 2, 2))
            else:
                b.quadratic_bezier_to(rng.uniform(0, 100, 2), rng.uniform(0, 100, 2),
                                      rng.uniform(0.5, 2, 2))
        b.end(bool(i % 2))
        b.build()
    batch = buf.as_batch()
    attrs = buf.attribute_table()
    opts = _options(batch.num_paths, 142)
    bad, exact, _ = compare_custom(gpu, batch, opts, attrs, width_attribute=1)
    assert len(bad) <= 1, bad
