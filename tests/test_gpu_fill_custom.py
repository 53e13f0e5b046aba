"""GPU parity of the custom-attribute fill output against the oracle: every vertex's sources
(FillVertex::sources, crates/tessellation/src/fill.rs:2172-2178, 2294-2337) and its interpolated
attributes (FillVertex::interpolated_attributes, :2208-2286), through
lyon_gpu_fill_paths_custom / lyon_gpu_fill_path_custom.

The fill is bit-exact, so everything is compared exactly: per path status, vertices, indices,
per-vertex source counts and the sources themselves; the interpolated attributes bit for bit
against the oracle's interpolation of the same sources. lyon's own fill_vertex_source_01/02/03
run through the single-path drop-in.
"""

import numpy as np
import pytest

from lyon_gb300 import workloads
from lyon_gb300 import tessellation as T
from lyon_gb300.options import FILL_OPTIONS_DTYPE, FillOptions, FillRule
from oracle import lyon_oracle as orc

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gpu():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import gpu_helpers
    return gpu_helpers


def _gpu_fill_custom(gpu, batch, opts, attrs, index_bits=32):
    import torch
    c = gpu.ctx()
    db = T.DeviceBatch.upload(batch, 0)
    od = T.upload_options(opts, 0)
    a = torch.from_numpy(np.ascontiguousarray(attrs, np.float32)).cuda()
    res = T.tessellate_paths("fill", db, od, len(opts), index_bits=index_bits,
                             index_mode=T.INDEX_PER_PATH, ctx=c, custom_attributes=a)
    c.synchronize()
    nv = res.total_vertices
    v = res.vertices().cpu().numpy() if nv else np.zeros((0, 2), np.float32)
    i = res.indices().cpu().numpy() if res.total_indices else np.zeros(0, np.int32)
    i = i.view(np.uint16) if index_bits == 16 else i.view(np.uint32)
    src = (res.sources().cpu().numpy().view(np.uint32) if res.total_sources
           else np.zeros((0, 3), np.uint32))
    soff = res.source_offsets().cpu().numpy().astype(np.int64)
    att = (res.custom_attributes().cpu().numpy() if nv and attrs.shape[1]
           else np.zeros((nv, attrs.shape[1]), np.float32))
    vo, io = res.offsets()
    return dict(vertices=v, indices=i, sources=src, source_offsets=soff, attributes=att,
                status=res.statuses().cpu().numpy(), vtx_offsets=vo.cpu().numpy(),
                idx_offsets=io.cpu().numpy())


def compare_fill_custom(gpu, batch, opts, attrs, index_bits=32):
    g = _gpu_fill_custom(gpu, batch, opts, attrs, index_bits)
    r = orc.batch_fill_sources(batch, opts, index_bits, 8)
    counts = np.diff(g["source_offsets"])
    if len(counts):
        want = orc.interpolate_fill_attributes(g["sources"], counts, attrs)
        assert np.array_equal(g["attributes"], want, equal_nan=True)
    assert g["source_offsets"][-1] == len(g["sources"])
    bad = []
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
        if (g1 - g0 != o1 - o0 or not np.array_equal(g["vertices"][g0:g1], r["vertices"][o0:o1])
                or not np.array_equal(g["indices"][gi0:gi1].astype(np.uint64), oi)):
            bad.append((p, "geometry"))
            continue
        if not np.array_equal(counts[g0:g1], r["source_counts"][o0:o1]):
            bad.append((p, "source counts"))
            continue
        s0, s1 = int(g["source_offsets"][g0]), int(g["source_offsets"][g1])
        r0, r1 = int(r["src_offsets"][p]), int(r["src_offsets"][p + 1])
        if not np.array_equal(g["sources"][s0:s1], r["sources"][r0:r1]):
            bad.append((p, "sources"))
    return bad, g


def _glyph_options(n, rule):
    o = np.zeros(n, FILL_OPTIONS_DTYPE)
    o["tolerance"] = 0.1
    o["fill_rule"] = rule
    o["handle_intersections"] = 1
    return o


@pytest.mark.parametrize("rule", [FillRule.NonZero, FillRule.EvenOdd])
def test_fill_custom_glyphs(gpu, rule):
    # Glyph-like paths with quadratic contours and 10 % self-intersecting stars (intersection
    # events carry their edges' sources), three attributes.
    batch, _ = workloads.glyph_fill(3000, seed=111, fill_rule=rule)
    opts = _glyph_options(batch.num_paths, rule)
    attrs = np.random.default_rng(112).normal(size=(len(batch.points), 3)).astype(np.float32)
    bad, g = compare_fill_custom(gpu, batch, opts, attrs)
    print(f"paths={batch.num_paths} sources={len(g['sources'])} bad={len(bad)}")
    assert not bad, bad[:10]


def test_fill_custom_u16_no_attributes(gpu):
    batch, _ = workloads.glyph_fill(800, seed=113)
    opts = _glyph_options(batch.num_paths, FillRule.NonZero)
    opts["tolerance"] = 0.5
    bad, _ = compare_fill_custom(gpu, batch, opts, np.zeros((len(batch.points), 0), np.float32),
                                 index_bits=16)
    assert not bad, bad[:10]


def test_fill_custom_matches_plain_fill(gpu):
    # Recording sources leaves the geometry alone.
    batch, _ = workloads.glyph_fill(1000, seed=114)
    opts = _glyph_options(batch.num_paths, FillRule.EvenOdd)
    g = _gpu_fill_custom(gpu, batch, opts, np.zeros((len(batch.points), 1), np.float32))
    f = gpu.gpu_batch("fill", batch, opts, index_bits=32, index_mode=T.INDEX_PER_PATH)
    assert np.array_equal(g["status"], f["status"])
    assert np.array_equal(g["vertices"], f["vertices"])
    assert np.array_equal(g["indices"], f["indices"])


def _single(gpu, path, attrs):
    buffers = T.VertexBuffers(32)
    builder = T.BuffersBuilder(buffers, vertex_ctor=lambda v: v)
    T.FillTessellator(gpu.ctx()).tessellate_path(path, FillOptions(), builder, attributes=attrs)
    v = buffers.vertices
    per_vertex = [builder.sources[int(f):int(f) + int(c)]
                  for f, c in zip(v["src_first"], v["src_count"])]
    ref = orc.fill(path, FillOptions(), 32, sources=True)
    assert np.array_equal(buffers.indices, ref.indices)
    assert np.array_equal(np.stack([v["x"], v["y"]], axis=1), ref.vertices)
    assert np.array_equal(builder.sources, ref.sources)
    return np.stack([v["x"], v["y"]], axis=1), per_vertex, v["attributes"]


def test_fill_vertex_source_kats_single_path(gpu):
    import test_oracle_sources as K
    verts, per_vertex, att = _single(gpu, *K.FILL_01)
    K.check_fill_vertex_source_01(verts, per_vertex, att)
    verts, per_vertex, att = _single(gpu, *K.FILL_02)
    assert len(verts) == 12
    K.check_fill_vertex_source_02(verts, per_vertex, att)
    verts, per_vertex, att = _single(gpu, *K.FILL_03)
    K.check_fill_vertex_source_03(verts, per_vertex, att)


def test_interpolate_fill_attributes_standalone(gpu):
    import torch
    c = gpu.ctx()
    rng = np.random.default_rng(115)
    attrs = rng.normal(size=(40, 2)).astype(np.float32)
    n = 3000
    counts = rng.integers(0, 4, size=n)
    offs = np.zeros(n + 1, np.int64)
    offs[1:] = np.cumsum(counts)
    ns = int(offs[-1])
    src = np.zeros((ns, 3), np.uint32)
    src[:, 0] = rng.integers(0, 41, size=ns)  # id 40 is out of range
    edge = rng.random(ns) < 0.5
    src[:, 1] = np.where(edge, rng.integers(0, 40, size=ns), orc.NO_ENDPOINT)
    src[:, 2] = rng.random(ns).astype(np.float32).view(np.uint32)
    d_src = torch.from_numpy(src.view(np.int32)).cuda()
    d_off = torch.from_numpy(offs).cuda()
    d_att = torch.from_numpy(attrs).cuda()
    d_out = torch.empty((n, 2), dtype=torch.float32, device="cuda")
    r = c.lib.lyon_gpu_interpolate_fill_attributes(c.h, d_src.data_ptr(), d_off.data_ptr(), n,
                                                   d_att.data_ptr(), 2, 40, d_out.data_ptr())
    assert r == 0
    c.synchronize()
    out = d_out.cpu().numpy()
    bad_v = np.zeros(n, bool)
    for v in range(n):
        s = src[offs[v]:offs[v + 1]]
        bad_v[v] = counts[v] == 0 or np.any(s[:, 0] >= 40)
    assert np.all(np.isnan(out[bad_v]))
    good = ~bad_v
    starts = offs[:-1][good]
    sel = np.concatenate([np.arange(a, a + k) for a, k in zip(starts, counts[good])])
    want = orc.interpolate_fill_attributes(src[sel], counts[good], attrs)
    assert np.array_equal(out[good], want)
