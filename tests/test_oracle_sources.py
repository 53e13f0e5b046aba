"""Vertex sources and interpolated custom attributes on the oracle (CPU).

lyon's own test `stroke_vertex_source_01` (crates/tessellation/src/stroke.rs:3039-3130) strokes
`begin(0,0) [1]; line_to(10,10) [2]; quadratic_bezier_to((10,20), (0,20)) [3]; close` with the
width read from attribute 0 and checks every vertex: at (0,0), (10,10) and (0,20) the source is
that endpoint and the interpolated attribute its value; in between the source is the curve
(from b to c, 0 < t < 1) and the attribute lies strictly between 2 and 3. The vertex records
carry positions, not positions on the path, so "at (0,0)" is checked as "within the stroke's
reach of (0,0)".
"""

import numpy as np

from oracle import lyon_oracle as orc
from lyon_gb300 import workloads
from lyon_gb300.options import StrokeOptions, STROKE_OPTIONS_DTYPE, LineJoin, LineCap
from lyon_gb300.path import Path, PathBatch, Verb

# Point layout of the test path: a = 0, b = 1, (ctrl = 2), c = 3, Close's repeated first point.
PATH = Path.from_arrays([Verb.BEGIN, Verb.LINE_TO, Verb.QUADRATIC_TO, Verb.CLOSE],
                        [[0, 0], [10, 10], [10, 20], [0, 20], [0, 0]])
ATTRS = np.array([[1.0], [2.0], [0.0], [3.0], [1.0]], np.float32)
A, B, C = 0, 1, 3


def _t(word):
    return float(np.array([word], np.uint32).view(np.float32)[0])


def check_vertex_source_01(vertices, sources, interpolated, reach):
    pts = PATH.points
    seen = set()
    for v, s, att in zip(vertices, sources, interpolated):
        frm, to, t = int(s[0]), int(s[1]), _t(s[2])
        if to == orc.NO_ENDPOINT:
            assert frm in (A, B, C), frm
            assert np.linalg.norm(v - pts[frm]) <= reach, (v, frm)
            assert att[0] == ATTRS[frm, 0], (att, frm)
            seen.add(frm)
        else:
            assert (frm, to) == (B, C), (frm, to)
            assert 0.0 < t < 1.0
            assert 2.0 < att[0] < 3.0, att
            seen.add("edge")
    assert seen == {A, B, C, "edge"}


def test_stroke_vertex_source_01_variable_width():
    opts = StrokeOptions()
    r = orc.stroke(PATH, opts, 32, widths=ATTRS[:, 0], sources=True)
    assert r.status == 0
    att = orc.interpolate_attributes(r.sources, ATTRS)
    # Half width at most 1.5, miter limit 4.
    check_vertex_source_01(r.vertices, r.sources, att, 4 * 1.5 + 1e-3)


def test_stroke_vertex_source_01_fixed_width():
    r = orc.stroke(PATH, StrokeOptions(), 32, sources=True)
    assert r.status == 0
    att = orc.interpolate_attributes(r.sources, ATTRS)
    check_vertex_source_01(r.vertices, r.sources, att, 4 * 0.5 + 1e-3)


def test_sources_do_not_change_geometry():
    # Recording sources is read-only: positions and indices equal the plain stroke's.
    batch, _ = workloads.batched_stroke(300, seed=5)
    o = np.zeros(1, STROKE_OPTIONS_DTYPE)
    o[0] = (LineCap.Round, LineCap.Square, LineJoin.Round, 3.0, 4.0, 0.05)
    plain = orc.batch("stroke", batch, o, 32, 4)
    src = orc.batch_stroke_sources(batch, o, 32, 4)
    assert np.array_equal(plain["vtx_counts"], src["vtx_counts"])
    assert np.array_equal(plain["vertices"], src["vertices"])
    assert np.array_equal(plain["indices"], src["indices"])


def test_sources_point_at_their_endpoints():
    # Every endpoint source names an endpoint of its own path, every edge source a curve's
    # two endpoints; t in (0, 1).
    batch, _ = workloads.batched_stroke(300, seed=6)
    o = np.zeros(1, STROKE_OPTIONS_DTYPE)
    o[0] = (LineCap.Butt, LineCap.Round, LineJoin.MiterClip, 2.0, 2.0, 0.1)
    res = orc.batch_stroke_sources(batch, o, 32, 4)
    vo = res["vtx_offsets"]
    for p in range(batch.num_paths):
        s = res["sources"][vo[p]:vo[p + 1]]
        lo, hi = int(batch.point_offsets[p]), int(batch.point_offsets[p + 1])
        assert np.all((s[:, 0] >= lo) & (s[:, 0] < hi))
        edge = s[:, 1] != orc.NO_ENDPOINT
        assert np.all((s[edge, 1] > s[edge, 0]) & (s[edge, 1] < hi))
        t = s[edge, 2].view(np.float32)
        assert np.all((t > 0) & (t < 1))


def test_interpolate_attributes_arithmetic():
    attrs = np.array([[1.0, -2.0], [3.0, 5.0], [0.5, 0.25]], np.float32)
    t = np.float32(0.3)
    src = np.array([[0, orc.NO_ENDPOINT, 0], [0, 1, t.view(np.uint32)],
                    [2, 1, np.float32(0.75).view(np.uint32)]], np.uint32)
    out = orc.interpolate_attributes(src, attrs)
    assert np.array_equal(out[0], attrs[0])
    one = np.float32(1.0)
    exp = attrs[0] * (one - t) + attrs[1] * t
    assert np.array_equal(out[1], exp.astype(np.float32))
    assert np.allclose(out[2], attrs[2] * 0.25 + attrs[1] * 0.75)


def test_threaded_interpolation_matches():
    batch, _ = workloads.batched_stroke(200, seed=7)
    o = np.zeros(1, STROKE_OPTIONS_DTYPE)
    o[0] = (LineCap.Round, LineCap.Round, LineJoin.Round, 2.0, 4.0, 0.1)
    res = orc.batch_stroke_sources(batch, o, 32, 4)
    attrs = np.random.default_rng(8).normal(size=(len(batch.points), 3)).astype(np.float32)
    a = orc.interpolate_attributes(res["sources"], attrs)
    b = orc.interpolate_attributes_threads(res["sources"], attrs, 4)
    assert np.array_equal(a, b)


# ---- fill: FillVertex::sources / interpolated_attributes (crates/tessellation/src/fill.rs) ----

from lyon_gb300.options import FillOptions  # noqa: E402

FILL_01 = (Path.from_arrays([Verb.BEGIN, Verb.LINE_TO, Verb.LINE_TO, Verb.CLOSE],
                            [[0, 0], [1, 1], [0, 2], [0, 0]]),
           np.array([[1, 0, 0], [0, 1, 0], [0, 0, 1], [9, 9, 9]], np.float32))
# Two closed squares crossing each other; ids a..d = 0..3, e..h = 5..8 (4 and 9 are the Close
# points).
FILL_02 = (Path.from_arrays([Verb.BEGIN, Verb.LINE_TO, Verb.LINE_TO, Verb.LINE_TO, Verb.CLOSE] * 2,
                            [[1, 0], [2, 0], [2, 4], [1, 4], [1, 0],
                             [0, 1], [0, 3], [3, 3], [3, 1], [0, 1]]),
           np.array([[1, 0, 1], [2, 0, 1], [3, 0, 1], [4, 0, 1], [9, 9, 9],
                     [0, 1, 2], [0, 2, 2], [0, 3, 2], [0, 4, 2], [9, 9, 9]], np.float32))
# Two triangles meeting at (1, 1): ids 0-2 and 4-6.
FILL_03 = (Path.from_arrays([Verb.BEGIN, Verb.LINE_TO, Verb.LINE_TO, Verb.CLOSE] * 2,
                            [[0, 0], [2, 0], [1, 1], [0, 0], [0, 2], [2, 2], [1, 1], [0, 2]]),
           np.array([[0], [0], [1], [9], [0], [0], [2], [9]], np.float32))


def _fill_sources(path, attrs):
    r = orc.fill(path, FillOptions(), 32, sources=True)
    assert r.status == 0
    att = orc.interpolate_fill_attributes(r.sources, r.source_counts, attrs)
    starts = np.concatenate([[0], np.cumsum(r.source_counts)]).astype(np.int64)
    per_vertex = [r.sources[starts[v]:starts[v + 1]] for v in range(len(r.vertices))]
    return r, per_vertex, att


def _on_edge(s, frm, to, d):
    t = _t(s[2])
    return (int(s[0]), int(s[1])) == (frm, to) and (abs(d - t) < 1e-5 or abs(1 - d - t) <= 1e-5)


def check_fill_vertex_source_01(vertices, per_vertex, att):
    # fill.rs:2680-2748
    expect = {(0.0, 0.0): 0, (1.0, 1.0): 1, (0.0, 2.0): 2}
    for v, srcs, a in zip(vertices, per_vertex, att):
        e = expect[(float(v[0]), float(v[1]))]
        for s in srcs:
            assert int(s[1]) == orc.NO_ENDPOINT and int(s[0]) == e
        assert np.array_equal(a, np.eye(3, dtype=np.float32)[e])


def check_fill_vertex_source_02(vertices, per_vertex, att):
    # fill.rs:2750-2905
    a, b, c, d, e, f, g, h = 0, 1, 2, 3, 5, 6, 7, 8
    ends = {(1, 0): a, (2, 0): b, (2, 4): c, (1, 4): d, (0, 1): e, (0, 3): f, (3, 3): g,
            (3, 1): h}
    edges = {(1, 1): [(h, e, 2 / 3), (d, a, 3 / 4)], (2, 1): [(h, e, 1 / 3), (b, c, 1 / 4)],
             (1, 3): [(f, g, 1 / 3), (d, a, 1 / 4)], (2, 3): [(f, g, 2 / 3), (b, c, 3 / 4)]}
    attrs = {(1, 0): [1, 0, 1], (2, 0): [2, 0, 1], (2, 4): [3, 0, 1], (1, 4): [4, 0, 1],
             (0, 1): [0, 1, 2], (0, 3): [0, 2, 2], (3, 3): [0, 3, 2], (3, 1): [0, 4, 2],
             (1, 1): [0.875, 1.0, 1.5], (2, 1): [1.125, 1.5, 1.5],
             (1, 3): [1.625, 1.16666, 1.5], (2, 3): [1.375, 1.33333, 1.5]}
    for v, srcs, at in zip(vertices, per_vertex, att):
        key = (int(round(float(v[0]))), int(round(float(v[1]))))
        assert np.allclose(v, key, atol=1e-5)
        for s in srcs:
            if key in ends:
                assert int(s[1]) == orc.NO_ENDPOINT and int(s[0]) == ends[key]
            else:
                assert any(_on_edge(s, *cand) for cand in edges[key]), (key, s)
        assert np.all(np.abs(at - np.array(attrs[key], np.float32)) < 1e-3), (key, at)


def check_fill_vertex_source_03(vertices, per_vertex, att):
    # fill.rs:2907-2981
    for v, srcs, a in zip(vertices, per_vertex, att):
        if np.allclose(v, (1.0, 1.0)):
            assert np.array_equal(a, [1.5]) and len(srcs) == 2
        else:
            assert np.array_equal(a, [0.0]) and len(srcs) == 1


def test_fill_vertex_source_01():
    path, attrs = FILL_01
    r, per_vertex, att = _fill_sources(path, attrs)
    check_fill_vertex_source_01(r.vertices, per_vertex, att)


def test_fill_vertex_source_02():
    path, attrs = FILL_02
    r, per_vertex, att = _fill_sources(path, attrs)
    assert len(r.vertices) == 12
    check_fill_vertex_source_02(r.vertices, per_vertex, att)


def test_fill_vertex_source_03():
    path, attrs = FILL_03
    r, per_vertex, att = _fill_sources(path, attrs)
    check_fill_vertex_source_03(r.vertices, per_vertex, att)


def test_fill_sources_batch_and_c_interpolation():
    # The batched oracle equals per-path calls (ids shifted to the batch), and the C
    # interpolation equals the numpy one bit for bit.
    batch, opts = workloads.glyph_fill(300, seed=9)
    res = orc.batch_fill_sources(batch, opts, 32, 4)
    for p in range(0, batch.num_paths, 37):
        r = orc.fill(batch.path(p), FillOptions(
            tolerance=float(opts[p if len(opts) > 1 else 0]["tolerance"]),
            fill_rule=int(opts[p if len(opts) > 1 else 0]["fill_rule"])), 32, sources=True)
        s0, s1 = int(res["src_offsets"][p]), int(res["src_offsets"][p + 1])
        got = res["sources"][s0:s1].copy()
        base = int(batch.point_offsets[p])
        got[:, 0] -= base
        edge = got[:, 1] != orc.NO_ENDPOINT
        got[edge, 1] -= base
        assert np.array_equal(got, r.sources)
    attrs = np.random.default_rng(10).normal(size=(len(batch.points), 2)).astype(np.float32)
    a = orc.interpolate_fill_attributes(res["sources"], res["source_counts"], attrs)
    b = orc.interpolate_fill_attributes_c(res["sources"], res["source_counts"], attrs)
    assert np.array_equal(a, b)
