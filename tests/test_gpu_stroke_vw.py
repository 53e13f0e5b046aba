"""GPU parity of the variable-line-width stroke (StrokeOptions::variable_line_width,
crates/tessellation/src/stroke.rs:646-767, 954-1067, 1380-1512) against the oracle.

Per path: status, vertex and index counts and the index topology exactly; positions within
`RTOL` of the path's scale (the attachment angles are evaluated in f64 with one rounding on both
sides, so they agree bit for bit in practice). lyon's variable-width stepper can produce NaN
positions (a join after a skipped flattening step reads side points that were never set); those
must be NaN on both sides.
"""

import json
import os

import numpy as np
import pytest

from lyon_gb300 import workloads
from lyon_gb300 import tessellation as T
from lyon_gb300.options import STROKE_OPTIONS_DTYPE, LineCap, LineJoin
from lyon_gb300.path import Path, PathBatch, Verb
from oracle import lyon_oracle as orc

from lyon_cases import GOLDEN, case_path, stroke_options_from_case

pytestmark = pytest.mark.gpu

RTOL = 1e-5


@pytest.fixture(scope="module")
def gpu():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import gpu_helpers
    return gpu_helpers


def _gpu_vw(gpu, batch, opts, widths, index_bits=32, attributes=False):
    import torch
    c = gpu.ctx()
    db = T.DeviceBatch.upload(batch, 0)
    od = T.upload_options(opts, 0)
    w = torch.from_numpy(np.ascontiguousarray(widths, np.float32)).cuda()
    res = T.tessellate_paths("stroke", db, od, len(opts), index_bits=index_bits,
                             index_mode=T.INDEX_PER_PATH, ctx=c, attributes=attributes, widths=w)
    c.synchronize()
    if attributes:
        rec = (res.records().cpu().numpy().view(T.STROKE_VERTEX_DTYPE).reshape(-1)
               if res.total_vertices else np.zeros(0, T.STROKE_VERTEX_DTYPE))
        v = np.stack([rec["x"], rec["y"]], axis=1)
    else:
        rec = None
        v = res.vertices().cpu().numpy() if res.total_vertices else np.zeros((0, 2), np.float32)
    i = res.indices().cpu().numpy() if res.total_indices else np.zeros(0, np.int32)
    i = i.view(np.uint16) if index_bits == 16 else i.view(np.uint32)
    vo, io = res.offsets()
    return dict(vertices=v, records=rec, indices=i, status=res.statuses().cpu().numpy(),
                vtx_offsets=vo.cpu().numpy(), idx_offsets=io.cpu().numpy())


def compare_vw(gpu, batch, opts, widths, index_bits=32, attributes=False):
    g = _gpu_vw(gpu, batch, opts, widths, index_bits, attributes)
    r = orc.batch("stroke", batch, opts, index_bits, 8, want_attributes=attributes,
                  widths=widths)
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
        gv, ov = g["vertices"][g0:g1], r["vertices"][o0:o1]
        if np.array_equal(gv, ov, equal_nan=True):
            exact += 1
        else:
            pts = batch.points[batch.point_offsets[p]:batch.point_offsets[p + 1]]
            wmax = float(np.max(widths[batch.point_offsets[p]:batch.point_offsets[p + 1]]))
            lw = float(opts[p if len(opts) > 1 else 0]["line_width"]) * max(1.0, wmax)
            scale = max(1.0, float(np.abs(pts).max()) if len(pts) else 1.0) + lw
            if not np.allclose(gv, ov, rtol=0, atol=RTOL * scale, equal_nan=True):
                bad.append((p, "positions"))
                continue
        if attributes:
            gr = g["records"][g0:g1]
            oa = r["attributes"][o0:o1]
            if not np.array_equal(gr["side"], oa[:, 3]):
                bad.append((p, "side"))
                continue
            of = oa[:, :3].copy().view(np.float32)
            gf = np.stack([gr["normal_x"], gr["normal_y"], gr["advancement"]], axis=1)
            length = float(np.nanmax(np.abs(of[:, 2]))) if len(of) else 0.0
            nscale = max(1.0, float(np.nanmax(np.abs(of[:, :2]))) if len(of) else 1.0)
            if not (np.allclose(gf[:, :2], of[:, :2], rtol=0, atol=RTOL * nscale,
                                equal_nan=True) and
                    np.allclose(gf[:, 2], of[:, 2], rtol=0, atol=RTOL * max(1.0, length),
                                equal_nan=True)):
                bad.append((p, "attributes"))
    return bad, exact


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


def test_vw_lyon_cases_single_path(gpu):
    # Every variable-width case of lyon's stroke tests (test_square, test_empty_caps,
    # issue_821, issue_894), one lyon_gpu_stroke_path_variable_width call each.
    with open(os.path.join(GOLDEN, "lyon_stroke_cases.json")) as f:
        cases = [c for c in json.load(f) if c["options"].get("variable_line_width")]
    assert len(cases) >= 9
    for case in cases:
        path = case_path(case)
        opts = stroke_options_from_case(case["options"])
        ref = orc.stroke(path, opts, 16, widths=case["widths"])
        buffers = T.VertexBuffers(16)
        builder = T.BuffersBuilder(buffers)
        tess = T.StrokeTessellator(gpu.ctx())
        try:
            tess.tessellate_path(path, opts, builder, widths=case["widths"])
            st = 0
        except T.TessellationError as e:
            st = e.code
        assert st == ref.status, case["src"]
        if st != 0:
            continue
        assert np.array_equal(buffers.indices, ref.indices), case["src"]
        assert np.allclose(buffers.vertices, ref.vertices, rtol=0, atol=1e-4), case["src"]
        if case["expect_triangles"] is not None:
            assert len(buffers.indices) // 3 == case["expect_triangles"], case["src"]


def test_vw_batched_curves(gpu):
    # Lines, quadratics (some with a sharp-turn split) and cubics, closed and open, every join
    # and cap, width factors 0.2-3 per endpoint.
    batch, _ = workloads.batched_stroke(1500, seed=81)
    opts = _options(batch.num_paths, 82)
    widths = np.random.default_rng(83).uniform(0.2, 3.0, size=len(batch.points)).astype(
        np.float32)
    bad, exact = compare_vw(gpu, batch, opts, widths)
    print(f"paths={batch.num_paths} exact={exact} bad={len(bad)}")
    assert len(bad) <= max(2, batch.num_paths // 500), bad[:10]


def test_vw_polylines_u16_and_attributes(gpu):
    poly, popts = workloads.map_polylines(2000, seed=84, max_len=200)
    rng = np.random.default_rng(85)
    widths = rng.uniform(0.5, 2.0, size=len(poly.points)).astype(np.float32)
    bad, exact = compare_vw(gpu, poly, popts, widths, index_bits=16)
    assert len(bad) <= max(2, poly.num_paths // 500), bad[:10]
    bad, exact = compare_vw(gpu, poly, popts, widths, attributes=True)
    print(f"paths={poly.num_paths} exact={exact} bad={len(bad)}")
    assert len(bad) <= max(2, poly.num_paths // 500), bad[:10]


def test_vw_constant_factor_keeps_topology_close_to_fixed_width(gpu):
    # With every factor 1 the variable-width stepper strokes straight segments like the fixed
    # width one: same vertex and index counts on line-only paths with miter joins within limit.
    verbs = [Verb.BEGIN, Verb.LINE_TO, Verb.LINE_TO, Verb.LINE_TO, Verb.END]
    pts = [[0.0, 0.0], [10.0, 0.0], [10.0, 10.0], [20.0, 12.0], [0.0, 0.0]][:4]
    path = Path.from_arrays(verbs, pts)
    batch = PathBatch.from_paths([path])
    opts = _options(1, 86)
    opts["line_join"] = LineJoin.Miter
    opts["miter_limit"] = 10.0
    g = _gpu_vw(gpu, batch, opts, np.ones(len(batch.points), np.float32))
    f = gpu.gpu_batch("stroke", batch, opts, index_bits=32, index_mode=T.INDEX_PER_PATH)
    assert len(g["vertices"]) == len(f["vertices"])
    assert np.array_equal(g["indices"], f["indices"])
    assert np.allclose(g["vertices"], f["vertices"], rtol=0, atol=1e-4)
