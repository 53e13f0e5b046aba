"""GPU parity of the stroke vertex attribute output (lyon_stroke_vertex: position, normal,
advancement, side — what lyon's StrokeVertex hands a vertex constructor,
crates/tessellation/src/stroke.rs:2667-2720) against the oracle, path by path.

Sides and the index topology match exactly; positions, normals and advancements within
`RTOL` of the path's scale (bit-identical in practice). The records' positions and indices also
equal the positions-only output byte for byte.
"""

import numpy as np
import pytest

from lyon_gb300 import workloads
from lyon_gb300 import tessellation as T
from lyon_gb300.options import STROKE_OPTIONS_DTYPE, LineCap, LineJoin, StrokeOptions
from lyon_gb300.path import Path, PathBatch, Verb
from oracle import lyon_oracle as orc

from lyon_cases import rust_logo

pytestmark = pytest.mark.gpu

RTOL = 1e-5


@pytest.fixture(scope="module")
def gpu():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import gpu_helpers
    return gpu_helpers


def _records(gpu, batch, opts, index_bits=32, index_mode=T.INDEX_PER_PATH):
    c = gpu.ctx()
    db = T.DeviceBatch.upload(batch, 0)
    od = T.upload_options(opts, 0)
    res = T.tessellate_paths("stroke", db, od, len(opts), index_bits=index_bits,
                             index_mode=index_mode, ctx=c, attributes=True)
    c.synchronize()
    rec = (res.records().cpu().numpy().view(T.STROKE_VERTEX_DTYPE).reshape(-1)
           if res.total_vertices else np.zeros(0, T.STROKE_VERTEX_DTYPE))
    idx = res.indices().cpu().numpy() if res.total_indices else np.zeros(0, np.int32)
    idx = idx.view(np.uint16) if index_bits == 16 else idx.view(np.uint32)
    vo, io = res.offsets()
    return dict(records=rec, indices=idx, status=res.statuses().cpu().numpy(),
                vtx_offsets=vo.cpu().numpy(), idx_offsets=io.cpu().numpy())


def compare_attributes(gpu, batch, opts, index_bits=32):
    g = _records(gpu, batch, opts, index_bits)
    plain = gpu.gpu_batch("stroke", batch, opts, index_bits=index_bits,
                          index_mode=T.INDEX_PER_PATH)
    # Same topology and positions as the positions-only output, byte for byte.
    assert np.array_equal(g["status"], plain["status"])
    assert np.array_equal(g["indices"], plain["indices"])
    pos = np.stack([g["records"]["x"], g["records"]["y"]], axis=1)
    assert np.array_equal(pos, plain["vertices"])

    r = orc.batch("stroke", batch, opts, index_bits, 8, want_attributes=True)
    bad, exact = [], 0
    for p in range(batch.num_paths):
        if int(g["status"][p]) != int(r["status"][p]):
            bad.append((p, "status"))
            continue
        if g["status"][p] != 0:
            continue
        g0, g1 = int(g["vtx_offsets"][p]), int(g["vtx_offsets"][p + 1])
        o0, o1 = int(r["vtx_offsets"][p]), int(r["vtx_offsets"][p + 1])
        if g1 - g0 != o1 - o0:
            bad.append((p, "count"))
            continue
        gr = g["records"][g0:g1]
        oa = r["attributes"][o0:o1]
        of = oa[:, :3].copy().view(np.float32)
        gf = np.stack([gr["normal_x"], gr["normal_y"], gr["advancement"]], axis=1)
        if not np.array_equal(gr["side"], oa[:, 3]):
            bad.append((p, "side"))
            continue
        if np.array_equal(gf.view(np.uint32), of.view(np.uint32)):
            exact += 1
            continue
        pts = batch.points[batch.point_offsets[p]:batch.point_offsets[p + 1]]
        lw = float(opts[p if len(opts) > 1 else 0]["line_width"])
        length = float(np.abs(of[:, 2]).max()) if len(of) else 0.0
        nscale = max(1.0, float(np.abs(of[:, :2]).max()) if len(of) else 1.0)
        scale = max(1.0, float(np.abs(pts).max()) if len(pts) else 1.0) + lw + length
        if not (np.allclose(gf[:, :2], of[:, :2], rtol=0, atol=RTOL * nscale) and
                np.allclose(gf[:, 2], of[:, 2], rtol=0, atol=RTOL * scale)):
            bad.append((p, "values"))
    return bad, exact


def _all_joins_caps(n, seed):
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


def test_attributes_plain_stroke_all_options(gpu):
    batch, _ = workloads.plain_stroke(600, seed=71)
    opts = _all_joins_caps(batch.num_paths, 72)
    bad, exact = compare_attributes(gpu, batch, opts, index_bits=16)
    print(f"paths={batch.num_paths} exact={exact} bad={len(bad)}")
    assert not bad, bad[:10]


def test_attributes_batched_stroke_subset(gpu):
    batch, opts = workloads.batched_stroke(4000, seed=73)
    bad, exact = compare_attributes(gpu, batch, opts)
    print(f"paths={batch.num_paths} exact={exact} bad={len(bad)}")
    assert len(bad) <= max(2, batch.num_paths // 1000), bad[:10]


def test_attributes_polylines_and_short_paths(gpu):
    # Long polylines (warp walk) and short ones (one thread per path), several sub-paths,
    # closed sub-paths and repeated points: the advancement carries across sub-paths.
    poly, popts = workloads.map_polylines(1500, seed=74, max_len=300)
    rng = np.random.default_rng(75)
    paths = [poly.path(i) for i in range(poly.num_paths)]
    for _ in range(1500):
        verbs, pts = [], []
        for _ in range(int(rng.integers(1, 4))):
            m = int(rng.integers(1, 12))
            steps = rng.normal(0.0, 10.0, size=(m, 2))
            steps[0] = 0.0
            steps[rng.random(m) < 0.1] = 0.0
            p = rng.uniform(0.0, 500.0, size=2) + np.cumsum(steps, axis=0)
            verbs.append(Verb.BEGIN)
            pts.append(p[0])
            for q in p[1:]:
                verbs.append(Verb.LINE_TO)
                pts.append(q)
            if rng.random() < 0.4:
                verbs.append(Verb.CLOSE)
                pts.append(p[0])
            else:
                verbs.append(Verb.END)
        paths.append(Path.from_arrays(verbs, pts))
    batch = PathBatch.from_paths(paths)
    opts = np.concatenate([popts, _all_joins_caps(1500, 76)])
    bad, exact = compare_attributes(gpu, batch, opts)
    print(f"paths={batch.num_paths} exact={exact} bad={len(bad)}")
    assert not bad, bad[:10]


def test_attributes_single_path_vertex_constructor(gpu):
    logo = rust_logo()
    for join in (LineJoin.Miter, LineJoin.Round):
        opts = StrokeOptions(line_width=2.0, tolerance=0.05, line_join=join,
                             start_cap=LineCap.Round, end_cap=LineCap.Square)
        buffers = T.VertexBuffers(32)
        # A constructor that keeps normal and advancement, as a lyon user writing
        # `|v: StrokeVertex| MyVertex { pos: v.position(), normal: v.normal(), ... }` would.
        ctor = lambda r: np.stack([r["x"], r["y"], r["normal_x"], r["normal_y"],  # noqa: E731
                                   r["advancement"]], axis=1)
        builder = T.BuffersBuilder(buffers, vertex_ctor=ctor)
        T.StrokeTessellator(gpu.ctx()).tessellate_path(logo, opts, builder)
        ref = orc.stroke(logo, opts, 32, attributes=True)
        assert ref.status == 0
        assert np.array_equal(buffers.indices, ref.indices)
        assert buffers.vertices.shape == (len(ref.vertices), 5)
        assert np.allclose(buffers.vertices[:, :2], ref.vertices, rtol=0, atol=1e-3)
        of = ref.attributes[:, :3].copy().view(np.float32)
        assert np.allclose(buffers.vertices[:, 2:], of, rtol=0, atol=1e-3)


def test_attributes_close_merges_last_point(gpu):
    # Closing a sub-path whose last point lies within the merge distance of its first point:
    # lyon moves the last point onto the first and computes its advancement from the moved
    # position (stroke.rs:1218-1236). Both walks (one path per warp, one per thread).
    import ctypes
    from lyon_gb300 import _native
    p0 = [286.95037841796875, 342.3468017578125]
    a, b, c = [280.5752258300781, 348.7850341796875], [287.58062744140625, 346.4263610839844], \
        [286.912109375, 342.6481628417969]
    L, C = Verb.LINE_TO, Verb.CLOSE
    closed = Path.from_arrays([Verb.BEGIN, L, L, L, C], [p0, a, b, c, p0])
    # The same with the last point repeated (merged away inside the walk first).
    repeated = Path.from_arrays([Verb.BEGIN, L, L, L, L, C], [p0, a, b, c, c, p0])
    batch = PathBatch.from_paths([closed, repeated])
    opts = np.zeros(2, STROKE_OPTIONS_DTYPE)
    opts[:] = (LineCap.Butt, LineCap.Round, LineJoin.MiterClip, 1.5497823, 10.0, 1.0)
    c = gpu.ctx()
    saved = _native.CStrokeTuning()
    c.lib.lyon_gpu_get_stroke_tuning(c.h, ctypes.byref(saved))
    try:
        for short in (32, 0):
            t = _native.CStrokeTuning(saved.long_path_points, saved.blocks_per_sm, short)
            assert c.lib.lyon_gpu_set_stroke_tuning(c.h, ctypes.byref(t)) == 0
            bad, exact = compare_attributes(gpu, batch, opts)
            assert not bad and exact == 2, (short, bad)
    finally:
        c.lib.lyon_gpu_set_stroke_tuning(c.h, ctypes.byref(saved))
