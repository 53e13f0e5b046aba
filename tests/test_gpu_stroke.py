"""GPU parity: the CUDA stroke path against the oracle on seeded inputs and lyon's fixtures.

The bar: per-path vertex and index counts and the index topology match exactly,
except where the oracle flags a count decided by a value within 1e-6 of an integer (counted and
reported); vertex positions match within 1e-5 relative (`RTOL`).
"""

import numpy as np
import pytest

from lyon_gb300 import workloads
from lyon_gb300 import tessellation as T
from lyon_gb300.options import LineCap, LineJoin, StrokeOptions, stroke_options_array
from lyon_gb300.path import PathBatch
from oracle import lyon_oracle as orc

from lyon_cases import case_path, load, rust_logo, stroke_options_from_case

pytestmark = pytest.mark.gpu

RTOL = 1e-5


@pytest.fixture(scope="module")
def gpu():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import gpu_helpers
    return gpu_helpers


def _report(s):
    print(f"paths={s['paths']} mismatches={len(s['mismatches'])} "
          f"near_tie_mismatches={s['near_tie_mismatches']} exact={s['exact_vertex_paths']}")


def test_plain_stroke_workload(gpu):
    # 1,000 paths x 16 segments, miter (4) / butt, width 4, tol 0.1, u16 per path.
    batch, opts = workloads.plain_stroke(1000, seed=1)
    s = gpu.compare_per_path("stroke", batch, opts, index_bits=16)
    _report(s)
    assert not s["mismatches"], s["mismatches"][:10]


def test_batched_stroke_workload_subset(gpu):
    # The batched workload's generator (round joins/caps, tol 0.05, widths 0.5-8, u32).
    batch, opts = workloads.batched_stroke(20000, seed=2)
    s = gpu.compare_per_path("stroke", batch, opts, index_bits=32)
    _report(s)
    assert not s["mismatches"], s["mismatches"][:10]
    assert s["near_tie_mismatches"] <= max(2, batch.num_paths // 1000)


@pytest.mark.parametrize("join", [LineJoin.Miter, LineJoin.MiterClip, LineJoin.Round,
                                  LineJoin.Bevel])
@pytest.mark.parametrize("cap", [LineCap.Butt, LineCap.Square, LineCap.Round])
def test_joins_and_caps(gpu, join, cap):
    batch, _ = workloads.plain_stroke(300, seed=7)
    rng = np.random.default_rng(join * 3 + cap)
    recs = []
    for i in range(batch.num_paths):
        o = StrokeOptions(line_join=join, line_width=float(rng.uniform(0.5, 40.0)),
                          miter_limit=float(rng.uniform(1.0, 6.0)),
                          tolerance=float(rng.choice([0.01, 0.1, 1.0]))).with_line_cap(cap)
        recs.append(o.to_record()[0])
    opts = stroke_options_array(recs)
    s = gpu.compare_per_path("stroke", batch, opts, index_bits=32)
    _report(s)
    assert not s["mismatches"], s["mismatches"][:10]


def test_lyon_stroke_fixtures(gpu):
    # Every stroke fixture of lyon's tests, through the single-path drop-in, equals the oracle.
    for case in load("lyon_stroke_cases.json"):
        path = case_path(case)
        opts = stroke_options_from_case(case["options"])
        ref = orc.stroke(path, opts, index_bits=16)
        buf = T.VertexBuffers(16)
        T.StrokeTessellator(gpu.ctx()).tessellate_path(path, opts, T.BuffersBuilder(buf))
        assert np.array_equal(buf.indices, ref.indices), case["src"]
        assert np.allclose(buf.vertices, ref.vertices, rtol=RTOL, atol=RTOL), case["src"]
        if case["expect_triangles"] is not None:
            assert len(buf.indices) // 3 == case["expect_triangles"]


def test_logo_all_options(gpu):
    logo = rust_logo()
    paths = [logo] * 12
    recs = []
    for join in (LineJoin.Miter, LineJoin.MiterClip, LineJoin.Round, LineJoin.Bevel):
        for cap in (LineCap.Butt, LineCap.Square, LineCap.Round):
            recs.append(StrokeOptions(line_join=join, tolerance=0.05).with_line_cap(cap)
                        .to_record()[0])
    batch = PathBatch.from_paths(paths)
    s = gpu.compare_per_path("stroke", batch, stroke_options_array(recs), index_bits=32)
    _report(s)
    assert not s["mismatches"]


def test_too_many_vertices_single_path(gpu):
    # stroke.rs test_too_many_vertices: a builder with 0/10/100 ids left fails and appends
    # nothing.
    for free in (0, 10, 100):
        buf = T.VertexBuffers(16)
        b = T.BuffersBuilder(buf, vertex_offset=65536 - free)
        with pytest.raises(T.TessellationError) as e:
            T.StrokeTessellator(gpu.ctx()).tessellate_path(rust_logo(),
                                                           StrokeOptions(tolerance=0.05), b)
        assert e.value.code == T.LYON_ERR_TOO_MANY_VERTICES
        assert len(buf.vertices) == 0 and len(buf.indices) == 0


def test_global_index_mode_matches_sequential_appends(gpu):
    # LYON_INDEX_GLOBAL: the batch equals tessellate_path called path by path on one
    # VertexBuffers (u32), including absolute indices.
    batch, opts = workloads.plain_stroke(200, seed=5)
    g = gpu.gpu_batch("stroke", batch, opts, index_bits=32, index_mode=T.INDEX_GLOBAL)
    out = orc.Output(32)
    for p in range(batch.num_paths):
        from lyon_gb300.options import StrokeOptions as SO
        o = SO(*[opts[0][k].item() for k in opts.dtype.names])
        assert out.stroke(batch.path(p), o) == 0
    ref = out.snapshot(0)
    assert np.array_equal(g["indices"], ref.indices32)
    assert np.allclose(g["vertices"], ref.vertices, rtol=RTOL, atol=RTOL)


def test_global_u16_overflow_rolls_back_per_path(gpu):
    # 1,000 plain-stroke paths (~1.4M vertices) into one u16 buffer: paths that would overflow
    # fail with TooManyVertices and are rolled back; later smaller paths may still fit.
    batch, opts = workloads.plain_stroke(300, seed=9)
    g = gpu.gpu_batch("stroke", batch, opts, index_bits=16, index_mode=T.INDEX_GLOBAL)
    out = orc.Output(16)
    from lyon_gb300.options import StrokeOptions as SO
    o = SO(*[opts[0][k].item() for k in opts.dtype.names])
    statuses = [out.stroke(batch.path(p), o) for p in range(batch.num_paths)]
    ref = out.snapshot(0)
    assert list(g["status"]) == statuses
    assert np.array_equal(g["indices"], ref.indices)
    assert np.allclose(g["vertices"], ref.vertices, rtol=RTOL, atol=RTOL)


def test_flatten_counts_and_points(gpu):
    import torch
    batch, _ = workloads.batched_stroke(3000, seed=21)
    c = gpu.ctx()
    db = T.DeviceBatch.upload(batch, 0)
    for tol in (0.01, 0.1, 1.0):
        counts = torch.zeros(len(batch.verbs), dtype=torch.int32, device="cuda")
        r = c.lib.lyon_gpu_flatten_counts(c.h, db.c(), tol, counts.data_ptr())
        assert r == 0
        import ctypes
        pp = ctypes.c_void_p()
        po = ctypes.c_void_p()
        tot = ctypes.c_uint64()
        r = c.lib.lyon_gpu_flatten_paths(c.h, db.c(), tol, ctypes.byref(pp), ctypes.byref(po),
                                         ctypes.byref(tot))
        assert r == 0
        c.synchronize()
        gc = counts.cpu().numpy().view(np.uint32)
        gp = torch.as_tensor(T._CudaArray(pp.value, (tot.value, 2), "<f4"),
                             device="cuda").cpu().numpy()
        oc = []
        op = []
        for p in range(batch.num_paths):
            cc, pts = orc.flatten(batch.path(p), tol)
            oc.append(cc)
            op.append(pts)
        oc = np.concatenate(oc)
        op = np.concatenate(op)
        assert np.array_equal(gc, oc)
        assert gp.shape == op.shape
        assert np.array_equal(gp, op)


@pytest.mark.parametrize("pinned", [False, True, "host_alloc"])
def test_host_buffer_entry_point_matches_device(gpu, pinned, monkeypatch):
    # lyon_gpu_stroke_paths_host in several chunks (staged copies for pageable buffers, direct
    # writes for pinned ones and for lyon_gpu_host_alloc's huge-page buffers, inputs included)
    # equals the device-buffer call; too-small buffers give CAPACITY.
    import ctypes
    import torch
    from lyon_gb300 import _native
    monkeypatch.setenv("LYON_GB300_HOST_CHUNK_PATHS", "700")
    batch, opts = workloads.batched_stroke(3000, seed=41)
    g = gpu.gpu_batch("stroke", batch, opts, index_bits=32, index_mode=T.INDEX_GLOBAL)
    tv, ti = int(g["total_vertices"]), int(g["total_indices"])
    keep = []

    def in_host_buffer(a):
        a = np.ascontiguousarray(a)
        if pinned != "host_alloc":
            return a
        hb_ = T.HostBuffer(a.nbytes)
        v_ = hb_.array(a.dtype, a.size)
        v_[...] = a.reshape(-1)
        keep.append(hb_)
        return v_

    if pinned == "host_alloc":
        out_v, out_i = T.HostBuffer(8 * tv), T.HostBuffer(4 * ti)
        keep += [out_v, out_i]
        vptr, iptr = out_v.ptr, out_i.ptr
        get = lambda: (out_v.array(np.float32).reshape(-1, 2), out_i.array(np.uint32))  # noqa: E731
    elif pinned:
        hv_t = torch.empty(2 * tv, dtype=torch.float32, pin_memory=True)
        hi_t = torch.empty(ti, dtype=torch.int32, pin_memory=True)
        vptr, iptr = hv_t.data_ptr(), hi_t.data_ptr()
        get = lambda: (hv_t.numpy().reshape(-1, 2), hi_t.numpy().view(np.uint32))  # noqa: E731
    else:
        hv = np.empty(2 * tv, np.float32)
        hi = np.empty(ti, np.uint32)
        vptr, iptr = hv.ctypes.data, hi.ctypes.data
        get = lambda: (hv.reshape(-1, 2), hi)  # noqa: E731
    lib = gpu.ctx().lib
    vs = in_host_buffer(batch.verbs)
    ps = in_host_buffer(batch.points)
    vo = in_host_buffer(batch.verb_offsets)
    po = in_host_buffer(batch.point_offsets)
    hb = _native.CPathBatch(vs.ctypes.data, ps.ctypes.data, vo.ctypes.data, po.ctypes.data,
                            batch.num_paths)
    oh = in_host_buffer(opts)
    status = np.full(batch.num_paths, -7, np.int32)
    a, b = ctypes.c_uint64(), ctypes.c_uint64()
    r = lib.lyon_gpu_stroke_paths_host(gpu.ctx().h, ctypes.byref(hb), oh.ctypes.data, len(oh),
                                       32, T.INDEX_GLOBAL, 0, vptr, tv, iptr, ti,
                                       status.ctypes.data, ctypes.byref(a), ctypes.byref(b))
    assert r == 0 and a.value == tv and b.value == ti
    v, i = get()
    assert np.array_equal(i, g["indices"])
    assert np.array_equal(v, g["vertices"])
    assert np.array_equal(status, g["status"])
    r = lib.lyon_gpu_stroke_paths_host(gpu.ctx().h, ctypes.byref(hb), oh.ctypes.data, len(oh),
                                       32, T.INDEX_GLOBAL, 0, vptr, tv // 2, iptr, ti, None,
                                       ctypes.byref(a), ctypes.byref(b))
    assert r == T.LYON_ERR_CAPACITY and a.value == tv and b.value == ti
    for hb_ in keep:
        hb_.close()


def test_batched_stroke_full_size_counts(gpu):
    # The full 1,000,000-path batched workload: every path's vertex and index counts and status
    # equal the oracle's (all host threads run the oracle).
    import os
    batch, opts = workloads.batched_stroke(1_000_000, seed=2)
    ref = orc.batch("stroke", batch, opts, 32, os.cpu_count() or 1, want_output=False)
    c = gpu.ctx()
    db = T.DeviceBatch.upload(batch, 0)
    od = T.upload_options(opts, 0)
    res = T.tessellate_paths("stroke", db, od, len(opts), 32, T.INDEX_PER_PATH, 0, c)
    c.synchronize()
    vo, io = res.offsets()
    gv = np.diff(vo.cpu().numpy())
    gi = np.diff(io.cpu().numpy())
    st = res.statuses().cpu().numpy()
    assert np.array_equal(st, ref["status"])
    bad = np.nonzero((gv != ref["vtx_counts"]) | (gi != ref["idx_counts"]))[0]
    assert len(bad) == 0, bad[:10]
    assert int(gv.sum()) == int(ref["vtx_counts"].sum())


@pytest.mark.parametrize("tol", [0.01, 0.1, 1.0])
def test_map_polylines_subset(gpu, tol):
    # The map-polyline generator (open polylines, Pareto lengths, miter/bevel/round joins, widths
    # 1-8, coordinates up to 65536) at each tolerance of its sweep.
    batch, opts = workloads.map_polylines(3000, seed=4, tolerance=tol, max_len=3000)
    s = gpu.compare_per_path("stroke", batch, opts, index_bits=32)
    _report(s)
    assert not s["mismatches"], s["mismatches"][:10]
    assert s["near_tie_mismatches"] <= max(2, batch.num_paths // 1000)


def test_autotuner_picks_a_setting_and_keeps_outputs(gpu):
    import ctypes
    from lyon_gb300 import _native
    batch, opts = workloads.map_polylines(4000, seed=44, max_len=5000)
    before = gpu.gpu_batch("stroke", batch, opts, index_bits=32)
    c = gpu.ctx()
    db = T.DeviceBatch.upload(batch, 0)
    od = T.upload_options(opts, 0)
    cb = db.c()
    best = _native.CStrokeTuning()
    times = (ctypes.c_float * 16)()
    nc = ctypes.c_uint32()
    saved = _native.CStrokeTuning()
    assert c.lib.lyon_gpu_get_stroke_tuning(c.h, ctypes.byref(saved)) == 0
    try:
        r = c.lib.lyon_gpu_autotune_stroke(c.h, ctypes.byref(cb), od.data_ptr(), len(opts), 2000,
                                           ctypes.byref(best), times, ctypes.byref(nc))
        assert r == 0 and nc.value == 16
        assert all(t > 0.0 for t in times)
        cur = _native.CStrokeTuning()
        c.lib.lyon_gpu_get_stroke_tuning(c.h, ctypes.byref(cur))
        assert (cur.long_path_points, cur.blocks_per_sm, cur.short_path_points) == (
            best.long_path_points, best.blocks_per_sm, best.short_path_points)
        after = gpu.gpu_batch("stroke", batch, opts, index_bits=32)
        assert np.array_equal(after["indices"], before["indices"])
        assert np.array_equal(after["vertices"], before["vertices"])
    finally:
        c.lib.lyon_gpu_set_stroke_tuning(c.h, ctypes.byref(saved))


def test_plain_per_path_entry_point_counts(gpu):
    # lyon_gpu_stroke_paths_each (the per-path pipeline the batched call is measured against)
    # strokes each path by itself: its vertex total equals the batched call's for those paths.
    import ctypes
    batch, opts = workloads.batched_stroke(300, seed=9)
    g = gpu.gpu_batch("stroke", batch, opts, index_bits=32)
    c = gpu.ctx()
    db = T.DeviceBatch.upload(batch, 0)
    od = T.upload_options(opts, 0)
    cb = db.c()
    tv = ctypes.c_uint64(0)
    r = c.lib.lyon_gpu_stroke_paths_each(c.h, ctypes.byref(cb), od.data_ptr(), len(opts), 32,
                                         100, 150, ctypes.byref(tv))
    assert r == 0
    assert tv.value == int(g["vtx_offsets"][250] - g["vtx_offsets"][100])
    bad = c.lib.lyon_gpu_stroke_paths_each(c.h, ctypes.byref(cb), od.data_ptr(), len(opts), 32,
                                           200, 101, ctypes.byref(tv))
    assert bad == T.LYON_ERR_INVALID_ARGUMENT
