"""lyon_gpu_stroke_paths_noalloc: the stroke pipeline with caller-provided outputs and the
library's fixed scratch array, checked against lyon_gpu_stroke_paths on the same inputs and,
path by path, against the oracle.

The file is named to be collected last: the no-allocation entry point must give the same
results in a fresh process and after every other test has used the device.
"""

import ctypes

import numpy as np
import pytest

from lyon_gb300 import _native, workloads
from lyon_gb300 import tessellation as T

RTOL = 1e-5
MAX_PATHS = 262144  # LYON_NOALLOC_MAX_PATHS


def _noalloc(lib, dbatch, opts_dev, num_options, index_bits, index_mode, vcap, icap):
    import torch
    n = dbatch.num_paths
    dev = torch.device("cuda", 0)
    vertices = torch.empty(max(1, 2 * vcap), dtype=torch.float32, device=dev)
    indices = torch.empty(max(1, icap * index_bits // 8), dtype=torch.uint8, device=dev)
    voff = torch.empty(n + 1, dtype=torch.int64, device=dev)
    ioff = torch.empty(n + 1, dtype=torch.int64, device=dev)
    status = torch.empty(max(1, n), dtype=torch.int32, device=dev)
    tv, ti, failed = _native.u64(), _native.u64(), _native.u32()
    err = ctypes.create_string_buffer(256)
    torch.cuda.synchronize()
    cb = dbatch.c()
    r = lib.lyon_gpu_stroke_paths_noalloc(
        ctypes.byref(cb), opts_dev.data_ptr(), num_options, index_bits, index_mode, 0,
        vertices.data_ptr(), vcap, indices.data_ptr(), icap, voff.data_ptr(), ioff.data_ptr(),
        status.data_ptr(), ctypes.byref(tv), ctypes.byref(ti), ctypes.byref(failed), None, err,
        len(err))
    torch.cuda.synchronize()
    assert r == T.LYON_OK, (r, err.value)
    idt = np.uint16 if index_bits == 16 else np.uint32
    return dict(
        vertices=vertices[:2 * tv.value].cpu().numpy().reshape(-1, 2),
        indices=indices[:ti.value * index_bits // 8].cpu().numpy().view(idt),
        vtx_offsets=voff.cpu().numpy(), idx_offsets=ioff.cpu().numpy(),
        status=status[:n].cpu().numpy(), total_vertices=tv.value, total_indices=ti.value,
        failed=failed.value)


def _existing(ctx, dbatch, opts_dev, num_options, index_bits, index_mode):
    res = T.tessellate_paths("stroke", dbatch, opts_dev, num_options, index_bits=index_bits,
                             index_mode=index_mode, ctx=ctx)
    ctx.synchronize()
    idt = np.uint16 if index_bits == 16 else np.uint32
    v = res.vertices().cpu().numpy() if res.total_vertices else np.zeros((0, 2), np.float32)
    i = res.indices().cpu().numpy().view(idt) if res.total_indices else np.zeros(0, idt)
    vo, io = res.offsets()
    return dict(vertices=v, indices=i, vtx_offsets=vo.cpu().numpy(),
                idx_offsets=io.cpu().numpy(), status=res.statuses().cpu().numpy(),
                total_vertices=res.total_vertices, total_indices=res.total_indices,
                failed=res.num_failed_paths)


def _check_same(a, b, batch, opts):
    assert a["total_vertices"] == b["total_vertices"]
    assert a["total_indices"] == b["total_indices"]
    assert a["failed"] == b["failed"]
    assert np.array_equal(a["status"], b["status"])
    assert np.array_equal(a["vtx_offsets"], b["vtx_offsets"])
    assert np.array_equal(a["idx_offsets"], b["idx_offsets"])
    assert np.array_equal(a["indices"], b["indices"])
    # Vertex tolerance of the parity tests: relative to the batch's coordinate scale.
    scale = max(1.0, float(np.abs(batch.points).max())) + float(opts["line_width"].max())
    assert np.abs(a["vertices"] - b["vertices"]).max(initial=0.0) <= RTOL * scale


def _check_oracle(got, batch, opts, index_bits, index_mode, vertex_offset=0):
    """Every path against the oracle's own VertexBuffers: same status; for paths that succeed,
    the same counts, the same triangles (global indices rebased to the path's first vertex) and
    vertices within RTOL of the batch's coordinate scale. Returns the number of paths that
    failed with TooManyVertices."""
    from oracle import lyon_oracle as orc
    ref = orc.batch("stroke", batch, opts, index_bits, 8)
    scale = max(1.0, float(np.abs(batch.points).max())) + float(opts["line_width"].max())
    vo, io = got["vtx_offsets"], got["idx_offsets"]
    too_many = 0
    for p in range(batch.num_paths):
        st = int(got["status"][p])
        if index_mode == T.INDEX_GLOBAL and st == T.LYON_ERR_TOO_MANY_VERTICES:
            # Rolled back by the global index range (BuffersBuilder overflow): no output.
            assert vo[p + 1] == vo[p] and io[p + 1] == io[p]
            too_many += 1
            continue
        assert st == int(ref["status"][p]), p
        if st != T.LYON_OK:
            continue
        rv0, rv1 = int(ref["vtx_offsets"][p]), int(ref["vtx_offsets"][p + 1])
        ri0, ri1 = int(ref["idx_offsets"][p]), int(ref["idx_offsets"][p + 1])
        assert int(vo[p + 1] - vo[p]) == rv1 - rv0, p
        assert int(io[p + 1] - io[p]) == ri1 - ri0, p
        gi = got["indices"][int(io[p]):int(io[p + 1])].astype(np.int64)
        if index_mode == T.INDEX_GLOBAL:
            gi = gi - (vertex_offset + int(vo[p]))
        oi = ref["indices"][ri0:ri1].astype(np.int64)
        if index_bits == 16:
            oi = oi & 0xFFFF
        assert np.array_equal(gi, oi), p
        gv = got["vertices"][int(vo[p]):int(vo[p + 1])]
        assert np.abs(gv - ref["vertices"][rv0:rv1]).max(initial=0.0) <= RTOL * scale, p
    return too_many


def test_rejects_batches_beyond_the_scratch_limit():
    # No device work: the size check comes before anything touches the GPU.
    lib = _native.load()
    dummy = np.zeros(64, np.uint8)
    p = dummy.ctypes.data
    cb = _native.CPathBatch(p, p, p, p, MAX_PATHS + 1)
    tv, ti, failed = _native.u64(7), _native.u64(7), _native.u32(7)
    err = ctypes.create_string_buffer(256)
    r = lib.lyon_gpu_stroke_paths_noalloc(
        ctypes.byref(cb), p, 1, 32, T.INDEX_PER_PATH, 0, p, 0, p, 0, p, p, p, ctypes.byref(tv),
        ctypes.byref(ti), ctypes.byref(failed), None, err, len(err))
    assert r == T.LYON_ERR_CAPACITY
    assert b"scratch limit" in err.value and str(MAX_PATHS).encode() in err.value
    assert tv.value == 0 and ti.value == 0 and failed.value == 0


@pytest.mark.gpu
def test_noalloc_matches_batched_entry_point_on_two_calls():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    lib = _native.load()
    ctx = T.Context(0)
    # Call 1: the batched workload's generator (round joins/caps, per-path options), global
    # u32 indices. Call 2: a smaller batch with one shared option record, u16 per-path indices,
    # so stale counts left in the scratch by call 1 would show. Both are also compared with the
    # oracle path by path.
    cases = [
        (workloads.batched_stroke(6000, seed=21), 32, T.INDEX_GLOBAL),
        (workloads.plain_stroke(700, seed=22), 16, T.INDEX_PER_PATH),
    ]
    for (batch, opts), bits, mode in cases:
        db = T.DeviceBatch.upload(batch, 0)
        od = T.upload_options(opts, 0)
        want = _existing(ctx, db, od, len(opts), bits, mode)
        got = _noalloc(lib, db, od, len(opts), bits, mode, want["total_vertices"],
                       want["total_indices"])
        assert want["total_vertices"] > 0
        _check_same(got, want, batch, opts)
        assert _check_oracle(got, batch, opts, bits, mode) == 0


@pytest.mark.gpu
def test_noalloc_global_u16_overflow_rolls_back_like_the_batched_entry_point():
    # Global 16-bit indices over 5,000 map polylines (about 101,600 vertices): the first path
    # past 65,535 vertices lies beyond the first 2,048-path chunk of the host fix-up, so the
    # running total is carried across chunks; every path that no longer fits fails with
    # TooManyVertices and writes nothing (BuffersBuilder's rollback,
    # geometry_builder.rs:338-350, 478-481), and later paths that fit still go through.
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    lib = _native.load()
    ctx = T.Context(0)
    batch, opts = workloads.map_polylines(5000, seed=24, tolerance=1.0)
    db = T.DeviceBatch.upload(batch, 0)
    od = T.upload_options(opts, 0)
    want = _existing(ctx, db, od, len(opts), 16, T.INDEX_GLOBAL)
    got = _noalloc(lib, db, od, len(opts), 16, T.INDEX_GLOBAL, want["total_vertices"],
                   want["total_indices"])
    _check_same(got, want, batch, opts)
    assert want["failed"] > 0
    too_many = np.nonzero(got["status"] == T.LYON_ERR_TOO_MANY_VERTICES)[0]
    assert len(too_many) == got["failed"] and too_many[0] >= 2048
    assert got["total_vertices"] <= 65536
    assert _check_oracle(got, batch, opts, 16, T.INDEX_GLOBAL) == got["failed"]


@pytest.mark.gpu
def test_noalloc_reports_sizes_when_outputs_are_too_small():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    lib = _native.load()
    batch, opts = workloads.plain_stroke(50, seed=23)
    db = T.DeviceBatch.upload(batch, 0)
    od = T.upload_options(opts, 0)
    want = _existing(T.Context(0), db, od, len(opts), 32, T.INDEX_PER_PATH)
    dev = torch.device("cuda", 0)
    buf = torch.zeros(16, dtype=torch.float32, device=dev)
    voff = torch.empty(batch.num_paths + 1, dtype=torch.int64, device=dev)
    ioff = torch.empty(batch.num_paths + 1, dtype=torch.int64, device=dev)
    status = torch.empty(batch.num_paths, dtype=torch.int32, device=dev)
    tv, ti, failed = _native.u64(), _native.u64(), _native.u32()
    err = ctypes.create_string_buffer(256)
    cb = db.c()
    r = lib.lyon_gpu_stroke_paths_noalloc(
        ctypes.byref(cb), od.data_ptr(), len(opts), 32, T.INDEX_PER_PATH, 0, buf.data_ptr(), 1,
        buf.data_ptr(), 1, voff.data_ptr(), ioff.data_ptr(), status.data_ptr(),
        ctypes.byref(tv), ctypes.byref(ti), ctypes.byref(failed), None, err, len(err))
    torch.cuda.synchronize()
    assert r == T.LYON_ERR_CAPACITY, err.value
    assert tv.value == want["total_vertices"] and ti.value == want["total_indices"]
    assert float(buf.abs().sum()) == 0.0
