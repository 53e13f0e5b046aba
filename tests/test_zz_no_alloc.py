"""lyon_gpu_stroke_paths_noalloc: the stroke pipeline with caller-provided outputs and the
library's fixed scratch array, checked against lyon_gpu_stroke_paths on the same inputs.

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
    # so stale counts left in the scratch by call 1 would show.
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
