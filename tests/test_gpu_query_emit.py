"""The sizing and emitting halves of the batched calls (lyon_gpu_query_sizes,
lyon_gpu_emit_into): totals first, then the output into caller-allocated device buffers, equal to
the one-call form's output."""

import ctypes

import numpy as np
import pytest

from lyon_gb300 import _native, workloads
from lyon_gb300 import tessellation as T

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gpu():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import gpu_helpers
    return gpu_helpers


@pytest.mark.parametrize("kind", ["stroke", "fill"])
def test_query_then_emit_matches_one_call(gpu, kind):
    import torch
    c = gpu.ctx()
    if kind == "stroke":
        batch, opts = workloads.batched_stroke(2000, seed=151)
    else:
        batch, opts = workloads.glyph_fill(2000, seed=152)
    ref = gpu.gpu_batch(kind, batch, opts, index_bits=32, index_mode=T.INDEX_GLOBAL,
                        vertex_offset=7)
    db = T.DeviceBatch.upload(batch, 0)
    od = T.upload_options(opts, 0)
    cb = db.c()
    k = 0 if kind == "stroke" else 1
    tv, ti, failed = ctypes.c_uint64(), ctypes.c_uint64(), ctypes.c_uint32()
    r = c.lib.lyon_gpu_query_sizes(c.h, k, ctypes.byref(cb), od.data_ptr(), len(opts), 32,
                                   T.INDEX_GLOBAL, 7, ctypes.byref(tv), ctypes.byref(ti),
                                   ctypes.byref(failed))
    assert r == 0
    assert tv.value == ref["total_vertices"] and ti.value == ref["total_indices"]
    verts = torch.empty((tv.value, 2), dtype=torch.float32, device="cuda")
    idx = torch.empty(ti.value, dtype=torch.int32, device="cuda")
    out = _native.CBatchOutput()
    r = c.lib.lyon_gpu_emit_into(c.h, k, ctypes.byref(cb), od.data_ptr(), len(opts), 32,
                                 T.INDEX_GLOBAL, 7, verts.data_ptr(), idx.data_ptr(),
                                 ctypes.byref(out))
    assert r == 0
    c.synchronize()
    assert int(out.vertices) == verts.data_ptr() and int(out.total_vertices) == tv.value
    assert np.array_equal(verts.cpu().numpy(), ref["vertices"])
    assert np.array_equal(idx.cpu().numpy().view(np.uint32), ref["indices"])
    # A second emit without a new query is refused.
    r = c.lib.lyon_gpu_emit_into(c.h, k, ctypes.byref(cb), od.data_ptr(), len(opts), 32,
                                 T.INDEX_GLOBAL, 7, verts.data_ptr(), idx.data_ptr(),
                                 ctypes.byref(out))
    assert r == T.LYON_ERR_INVALID_ARGUMENT


def test_emit_with_other_arguments_is_refused(gpu):
    c = gpu.ctx()
    batch, opts = workloads.batched_stroke(100, seed=153)
    db = T.DeviceBatch.upload(batch, 0)
    od = T.upload_options(opts, 0)
    cb = db.c()
    tv, ti = ctypes.c_uint64(), ctypes.c_uint64()
    assert c.lib.lyon_gpu_query_sizes(c.h, 0, ctypes.byref(cb), od.data_ptr(), len(opts), 32,
                                      T.INDEX_PER_PATH, 0, ctypes.byref(tv), ctypes.byref(ti),
                                      None) == 0
    out = _native.CBatchOutput()
    # index bits differ from the query
    assert c.lib.lyon_gpu_emit_into(c.h, 0, ctypes.byref(cb), od.data_ptr(), len(opts), 16,
                                    T.INDEX_PER_PATH, 0, None, None,
                                    ctypes.byref(out)) == T.LYON_ERR_INVALID_ARGUMENT


def test_deferred_calls_equal_sequential_calls():
    # DeferredTessellator: 300 strokes and 60 fills recorded into two builders (one u16, which
    # overflows part-way, one u32) and run as one batched launch per kind at flush(), against the
    # same calls made one by one through the single-path drop-in.
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from lyon_gb300 import workloads
    from lyon_gb300.options import FillOptions, StrokeOptions
    sb, so = workloads.plain_stroke(300, seed=61)
    fb, _ = workloads.glyph_fill(60, seed=62)
    sopt = StrokeOptions(*[so[0][k].item() for k in so.dtype.names])
    fopt = FillOptions(tolerance=0.1)
    ctx = T.Context(0)
    seq = [T.VertexBuffers(16), T.VertexBuffers(32)]
    dfr = [T.VertexBuffers(16), T.VertexBuffers(32)]
    seq_b = [T.BuffersBuilder(b) for b in seq]
    dfr_b = [T.BuffersBuilder(b) for b in dfr]
    d = T.DeferredTessellator(ctx)
    seq_err = []
    st, ft = T.StrokeTessellator(ctx), T.FillTessellator(ctx)
    for k in range(sb.num_paths + fb.num_paths):
        which = k % 2
        if k < sb.num_paths:
            path, kind = sb.path(k), "stroke"
        else:
            path, kind = fb.path(k - sb.num_paths), "fill"
        try:
            if kind == "stroke":
                st.tessellate_path(path, sopt, seq_b[which])
            else:
                ft.tessellate_path(path, fopt, seq_b[which])
            seq_err.append(None)
        except T.TessellationError as e:
            seq_err.append(e.code)
        if kind == "stroke":
            d.stroke(path, sopt, dfr_b[which])
        else:
            d.fill(path, fopt, dfr_b[which])
    got = [None if e is None else e.code for e in d.flush()]
    assert got == seq_err
    assert any(e == T.LYON_ERR_TOO_MANY_VERTICES for e in got)
    for a, b in zip(seq, dfr):
        assert np.array_equal(a.indices, b.indices)
        assert np.array_equal(a.vertices, b.vertices)
