"""Shared helpers for the GPU parity tests (run the CUDA library and the oracle on the same
seeded inputs and compare)."""

from __future__ import annotations

import numpy as np

from lyon_gb300 import tessellation as T
from oracle import lyon_oracle as orc

_CTX = None


def ctx():
    global _CTX
    if _CTX is None:
        _CTX = T.Context(0)
    return _CTX


def gpu_batch(kind, batch, opts, index_bits=32, index_mode=T.INDEX_PER_PATH, vertex_offset=0):
    """Runs a batched call and returns host copies: vertices, indices (u32 view), status,
    per-path vertex/index offsets."""
    c = ctx()
    db = T.DeviceBatch.upload(batch, 0)
    od = T.upload_options(opts, 0)
    res = T.tessellate_paths(kind, db, od, len(opts), index_bits=index_bits,
                             index_mode=index_mode, vertex_offset=vertex_offset, ctx=c)
    c.synchronize()
    v = res.vertices().cpu().numpy() if res.total_vertices else np.zeros((0, 2), np.float32)
    if res.total_indices:
        i = res.indices().cpu().numpy()
        i = i.view(np.uint16) if index_bits == 16 else i.view(np.uint32)
    else:
        i = np.zeros(0, np.uint16 if index_bits == 16 else np.uint32)
    st = res.statuses().cpu().numpy()
    vo, io = res.offsets()
    return dict(vertices=v, indices=i, status=st, vtx_offsets=vo.cpu().numpy(),
                idx_offsets=io.cpu().numpy(), total_vertices=res.total_vertices,
                total_indices=res.total_indices, failed=res.num_failed_paths)


def compare_per_path(kind, batch, opts, index_bits=32, rtol=1e-5, allow_near_ties=True):
    """GPU (per-path indices) vs oracle path by path. Returns a summary dict; raises on any
    mismatch that is not explained by a near-integer count decision flagged by the oracle."""
    g = gpu_batch(kind, batch, opts, index_bits=index_bits, index_mode=T.INDEX_PER_PATH)
    r = orc.batch(kind, batch, opts, index_bits, 8)
    n = batch.num_paths
    mism = []
    tie_mism = 0
    exact_vertices = 0
    for p in range(n):
        gst = int(g["status"][p])
        ost = int(r["status"][p])
        gv0, gv1 = int(g["vtx_offsets"][p]), int(g["vtx_offsets"][p + 1])
        gi0, gi1 = int(g["idx_offsets"][p]), int(g["idx_offsets"][p + 1])
        ov0, ov1 = int(r["vtx_offsets"][p]), int(r["vtx_offsets"][p + 1])
        oi0, oi1 = int(r["idx_offsets"][p]), int(r["idx_offsets"][p + 1])
        ok = gst == ost
        if ok and gst == 0:
            gi = g["indices"][gi0:gi1].astype(np.uint64)
            oi = r["indices"][oi0:oi1].astype(np.uint64)
            if index_bits == 16:
                oi = oi & 0xFFFF
            ok = (gv1 - gv0 == ov1 - ov0) and np.array_equal(gi, oi)
            if ok:
                gv = g["vertices"][gv0:gv1]
                ov = r["vertices"][ov0:ov1]
                if np.array_equal(gv, ov):
                    exact_vertices += 1
                else:
                    # "Relative" is taken against the path's coordinate scale (its largest input
                    # coordinate plus its line width): a vertex near the origin carries the same
                    # absolute rounding as one far from it.
                    pp0 = batch.point_offsets[p]
                    pp1 = batch.point_offsets[p + 1]
                    pts = batch.points[pp0:pp1]
                    lw = float(opts[p if len(opts) > 1 else 0]["line_width"]) \
                        if "line_width" in (opts.dtype.names or ()) else 0.0
                    scale = max(1.0, float(np.abs(pts).max()) if len(pts) else 1.0) + lw
                    ok = bool((np.abs(gv - ov) <= rtol * np.maximum(np.abs(ov), scale)).all())
        if not ok:
            if allow_near_ties and int(r["near_ties"][p]) > 0:
                tie_mism += 1
            else:
                mism.append(p)
    return dict(paths=n, mismatches=mism, near_tie_mismatches=tie_mism,
                exact_vertex_paths=exact_vertices, gpu=g, oracle=r)
