"""ctypes binding of the oracle (TEST INFRASTRUCTURE ONLY).

The oracle is a CPU restatement of lyon's flattening, stroke and fill tessellators
(oracle/lyon_oracle.cpp). Only tests, `__graft_entry__.smoke()` and the CPU-baseline leg of
`bench.py` use it, as the checker; the product never imports this module.
"""

from __future__ import annotations

import ctypes
import os
import subprocess
import threading
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liblyon_oracle.so")

_lib = None
_lock = threading.Lock()


def build(force: bool = False) -> str:
    """Compiles the oracle with its Makefile (g++ only, a few seconds)."""
    if force or not os.path.exists(LIB_PATH) or (
            os.path.getmtime(LIB_PATH) < os.path.getmtime(os.path.join(HERE, "lyon_oracle.cpp"))):
        subprocess.check_call(["make", "-s", "-C", HERE], stdout=subprocess.DEVNULL)
    return LIB_PATH


def lib():
    global _lib
    with _lock:
        if _lib is None:
            build()
            L = ctypes.CDLL(LIB_PATH)
            c_p = ctypes.c_void_p
            L.lyon_oracle_out_new.restype = c_p
            L.lyon_oracle_out_new.argtypes = [ctypes.c_int, ctypes.c_uint64]
            L.lyon_oracle_out_free.argtypes = [c_p]
            L.lyon_oracle_out_clear.argtypes = [c_p]
            for n in ("num_vertices", "num_indices"):
                f = getattr(L, "lyon_oracle_out_" + n)
                f.restype = ctypes.c_uint64
                f.argtypes = [c_p]
            L.lyon_oracle_out_vertices.restype = ctypes.POINTER(ctypes.c_float)
            L.lyon_oracle_out_vertices.argtypes = [c_p]
            L.lyon_oracle_out_indices32.restype = ctypes.POINTER(ctypes.c_uint32)
            L.lyon_oracle_out_indices32.argtypes = [c_p]
            L.lyon_oracle_out_near_ties.restype = ctypes.c_uint32
            L.lyon_oracle_out_near_ties.argtypes = [c_p]
            for n in ("fast_atan2", "angle_to"):
                f = getattr(L, "lyon_oracle_" + n)
                f.restype = ctypes.c_float
                f.argtypes = [ctypes.c_float, ctypes.c_float]
            for n in ("stroke", "fill"):
                f = getattr(L, f"lyon_oracle_{n}_path")
                f.restype = ctypes.c_int
                f.argtypes = [c_p, c_p, ctypes.c_uint32, c_p, ctypes.c_uint32, c_p]
            L.lyon_oracle_flatten_path.restype = ctypes.c_uint64
            L.lyon_oracle_flatten_path.argtypes = [c_p, ctypes.c_uint32, c_p, ctypes.c_uint32,
                                                   ctypes.c_float, c_p, c_p, ctypes.c_uint64]
            L.lyon_oracle_wang.restype = ctypes.c_float
            L.lyon_oracle_wang.argtypes = [c_p, ctypes.c_int, ctypes.c_float]
            L.lyon_oracle_out_set_attributes.argtypes = [c_p, ctypes.c_int]
            L.lyon_oracle_out_attributes.restype = ctypes.POINTER(ctypes.c_uint32)
            L.lyon_oracle_out_attributes.argtypes = [c_p]
            L.lyon_oracle_batch_stroke_attributes.restype = ctypes.c_int
            L.lyon_oracle_batch_stroke_attributes.argtypes = [c_p, c_p, ctypes.c_uint32,
                                                              ctypes.c_int, c_p, c_p]
            L.lyon_oracle_fill_rectangle.restype = ctypes.c_int
            L.lyon_oracle_fill_rectangle.argtypes = [c_p] + [ctypes.c_float] * 4
            L.lyon_oracle_fill_circle.restype = ctypes.c_int
            L.lyon_oracle_fill_circle.argtypes = [c_p] + [ctypes.c_float] * 4
            L.lyon_oracle_stroke_path_vw.restype = ctypes.c_int
            L.lyon_oracle_stroke_path_vw.argtypes = [c_p, c_p, ctypes.c_uint32, c_p,
                                                     ctypes.c_uint32, c_p, c_p]
            L.lyon_oracle_batch_stroke_vw.restype = ctypes.c_int
            L.lyon_oracle_batch_stroke_vw.argtypes = [c_p, c_p, c_p, ctypes.c_uint32,
                                                      ctypes.c_int, ctypes.c_int] + [c_p] * 9
            L.lyon_oracle_out_set_sources.argtypes = [c_p, ctypes.c_int]
            L.lyon_oracle_out_sources.restype = ctypes.POINTER(ctypes.c_uint32)
            L.lyon_oracle_out_sources.argtypes = [c_p]
            L.lyon_oracle_batch_stroke_sources.restype = ctypes.c_int
            L.lyon_oracle_batch_stroke_sources.argtypes = [c_p, c_p, c_p, ctypes.c_uint32,
                                                           ctypes.c_int, ctypes.c_int] + [c_p] * 9
            L.lyon_oracle_interpolate.restype = None
            L.lyon_oracle_interpolate.argtypes = [c_p, ctypes.c_uint64, c_p, ctypes.c_uint32, c_p,
                                                  ctypes.c_int]
            L.lyon_oracle_out_num_fill_sources.restype = ctypes.c_uint64
            L.lyon_oracle_out_num_fill_sources.argtypes = [c_p]
            L.lyon_oracle_out_fill_sources.restype = ctypes.POINTER(ctypes.c_uint32)
            L.lyon_oracle_out_fill_sources.argtypes = [c_p]
            L.lyon_oracle_out_fill_source_counts.restype = ctypes.POINTER(ctypes.c_uint32)
            L.lyon_oracle_out_fill_source_counts.argtypes = [c_p]
            L.lyon_oracle_batch_fill_sources.restype = ctypes.c_int
            L.lyon_oracle_batch_fill_sources.argtypes = [c_p, c_p, ctypes.c_uint32, ctypes.c_int,
                                                         ctypes.c_int] + [c_p] * 11
            L.lyon_oracle_interpolate_fill.restype = None
            L.lyon_oracle_interpolate_fill.argtypes = [c_p, c_p, ctypes.c_uint64, c_p,
                                                       ctypes.c_uint32, c_p]
            L.lyon_oracle_flatten_arcs.restype = None
            L.lyon_oracle_flatten_arcs.argtypes = [c_p, ctypes.c_uint32, ctypes.c_float, c_p,
                                                   c_p, c_p, c_p, c_p]
            L.lyon_oracle_hatch.restype = None
            L.lyon_oracle_hatch.argtypes = [c_p, c_p, c_p, c_p, c_p, c_p]
            L.lyon_oracle_batch.restype = ctypes.c_int
            L.lyon_oracle_batch.argtypes = [ctypes.c_int, c_p, c_p, ctypes.c_uint32, ctypes.c_int,
                                            ctypes.c_int, c_p, c_p, c_p, c_p, c_p, c_p, c_p, c_p]
            _lib = L
    return _lib


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.c_void_p) if a is not None and a.size else None


class Result:
    """Output of one oracle call: positions, indices (u32 VertexId values), status."""

    def __init__(self, status, vertices, indices, near_ties, index_bits, attributes=None,
                 sources=None):
        self.status = status
        self.vertices = vertices
        # Vertex sources when requested: (V, 3) u32 words (from, to, t as f32 bits; `to` is
        # NO_ENDPOINT for VertexSource::Endpoint { id: from }).
        self.sources = sources
        # Stroke vertex attributes when requested: (V, 4) u32 words (normal x, normal y,
        # advancement as f32 bits; side 0 positive / 1 negative).
        self.attributes = attributes
        self.indices = indices if index_bits == 32 else indices.astype(np.uint16)
        self.indices32 = indices
        self.near_ties = near_ties

    @property
    def num_triangles(self):
        return len(self.indices) // 3


class Output:
    """A VertexBuffers + BuffersBuilder pair on the oracle side (append semantics)."""

    def __init__(self, index_bits: int = 32, vertex_offset: int = 0, attributes: bool = False,
                 sources: bool = False):
        self.L = lib()
        self.h = self.L.lyon_oracle_out_new(index_bits, vertex_offset)
        self.index_bits = index_bits
        self.attributes = attributes
        self.sources = sources
        if attributes:
            self.L.lyon_oracle_out_set_attributes(self.h, 1)
        if sources:
            self.L.lyon_oracle_out_set_sources(self.h, 1)

    def __del__(self):
        try:
            self.L.lyon_oracle_out_free(self.h)
        except Exception:
            pass

    def clear(self):
        self.L.lyon_oracle_out_clear(self.h)

    def snapshot(self, status) -> Result:
        nv = self.L.lyon_oracle_out_num_vertices(self.h)
        ni = self.L.lyon_oracle_out_num_indices(self.h)
        v = np.ctypeslib.as_array(self.L.lyon_oracle_out_vertices(self.h), shape=(nv * 2,)).copy() \
            if nv else np.zeros(0, np.float32)
        i = np.ctypeslib.as_array(self.L.lyon_oracle_out_indices32(self.h), shape=(ni,)).copy() \
            if ni else np.zeros(0, np.uint32)
        a = None
        if self.attributes:
            a = np.ctypeslib.as_array(self.L.lyon_oracle_out_attributes(self.h),
                                      shape=(nv * 4,)).copy().reshape(-1, 4) \
                if nv else np.zeros((0, 4), np.uint32)
        src = None
        res_fill = None
        if self.sources:
            nfs = self.L.lyon_oracle_out_num_fill_sources(self.h)
            if nfs or self._filled:
                fs = np.ctypeslib.as_array(self.L.lyon_oracle_out_fill_sources(self.h),
                                           shape=(nfs * 3,)).copy().reshape(-1, 3) \
                    if nfs else np.zeros((0, 3), np.uint32)
                fc = np.ctypeslib.as_array(self.L.lyon_oracle_out_fill_source_counts(self.h),
                                           shape=(nv,)).copy() if nv else np.zeros(0, np.uint32)
                res_fill = (fs, fc)
            else:
                src = np.ctypeslib.as_array(self.L.lyon_oracle_out_sources(self.h),
                                            shape=(nv * 3,)).copy().reshape(-1, 3) \
                    if nv else np.zeros((0, 3), np.uint32)
        r = Result(status, v.reshape(-1, 2), i, self.L.lyon_oracle_out_near_ties(self.h),
                   self.index_bits, a, src)
        if res_fill is not None:
            # Fill sources: (S, 3) words and the number of sources of each vertex.
            r.sources, r.source_counts = res_fill
        return r

    def stroke(self, path, options, widths=None):
        """`widths`: one variable-line-width factor per point (StrokeOptions::
        variable_line_width), or None for a fixed width."""
        o = options.to_c()
        v = np.ascontiguousarray(path.verbs, dtype=np.uint8)
        p = np.ascontiguousarray(path.points, dtype=np.float32)
        if widths is not None:
            w = np.ascontiguousarray(widths, dtype=np.float32)
            assert len(w) == len(p)
            return self.L.lyon_oracle_stroke_path_vw(self.h, _ptr(v), len(v), _ptr(p), len(p),
                                                     _ptr(w), ctypes.byref(o))
        return self.L.lyon_oracle_stroke_path(self.h, _ptr(v), len(v), _ptr(p), len(p),
                                              ctypes.byref(o))

    _filled = False

    def fill(self, path, options):
        self._filled = True
        o = options.to_c()
        v = np.ascontiguousarray(path.verbs, dtype=np.uint8)
        p = np.ascontiguousarray(path.points, dtype=np.float32)
        return self.L.lyon_oracle_fill_path(self.h, _ptr(v), len(v), _ptr(p), len(p),
                                            ctypes.byref(o))


def stroke(path, options, index_bits: int = 32, vertex_offset: int = 0,
           attributes: bool = False, widths=None, sources: bool = False) -> Result:
    out = Output(index_bits, vertex_offset, attributes, sources)
    st = out.stroke(path, options, widths)
    return out.snapshot(st)


NO_ENDPOINT = 0xFFFFFFFF


def interpolate_attributes(sources: np.ndarray, attributes: np.ndarray) -> np.ndarray:
    """StrokeVertex::interpolated_attributes (crates/tessellation/src/stroke.rs:2728-2747) for
    (V, 3) source words over an (endpoints, A) f32 attribute store: the endpoint's attributes,
    or a * (1 - t) + b * t along an edge, in f32 operation by operation."""
    src = np.asarray(sources, np.uint32).reshape(-1, 3)
    attrs = np.asarray(attributes, np.float32)
    attrs = attrs.reshape(len(attrs), -1)
    frm = src[:, 0].astype(np.int64)
    to = src[:, 1]
    t = src[:, 2].copy().view(np.float32)[:, None]
    edge = to != NO_ENDPOINT
    a = attrs[frm]
    b = attrs[np.where(edge, to, 0).astype(np.int64)]
    one = np.float32(1.0)
    lerp = (a * (one - t)).astype(np.float32) + (b * t).astype(np.float32)
    return np.where(edge[:, None], lerp, a).astype(np.float32)


def fill_rectangle(rect, index_bits: int = 32, vertex_offset: int = 0) -> Result:
    """FillTessellator::tessellate_rectangle (basic_shapes.rs:12-38); rect = (min_x, min_y,
    max_x, max_y)."""
    out = Output(index_bits, vertex_offset)
    st = out.L.lyon_oracle_fill_rectangle(out.h, *[float(x) for x in rect])
    return out.snapshot(st)


def fill_circle(center, radius, tolerance, index_bits: int = 32,
                vertex_offset: int = 0) -> Result:
    """FillTessellator::tessellate_circle (basic_shapes.rs:40-124)."""
    out = Output(index_bits, vertex_offset)
    st = out.L.lyon_oracle_fill_circle(out.h, float(center[0]), float(center[1]), float(radius),
                                       float(tolerance))
    return out.snapshot(st)


def fill(path, options, index_bits: int = 32, vertex_offset: int = 0,
         sources: bool = False) -> Result:
    """With `sources`, Result.sources holds every vertex's sources ((S, 3) words, path-local
    ids) and Result.source_counts the number per vertex."""
    out = Output(index_bits, vertex_offset, sources=sources)
    st = out.fill(path, options)
    return out.snapshot(st)


def interpolate_fill_attributes(sources: np.ndarray, counts: np.ndarray,
                                attributes: np.ndarray) -> np.ndarray:
    """FillVertex::interpolated_attributes (crates/tessellation/src/fill.rs:2208-2286): the
    first source's attributes (the endpoint's, or a * (1 - t) + b * t), the next sources' added
    in order, divided by the number of sources when there are several; f32 throughout."""
    src = np.ascontiguousarray(sources, np.uint32).reshape(-1, 3)
    cnt = np.asarray(counts, np.int64)
    attrs = np.asarray(attributes, np.float32)
    attrs = attrs.reshape(len(attrs), -1)
    vals = interpolate_attributes(src, attrs) if len(src) else np.zeros((0, attrs.shape[1]),
                                                                           np.float32)
    out = np.zeros((len(cnt), attrs.shape[1]), np.float32)
    starts = np.concatenate([[0], np.cumsum(cnt)[:-1]]) if len(cnt) else np.zeros(0, np.int64)
    kmax = int(cnt.max()) if len(cnt) else 0
    acc = np.zeros_like(out)
    for k in range(kmax):
        has = cnt > k
        idx = starts[has] + k
        acc[has] = vals[idx] if k == 0 else (acc[has] + vals[idx]).astype(np.float32)
    div = np.maximum(cnt, 1).astype(np.float32)[:, None]
    out = np.where(cnt[:, None] > 1, (acc / div).astype(np.float32), acc)
    return out.astype(np.float32)


def interpolate_fill_attributes_c(sources: np.ndarray, counts: np.ndarray,
                                  attributes: np.ndarray) -> np.ndarray:
    """interpolate_fill_attributes in C (the CPU baseline's version)."""
    src = np.ascontiguousarray(sources, np.uint32).reshape(-1, 3)
    cnt = np.asarray(counts, np.uint64)
    offs = np.zeros(len(cnt) + 1, np.uint64)
    offs[1:] = np.cumsum(cnt, dtype=np.uint64)
    attrs = np.ascontiguousarray(attributes, np.float32)
    attrs = attrs.reshape(len(attrs), -1)
    out = np.zeros((len(cnt), attrs.shape[1]), np.float32)
    lib().lyon_oracle_interpolate_fill(_ptr(src), _ptr(offs), len(cnt), _ptr(attrs),
                                       attrs.shape[1], _ptr(out))
    return out


def batch_fill_sources(pb, options_records: np.ndarray, index_bits: int = 32,
                       num_threads: int = 1):
    """Fills every path of a PathBatch with the oracle, recording each vertex's sources
    ((S, 3) words, ids indexing the batch's points) and the number per vertex."""
    L = lib()
    n = pb.num_paths
    cb = _CBatch(_ptr(pb.verbs), _ptr(pb.points), _ptr(pb.verb_offsets),
                 _ptr(pb.point_offsets), n)
    opts = np.ascontiguousarray(options_records)
    vc = np.zeros(n, np.uint32)
    ic = np.zeros(n, np.uint32)
    sc = np.zeros(n, np.uint32)
    st = np.zeros(n, np.int32)
    L.lyon_oracle_batch_fill_sources(ctypes.byref(cb), _ptr(opts), len(opts), index_bits,
                                     num_threads, _ptr(vc), _ptr(ic), _ptr(sc), _ptr(st), None,
                                     None, None, None, None, None, None)
    offs = []
    for c in (vc, ic, sc):
        o = np.zeros(n + 1, np.uint64)
        o[1:] = np.cumsum(c, dtype=np.uint64)
        offs.append(o)
    vo, io, so = offs
    verts = np.zeros((int(vo[-1]), 2), np.float32)
    idx = np.zeros(int(io[-1]), np.uint32)
    srcs = np.zeros((int(so[-1]), 3), np.uint32)
    counts = np.zeros(int(vo[-1]), np.uint32)
    t0 = time.perf_counter()
    L.lyon_oracle_batch_fill_sources(ctypes.byref(cb), _ptr(opts), len(opts), index_bits,
                                     num_threads, None, None, None, None, _ptr(verts), _ptr(idx),
                                     _ptr(srcs), _ptr(counts), _ptr(vo), _ptr(io), _ptr(so))
    return {"vtx_counts": vc, "idx_counts": ic, "src_counts": sc, "status": st,
            "vertices": verts, "indices": idx, "sources": srcs, "source_counts": counts,
            "vtx_offsets": vo, "idx_offsets": io, "src_offsets": so,
            "output_pass_s": time.perf_counter() - t0}


def flatten(path, tolerance: float):
    """path.iter().flattened(tol): (per-verb counts, points)."""
    L = lib()
    v = np.ascontiguousarray(path.verbs, dtype=np.uint8)
    p = np.ascontiguousarray(path.points, dtype=np.float32)
    counts = np.zeros(max(len(v), 1), dtype=np.uint32)
    n = L.lyon_oracle_flatten_path(_ptr(v), len(v), _ptr(p), len(p), tolerance, _ptr(counts),
                                   None, 0)
    pts = np.zeros((max(n, 1), 2), dtype=np.float32)
    L.lyon_oracle_flatten_path(_ptr(v), len(v), _ptr(p), len(p), tolerance, _ptr(counts),
                               _ptr(pts), n)
    return counts[:len(v)], pts[:n]


def wang(points, tolerance: float) -> float:
    a = np.ascontiguousarray(np.asarray(points, dtype=np.float32).reshape(-1))
    return float(lib().lyon_oracle_wang(_ptr(a), len(a) // 2, tolerance))


class _CBatch(ctypes.Structure):
    _fields_ = [("verbs", ctypes.c_void_p), ("points", ctypes.c_void_p),
                ("verb_offsets", ctypes.c_void_p), ("point_offsets", ctypes.c_void_p),
                ("num_paths", ctypes.c_uint32)]


def interpolate_attributes_threads(sources: np.ndarray, attributes: np.ndarray,
                                   num_threads: int = 1) -> np.ndarray:
    """interpolate_attributes in C on `num_threads` threads (the CPU baseline's version)."""
    src = np.ascontiguousarray(sources, np.uint32).reshape(-1, 3)
    attrs = np.ascontiguousarray(attributes, np.float32)
    attrs = attrs.reshape(len(attrs), -1)
    out = np.zeros((len(src), attrs.shape[1]), np.float32)
    lib().lyon_oracle_interpolate(_ptr(src), len(src), _ptr(attrs), attrs.shape[1], _ptr(out),
                                  num_threads)
    return out


def batch_stroke_sources(pb, options_records: np.ndarray, index_bits: int = 32,
                         num_threads: int = 1, widths=None, want_attributes: bool = False):
    """Strokes every path of a PathBatch with the oracle, recording each vertex's
    VertexSource ((V, 3) words, endpoint ids indexing the batch's points) next to the outputs
    `batch` returns."""
    L = lib()
    n = pb.num_paths
    cb = _CBatch(_ptr(pb.verbs), _ptr(pb.points), _ptr(pb.verb_offsets),
                 _ptr(pb.point_offsets), n)
    opts = np.ascontiguousarray(options_records)
    w = None
    if widths is not None:
        w = np.ascontiguousarray(widths, dtype=np.float32)
        assert len(w) == len(pb.points)
    vc = np.zeros(n, np.uint32)
    ic = np.zeros(n, np.uint32)
    st = np.zeros(n, np.int32)
    L.lyon_oracle_batch_stroke_sources(ctypes.byref(cb), _ptr(w), _ptr(opts), len(opts),
                                       index_bits, num_threads, _ptr(vc), _ptr(ic), _ptr(st),
                                       None, None, None, None, None, None)
    vo = np.zeros(n + 1, np.uint64)
    io = np.zeros(n + 1, np.uint64)
    vo[1:] = np.cumsum(vc, dtype=np.uint64)
    io[1:] = np.cumsum(ic, dtype=np.uint64)
    verts = np.zeros((int(vo[-1]), 2), np.float32)
    idx = np.zeros(int(io[-1]), np.uint32)
    attrs = np.zeros((int(vo[-1]), 4), np.uint32) if want_attributes else None
    srcs = np.zeros((int(vo[-1]), 3), np.uint32)
    t0 = time.perf_counter()
    L.lyon_oracle_batch_stroke_sources(ctypes.byref(cb), _ptr(w), _ptr(opts), len(opts),
                                       index_bits, num_threads, None, None, None, _ptr(verts),
                                       _ptr(idx), _ptr(vo), _ptr(io), _ptr(attrs), _ptr(srcs))
    res = {"vtx_counts": vc, "idx_counts": ic, "status": st, "vertices": verts, "indices": idx,
           "vtx_offsets": vo, "idx_offsets": io, "sources": srcs,
           "output_pass_s": time.perf_counter() - t0}
    if want_attributes:
        res["attributes"] = attrs
    return res


def batch(kind: str, pb, options_records: np.ndarray, index_bits: int = 32,
          num_threads: int = 1, want_output: bool = True, want_attributes: bool = False,
          widths=None):
    """Tessellates every path of a PathBatch with the oracle (per-path buffers).

    Returns dict with per-path vertex/index counts, statuses, near-tie counts and, when
    `want_output`, the concatenated outputs with per-path offsets (and, for strokes with
    `want_attributes`, the (V, 4) vertex attribute words of `Result.attributes`)."""
    L = lib()
    n = pb.num_paths
    cb = _CBatch(_ptr(pb.verbs), _ptr(pb.points), _ptr(pb.verb_offsets),
                 _ptr(pb.point_offsets), n)
    opts = np.ascontiguousarray(options_records)
    vc = np.zeros(n, np.uint32)
    ic = np.zeros(n, np.uint32)
    st = np.zeros(n, np.int32)
    nt = np.zeros(n, np.uint32)
    k = 0 if kind == "stroke" else 1
    if widths is not None:
        # Variable line width: one factor per point of the batch.
        assert kind == "stroke"
        w = np.ascontiguousarray(widths, dtype=np.float32)
        assert len(w) == len(pb.points)
        L.lyon_oracle_batch_stroke_vw(ctypes.byref(cb), _ptr(w), _ptr(opts), len(opts),
                                      index_bits, num_threads, _ptr(vc), _ptr(ic), _ptr(st),
                                      _ptr(nt), None, None, None, None, None)
        res = {"vtx_counts": vc, "idx_counts": ic, "status": st, "near_ties": nt}
        if want_output:
            vo = np.zeros(n + 1, np.uint64)
            io = np.zeros(n + 1, np.uint64)
            vo[1:] = np.cumsum(vc, dtype=np.uint64)
            io[1:] = np.cumsum(ic, dtype=np.uint64)
            verts = np.zeros((int(vo[-1]), 2), np.float32)
            idx = np.zeros(int(io[-1]), np.uint32)
            attrs = np.zeros((int(vo[-1]), 4), np.uint32) if want_attributes else None
            L.lyon_oracle_batch_stroke_vw(ctypes.byref(cb), _ptr(w), _ptr(opts), len(opts),
                                          index_bits, num_threads, None, None, None, None,
                                          _ptr(verts), _ptr(idx), _ptr(vo), _ptr(io), _ptr(attrs))
            res.update(vertices=verts, indices=idx, vtx_offsets=vo, idx_offsets=io)
            if want_attributes:
                res["attributes"] = attrs
        return res
    L.lyon_oracle_batch(k, ctypes.byref(cb), _ptr(opts), len(opts), index_bits, num_threads,
                        _ptr(vc), _ptr(ic), _ptr(st), _ptr(nt), None, None, None, None)
    res = {"vtx_counts": vc, "idx_counts": ic, "status": st, "near_ties": nt}
    if want_output:
        vo = np.zeros(n + 1, np.uint64)
        io = np.zeros(n + 1, np.uint64)
        vo[1:] = np.cumsum(vc, dtype=np.uint64)
        io[1:] = np.cumsum(ic, dtype=np.uint64)
        verts = np.zeros((int(vo[-1]), 2), np.float32)
        idx = np.zeros(int(io[-1]), np.uint32)
        L.lyon_oracle_batch(k, ctypes.byref(cb), _ptr(opts), len(opts), index_bits, num_threads,
                            None, None, None, None, _ptr(verts), _ptr(idx), _ptr(vo), _ptr(io))
        res.update(vertices=verts, indices=idx, vtx_offsets=vo, idx_offsets=io)
        if want_attributes and kind == "stroke":
            attrs = np.zeros((int(vo[-1]), 4), np.uint32)
            L.lyon_oracle_batch_stroke_attributes(ctypes.byref(cb), _ptr(opts), len(opts),
                                                  num_threads, _ptr(vo), _ptr(attrs))
            res["attributes"] = attrs
    return res


ARC_DTYPE = np.dtype([("center_x", "<f4"), ("center_y", "<f4"), ("radius_x", "<f4"),
                      ("radius_y", "<f4"), ("start_angle", "<f4"), ("sweep_angle", "<f4"),
                      ("x_rotation", "<f4")])


def flatten_arcs(arcs: np.ndarray, tolerance: float):
    """Arc::for_each_flattened_with_t (crates/geom/src/arc.rs:339-367) for every arc (an
    ARC_DTYPE array): (points (P, 2), t (P,), offsets (n + 1,), status (n,)); each arc's points
    start with its start point."""
    L = lib()
    a = np.ascontiguousarray(arcs).view(np.float32).reshape(-1, 7)
    n = len(a)
    counts = np.zeros(n, np.uint32)
    st = np.zeros(n, np.int32)
    L.lyon_oracle_flatten_arcs(_ptr(a), n, tolerance, _ptr(counts), _ptr(st), None, None, None)
    offs = np.zeros(n + 1, np.uint64)
    offs[1:] = np.cumsum(counts, dtype=np.uint64)
    pts = np.zeros((int(offs[-1]), 2), np.float32)
    ts = np.zeros(int(offs[-1]), np.float32)
    L.lyon_oracle_flatten_arcs(_ptr(a), n, tolerance, None, None, _ptr(offs), _ptr(pts),
                               _ptr(ts))
    return pts, ts, offs, st


HATCH_SEGMENT_DTYPE = np.dtype([("a_x", "<f4"), ("a_y", "<f4"), ("a_tangent_x", "<f4"),
                                ("a_tangent_y", "<f4"), ("a_u", "<f4"), ("b_x", "<f4"),
                                ("b_y", "<f4"), ("b_tangent_x", "<f4"), ("b_tangent_y", "<f4"),
                                ("b_u", "<f4"), ("row", "<u4"), ("v", "<f4")])
DOT_DTYPE = np.dtype([("x", "<f4"), ("y", "<f4"), ("u", "<f4"), ("v", "<f4"), ("column", "<u4"),
                      ("row", "<u4")])


def hatch(pb, params):
    """Hatcher::hatch_path / dot_path (crates/algorithms/src/hatching.rs) over a PathBatch.
    `params`: 11 floats (see lyon_oracle_hatch). Returns (records, offsets, status)."""
    L = lib()
    n = pb.num_paths
    cb = _CBatch(_ptr(pb.verbs), _ptr(pb.points), _ptr(pb.verb_offsets),
                 _ptr(pb.point_offsets), n)
    prm = np.ascontiguousarray(params, np.float32)
    counts = np.zeros(n, np.uint32)
    st = np.zeros(n, np.int32)
    L.lyon_oracle_hatch(ctypes.byref(cb), _ptr(prm), _ptr(counts), _ptr(st), None, None)
    offs = np.zeros(n + 1, np.uint64)
    offs[1:] = np.cumsum(counts, dtype=np.uint64)
    dt = DOT_DTYPE if prm[9] != 0 else HATCH_SEGMENT_DTYPE
    out = np.zeros(int(offs[-1]), dt)
    L.lyon_oracle_hatch(ctypes.byref(cb), _ptr(prm), None, None, _ptr(offs),
                        out.ctypes.data_as(ctypes.c_void_p) if len(out) else None)
    return out, offs, st
