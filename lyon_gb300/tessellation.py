"""Host-side mirror of lyon's tessellation API over the CUDA library.

Mirrors (names, argument meaning, error behaviour):
  StrokeTessellator.tessellate_path(path, options, builder)  crates/tessellation/src/stroke.rs:164-177
  FillTessellator.tessellate_path(path, options, builder)    crates/tessellation/src/fill.rs:628-641
  VertexBuffers / BuffersBuilder (append, vertex offset, abort on error)
                                           crates/tessellation/src/geometry_builder.rs:262-351,451-508
  TessellationError / GeometryBuilderError / InternalError   crates/tessellation/src/error.rs:1-142
plus the batched `tessellate_paths` the reference has no counterpart for.

Every call goes to liblyon_gb300.so (lyon_gb300/_native.py); there is no CPU path.
"""

from __future__ import annotations

import ctypes
import threading
from dataclasses import dataclass
from typing import Optional

import numpy as np

from . import _native
from .options import (FILL_OPTIONS_DTYPE, STROKE_OPTIONS_DTYPE, FillOptions, StrokeOptions)
from .path import Path, PathBatch, PathBuilder

LYON_OK = 0
LYON_ERR_POSITION_IS_NAN = 1
LYON_ERR_TOLERANCE_IS_NAN = 2
LYON_ERR_TOO_MANY_VERTICES = 3
LYON_ERR_INVALID_VERTEX = 4
LYON_ERR_INTERNAL = 5
LYON_ERR_INVALID_ARGUMENT = 100
LYON_ERR_CUDA = 101
LYON_ERR_OUT_OF_MEMORY = 102
LYON_ERR_CAPACITY = 103
LYON_ERR_UNSUPPORTED = 104

INDEX_GLOBAL = 0
INDEX_PER_PATH = 1

# lyon_stroke_vertex: the StrokeVertex attributes a vertex constructor reads
# (crates/tessellation/src/stroke.rs:2667-2720); side 0 = Positive, 1 = Negative.
STROKE_VERTEX_DTYPE = np.dtype([("x", "<f4"), ("y", "<f4"), ("normal_x", "<f4"),
                                ("normal_y", "<f4"), ("advancement", "<f4"), ("side", "<u4")])

_ERROR_NAMES = {
    LYON_ERR_POSITION_IS_NAN: "UnsupportedParamater(PositionIsNaN)",
    LYON_ERR_TOLERANCE_IS_NAN: "UnsupportedParamater(ToleranceIsNaN)",
    LYON_ERR_TOO_MANY_VERTICES: "GeometryBuilder(TooManyVertices)",
    LYON_ERR_INVALID_VERTEX: "GeometryBuilder(InvalidVertex)",
    LYON_ERR_INTERNAL: "Internal",
    LYON_ERR_INVALID_ARGUMENT: "InvalidArgument",
    LYON_ERR_CUDA: "Cuda",
    LYON_ERR_OUT_OF_MEMORY: "OutOfMemory",
    LYON_ERR_CAPACITY: "Capacity",
    LYON_ERR_UNSUPPORTED: "Unsupported",
}


class TessellationError(Exception):
    """lyon's TessellationError; `code` is the C ABI status."""

    def __init__(self, code: int, detail: str = ""):
        self.code = code
        name = _ERROR_NAMES.get(code, f"status {code}")
        super().__init__(f"{name}{': ' + detail if detail else ''}")


class VertexBuffers:
    """`VertexBuffers<Point, u16|u32>`: positions (N x 2 f32) and indices."""

    def __init__(self, index_bits: int = 16):
        assert index_bits in (16, 32)
        self.index_bits = index_bits
        self.vertices = np.zeros((0, 2), dtype=np.float32)
        self.indices = np.zeros(0, dtype=np.uint16 if index_bits == 16 else np.uint32)

    def clear(self):
        self.vertices = self.vertices[:0]
        self.indices = self.indices[:0]


class BuffersBuilder:
    """`BuffersBuilder::new(&mut buffers, ctor)` with an optional vertex offset.

    Without `vertex_ctor` the vertices are positions (lyon's `Positions` constructor). With it,
    a stroke hands the constructor every vertex as a STROKE_VERTEX_DTYPE record array (position,
    normal, advancement, side: what lyon's StrokeVertex exposes) and a fill hands it the (N, 2)
    positions; the constructor returns one output row per vertex (vectorised, where lyon calls
    it once per vertex)."""

    def __init__(self, buffers: VertexBuffers, vertex_offset: int = 0, vertex_ctor=None):
        self.buffers = buffers
        self.vertex_offset = vertex_offset
        self.vertex_ctor = vertex_ctor
        # Fills with custom attributes: every vertex's sources, (S, 3) u32 words (from, to, t
        # bits), which the fill vertex records index (src_first, src_count).
        self.sources = np.zeros((0, 3), np.uint32)

    def with_vertex_offset(self, offset: int) -> "BuffersBuilder":
        self.vertex_offset = offset
        return self

    def next_index(self) -> int:
        return len(self.buffers.vertices) + self.vertex_offset

    def append(self, vertices: np.ndarray, indices: np.ndarray) -> None:
        b = self.buffers
        if self.vertex_ctor is not None:
            made = np.asarray(self.vertex_ctor(vertices))
            b.vertices = made.copy() if len(b.vertices) == 0 else np.concatenate([b.vertices, made])
        else:
            b.vertices = np.concatenate([b.vertices, vertices.reshape(-1, 2)])
        b.indices = np.concatenate([b.indices, indices.astype(b.indices.dtype)])


def simple_builder(buffers: VertexBuffers) -> BuffersBuilder:
    return BuffersBuilder(buffers)


class Context:
    """A `lyon_gpu_context` (device, stream, arenas)."""

    _default: Optional["Context"] = None
    _lock = threading.Lock()

    def __init__(self, device: int = 0):
        self.lib = _native.load()
        self.device = device
        self.h = self.lib.lyon_gpu_create(device)
        if not self.h:
            raise RuntimeError(f"lyon_gpu_create({device}) failed (no CUDA device?)")

    @classmethod
    def default(cls) -> "Context":
        with cls._lock:
            if cls._default is None:
                cls._default = Context(0)
            return cls._default

    def close(self):
        if self.h:
            self.lib.lyon_gpu_destroy(self.h)
            self.h = None

    def last_error(self) -> str:
        return self.lib.lyon_gpu_last_error(self.h).decode()

    def synchronize(self):
        r = self.lib.lyon_gpu_synchronize(self.h)
        if r != LYON_OK:
            raise TessellationError(r, self.last_error())

    @property
    def stream(self) -> int:
        return int(self.lib.lyon_gpu_stream(self.h) or 0)


class HostBuffer:
    """Page-locked host memory backed by huge pages (lyon_gpu_host_alloc), for the host-buffer
    calls' inputs and outputs: large outputs copy out at the link's rate into it, about twice
    the rate into ordinary pinned memory on a GB300. `array(dtype, count)` views it as numpy."""

    def __init__(self, nbytes: int):
        self.lib = _native.load()
        self.nbytes = int(nbytes)
        self.ptr = self.lib.lyon_gpu_host_alloc(max(self.nbytes, 1))
        if not self.ptr:
            raise MemoryError(f"lyon_gpu_host_alloc({self.nbytes}) failed")

    def array(self, dtype, count: Optional[int] = None) -> np.ndarray:
        dtype = np.dtype(dtype)
        n = self.nbytes // dtype.itemsize if count is None else int(count)
        if n * dtype.itemsize > self.nbytes:
            raise ValueError("view larger than the buffer")
        raw = (ctypes.c_char * (n * dtype.itemsize)).from_address(self.ptr)
        return np.frombuffer(raw, dtype=dtype, count=n)

    def close(self) -> None:
        if self.ptr:
            self.lib.lyon_gpu_host_free(self.ptr)
            self.ptr = None

    def __del__(self):
        try:
            self.close()
        except Exception:  # noqa: BLE001
            pass


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.c_void_p) if a is not None and a.size else None


def custom_vertex_dtype(num_attributes: int) -> np.dtype:
    """What the vertex constructor receives for a path with custom attributes: the
    lyon_stroke_vertex fields, the vertex's source (StrokeVertex::source: `src_to` is
    NO_ENDPOINT for an endpoint) and its interpolated attributes
    (StrokeVertex::interpolated_attributes)."""
    fields = list(STROKE_VERTEX_DTYPE.descr) + [("src_from", "<u4"), ("src_to", "<u4"),
                                                 ("src_t", "<f4")]
    if num_attributes:
        fields.append(("attributes", "<f4", (num_attributes,)))
    return np.dtype(fields)


NO_ENDPOINT = 0xFFFFFFFF


def _single_custom(ctx: Context, path: Path, options, builder: BuffersBuilder,
                   attributes) -> None:
    """One path with custom endpoint attributes (lyon_gpu_stroke_path_custom)."""
    bits = builder.buffers.index_bits
    verbs = np.ascontiguousarray(path.verbs, dtype=np.uint8)
    pts = np.ascontiguousarray(path.points, dtype=np.float32)
    attrs = np.ascontiguousarray(attributes, dtype=np.float32)
    attrs = attrs.reshape(len(pts), -1) if attrs.size else np.zeros((len(pts), 0), np.float32)
    if attrs.shape[0] != len(pts):
        raise ValueError("one attribute row per point")
    na = attrs.shape[1]
    wa = -1 if options.variable_line_width is None else int(options.variable_line_width)
    opt = options.to_c()
    res = _native.CResult()
    src_p = ctypes.c_void_p()
    att_p = ctypes.c_void_p()
    records = builder.vertex_ctor is not None
    r = ctx.lib.lyon_gpu_stroke_path_custom(
        ctx.h, _ptr(verbs), len(verbs), _ptr(pts), len(pts), _ptr(attrs), na, wa,
        ctypes.byref(opt), bits, builder.next_index(), 1 if records else 0, ctypes.byref(res),
        ctypes.byref(src_p), ctypes.byref(att_p))
    if r != LYON_OK:
        raise TessellationError(r, ctx.last_error() if r >= 100 else "")
    nv, ni = res.num_vertices, res.num_indices
    ctype = ctypes.c_uint16 if bits == 16 else ctypes.c_uint32
    i = np.ctypeslib.as_array(ctypes.cast(res.indices, ctypes.POINTER(ctype)),
                              shape=(ni,)).copy() if ni else np.zeros(0, builder.buffers.indices.dtype)
    if not records:
        v = np.ctypeslib.as_array(ctypes.cast(res.vertices, ctypes.POINTER(ctypes.c_float)),
                                  shape=(nv * 2,)).copy() if nv else np.zeros(0, np.float32)
        builder.append(v.reshape(-1, 2), i)
        return
    out = np.zeros(nv, custom_vertex_dtype(na))
    if nv:
        raw = np.ctypeslib.as_array(ctypes.cast(res.vertices, ctypes.POINTER(ctypes.c_uint8)),
                                    shape=(nv * STROKE_VERTEX_DTYPE.itemsize,)).copy()
        rec = raw.view(STROKE_VERTEX_DTYPE)
        for f in STROKE_VERTEX_DTYPE.names:
            out[f] = rec[f]
        src = np.ctypeslib.as_array(ctypes.cast(src_p, ctypes.POINTER(ctypes.c_uint32)),
                                    shape=(nv * 3,)).copy().reshape(-1, 3)
        out["src_from"] = src[:, 0]
        out["src_to"] = src[:, 1]
        out["src_t"] = src[:, 2].view(np.float32)
        if na:
            out["attributes"] = np.ctypeslib.as_array(
                ctypes.cast(att_p, ctypes.POINTER(ctypes.c_float)), shape=(nv * na,)).copy(
                ).reshape(-1, na)
    builder.append(out, i)


def fill_vertex_dtype(num_attributes: int) -> np.dtype:
    """What the vertex constructor receives for a fill of a path with custom attributes: the
    position, the vertex's sources (FillVertex::sources) as a range of BuffersBuilder.sources,
    and its interpolated attributes (FillVertex::interpolated_attributes)."""
    fields = [("x", "<f4"), ("y", "<f4"), ("src_first", "<u8"), ("src_count", "<u4")]
    if num_attributes:
        fields.append(("attributes", "<f4", (num_attributes,)))
    return np.dtype(fields)


def _single_fill_custom(ctx: Context, path: Path, options, builder: BuffersBuilder,
                        attributes) -> None:
    """One path with custom endpoint attributes (lyon_gpu_fill_path_custom)."""
    bits = builder.buffers.index_bits
    verbs = np.ascontiguousarray(path.verbs, dtype=np.uint8)
    pts = np.ascontiguousarray(path.points, dtype=np.float32)
    attrs = np.ascontiguousarray(attributes, dtype=np.float32)
    attrs = attrs.reshape(len(pts), -1) if attrs.size else np.zeros((len(pts), 0), np.float32)
    if attrs.shape[0] != len(pts):
        raise ValueError("one attribute row per point")
    na = attrs.shape[1]
    opt = options.to_c()
    res = _native.CResult()
    src_p, off_p, att_p = ctypes.c_void_p(), ctypes.c_void_p(), ctypes.c_void_p()
    r = ctx.lib.lyon_gpu_fill_path_custom(
        ctx.h, _ptr(verbs), len(verbs), _ptr(pts), len(pts), _ptr(attrs), na, ctypes.byref(opt),
        bits, builder.next_index(), ctypes.byref(res), ctypes.byref(src_p), ctypes.byref(off_p),
        ctypes.byref(att_p))
    if r != LYON_OK:
        raise TessellationError(r, ctx.last_error() if r >= 100 else "")
    nv, ni = res.num_vertices, res.num_indices
    ctype = ctypes.c_uint16 if bits == 16 else ctypes.c_uint32
    i = np.ctypeslib.as_array(ctypes.cast(res.indices, ctypes.POINTER(ctype)),
                              shape=(ni,)).copy() if ni else np.zeros(0, builder.buffers.indices.dtype)
    v = np.ctypeslib.as_array(ctypes.cast(res.vertices, ctypes.POINTER(ctypes.c_float)),
                              shape=(nv * 2,)).copy().reshape(-1, 2) if nv else np.zeros((0, 2),
                                                                                       np.float32)
    if builder.vertex_ctor is None:
        builder.append(v, i)
        return
    offs = np.ctypeslib.as_array(ctypes.cast(off_p, ctypes.POINTER(ctypes.c_uint64)),
                                 shape=(nv + 1,)).copy() if nv else np.zeros(1, np.uint64)
    ns = int(offs[-1])
    src = np.ctypeslib.as_array(ctypes.cast(src_p, ctypes.POINTER(ctypes.c_uint32)),
                                shape=(ns * 3,)).copy().reshape(-1, 3) if ns else np.zeros(
        (0, 3), np.uint32)
    out = np.zeros(nv, fill_vertex_dtype(na))
    out["x"] = v[:, 0]
    out["y"] = v[:, 1]
    out["src_first"] = offs[:-1] + len(builder.sources)
    out["src_count"] = np.diff(offs)
    if na and nv:
        out["attributes"] = np.ctypeslib.as_array(
            ctypes.cast(att_p, ctypes.POINTER(ctypes.c_float)), shape=(nv * na,)).copy(
            ).reshape(-1, na)
    builder.sources = np.concatenate([builder.sources, src])
    builder.append(out, i)


def _single(kind: str, ctx: Context, path: Path, options, builder: BuffersBuilder,
            widths=None) -> None:
    bits = builder.buffers.index_bits
    verbs = np.ascontiguousarray(path.verbs, dtype=np.uint8)
    pts = np.ascontiguousarray(path.points, dtype=np.float32)
    opt = options.to_c()
    res = _native.CResult()
    records = kind == "stroke" and builder.vertex_ctor is not None
    if widths is not None:
        w = np.ascontiguousarray(widths, dtype=np.float32)
        if len(w) != len(pts):
            raise ValueError("one width factor per point")
        r = ctx.lib.lyon_gpu_stroke_path_variable_width(
            ctx.h, _ptr(verbs), len(verbs), _ptr(pts), len(pts), _ptr(w), ctypes.byref(opt), bits,
            builder.next_index(), 1 if records else 0, ctypes.byref(res))
    else:
        if records:
            fn = ctx.lib.lyon_gpu_stroke_path_attributes
        else:
            fn = ctx.lib.lyon_gpu_stroke_path if kind == "stroke" else ctx.lib.lyon_gpu_fill_path
        r = fn(ctx.h, _ptr(verbs), len(verbs), _ptr(pts), len(pts), ctypes.byref(opt), bits,
               builder.next_index(), ctypes.byref(res))
    if r != LYON_OK:
        raise TessellationError(r, ctx.last_error() if r >= 100 else "")
    nv, ni = res.num_vertices, res.num_indices
    if records:
        raw = np.ctypeslib.as_array(ctypes.cast(res.vertices, ctypes.POINTER(ctypes.c_uint8)),
                                    shape=(nv * STROKE_VERTEX_DTYPE.itemsize,)).copy() \
            if nv else np.zeros(0, np.uint8)
        v = raw.view(STROKE_VERTEX_DTYPE)
        ctype = ctypes.c_uint16 if bits == 16 else ctypes.c_uint32
        i = np.ctypeslib.as_array(ctypes.cast(res.indices, ctypes.POINTER(ctype)),
                                  shape=(ni,)).copy() if ni else np.zeros(0, builder.buffers.indices.dtype)
        builder.append(v, i)
        return
    v = np.ctypeslib.as_array(ctypes.cast(res.vertices, ctypes.POINTER(ctypes.c_float)),
                              shape=(nv * 2,)).copy() if nv else np.zeros(0, np.float32)
    ctype = ctypes.c_uint16 if bits == 16 else ctypes.c_uint32
    i = np.ctypeslib.as_array(ctypes.cast(res.indices, ctypes.POINTER(ctype)),
                              shape=(ni,)).copy() if ni else np.zeros(0, builder.buffers.indices.dtype)
    builder.append(v.reshape(-1, 2), i)


def _append_result(res: "BatchResult", builder: BuffersBuilder) -> None:
    import torch  # noqa: F401  (device copies)
    if res.num_failed_paths:
        st = int(res.statuses().cpu().numpy()[0])
        raise TessellationError(st)
    v = res.vertices().cpu().numpy() if res.total_vertices else np.zeros((0, 2), np.float32)
    if res.total_indices:
        i = res.indices().cpu().numpy()
        i = i.view(np.uint16) if res.index_bits == 16 else i.view(np.uint32)
    else:
        i = np.zeros(0, builder.buffers.indices.dtype)
    builder.append(v.reshape(-1, 2), i)


def fill_shapes(kind: int, params_dev, num_shapes: int, options_dev=None, num_options: int = 0,
                index_bits: int = 32, index_mode: int = INDEX_GLOBAL, vertex_offset: int = 0,
                ctx: Optional[Context] = None) -> "BatchResult":
    """Batched basic shapes (lyon_gpu_fill_shapes): SHAPE_RECTANGLE params are (min x, min y,
    max x, max y) per shape, SHAPE_CIRCLE (center x, center y, radius); device tensors."""
    ctx = ctx or Context.default()
    out = _native.CBatchOutput()
    r = ctx.lib.lyon_gpu_fill_shapes(ctx.h, kind, params_dev.data_ptr() if num_shapes else None,
                                     num_shapes,
                                     options_dev.data_ptr() if options_dev is not None else None,
                                     num_options, index_bits, index_mode, vertex_offset,
                                     ctypes.byref(out))
    if r != LYON_OK:
        raise TessellationError(r, ctx.last_error())
    return BatchResult(r, int(out.total_vertices), int(out.total_indices),
                       int(out.num_failed_paths), int(out.vertices or 0), int(out.indices or 0),
                       int(out.status or 0), index_bits, num_shapes,
                       int(out.vertex_offsets or 0), int(out.index_offsets or 0))


SHAPE_RECTANGLE = 0
SHAPE_CIRCLE = 1

# lyon_arc (lyon_geom::Arc, crates/geom/src/arc.rs:21-28), angles in radians.
ARC_DTYPE = np.dtype([("center_x", "<f4"), ("center_y", "<f4"), ("radius_x", "<f4"),
                      ("radius_y", "<f4"), ("start_angle", "<f4"), ("sweep_angle", "<f4"),
                      ("x_rotation", "<f4")])


@dataclass
class ArcFlattening:
    """Device tensors of lyon_gpu_flatten_arcs (owned by the context until its next call):
    arc i's points are points[offsets[i]:offsets[i + 1]] (its start point first)."""
    points: object   # (P, 2) f32
    t: object        # (P,) f32
    offsets: object  # (n + 1,) int64
    status: object   # (n,) int32
    total_points: int


def flatten_arcs(arcs_dev, num_arcs: int, tolerance: float,
                 ctx: Optional[Context] = None) -> ArcFlattening:
    """Arc::for_each_flattened_with_t (crates/geom/src/arc.rs:339-367) for `num_arcs` arcs in
    a device tensor of ARC_DTYPE records (7 f32 each)."""
    import torch
    ctx = ctx or Context.default()
    out = _native.CArcOutput()
    r = ctx.lib.lyon_gpu_flatten_arcs(ctx.h, arcs_dev.data_ptr() if num_arcs else None,
                                      num_arcs, tolerance, ctypes.byref(out))
    if r != LYON_OK:
        raise TessellationError(r, ctx.last_error())
    tp = int(out.total_points)

    def dev(ptr, shape, ts):
        return torch.as_tensor(_CudaArray(int(ptr or 0), shape, ts), device="cuda")
    return ArcFlattening(dev(out.points, (tp, 2), "<f4"), dev(out.t, (tp,), "<f4"),
                         dev(out.offsets, (num_arcs + 1,), "<i8"),
                         dev(out.status, (num_arcs,), "<i4"), tp)


class DeferredTessellator:
    """Collects `tessellate_path` calls (strokes with fixed width and fills, `Positions`
    vertices) and runs each kind as one batched launch at `flush()`. Each call's builder then
    receives what lyon's `tessellate_path` would have appended (stroke.rs:164-177,
    fill.rs:628-641), in call order: ids count from the builder's next index, and a call whose
    last id would pass the index type's range fails with TooManyVertices and appends nothing
    (geometry_builder.rs:338-350, 478-481), so several calls into one BuffersBuilder give what
    the same calls in sequence give. The launch and synchronisation cost of a GPU call is paid
    once per flush instead of once per path."""

    def __init__(self, ctx: Optional[Context] = None):
        self.ctx = ctx or Context.default()
        self._calls = []  # (kind, path, options, builder)

    def stroke(self, path: Path, options: StrokeOptions, builder: BuffersBuilder) -> int:
        if builder.vertex_ctor is not None or options.variable_line_width is not None:
            raise ValueError("deferred calls write positions with a fixed line width")
        self._calls.append(("stroke", path, options, builder))
        return len(self._calls) - 1

    def fill(self, path: Path, options: FillOptions, builder: BuffersBuilder) -> int:
        if builder.vertex_ctor is not None:
            raise ValueError("deferred calls write positions")
        self._calls.append(("fill", path, options, builder))
        return len(self._calls) - 1

    def flush(self):
        """Runs the pending calls; returns, per call in order, None or its TessellationError."""
        calls, self._calls = self._calls, []
        results = {}
        for kind in ("stroke", "fill"):
            idx = [k for k, c in enumerate(calls) if c[0] == kind]
            if not idx:
                continue
            batch = PathBatch.from_paths([calls[k][1] for k in idx])
            recs = np.concatenate([calls[k][2].to_record() for k in idx])
            db = DeviceBatch.upload(batch, self.ctx.device)
            od = upload_options(recs, self.ctx.device)
            res = tessellate_paths(kind, db, od, len(recs), 32, INDEX_PER_PATH, 0, self.ctx)
            self.ctx.synchronize()
            v = res.vertices().cpu().numpy() if res.total_vertices else np.zeros((0, 2), np.float32)
            i = (res.indices().cpu().numpy().view(np.uint32) if res.total_indices
                 else np.zeros(0, np.uint32))
            st = res.statuses().cpu().numpy()
            vo, io = res.offsets()
            vo, io = vo.cpu().numpy(), io.cpu().numpy()
            for j, k in enumerate(idx):
                results[k] = (int(st[j]), v[vo[j]:vo[j + 1]], i[io[j]:io[j + 1]])
        out = []
        for k, (kind, path, options, builder) in enumerate(calls):
            status, v, i = results[k]
            if status == LYON_OK:
                base = builder.next_index()
                top = 65535 if builder.buffers.index_bits == 16 else 0xFFFFFFFE
                if len(v) > 0 and base + len(v) - 1 > top:
                    status = LYON_ERR_TOO_MANY_VERTICES
                else:
                    builder.append(v, (i.astype(np.uint64) + base).astype(
                        builder.buffers.indices.dtype))
            out.append(None if status == LYON_OK else TessellationError(status))
        return out


class StrokeTessellator:
    """lyon's StrokeTessellator (fixed line width, `Positions` vertices)."""

    def __init__(self, ctx: Optional[Context] = None):
        self.ctx = ctx or Context.default()

    def tessellate_path(self, path: Path, options: StrokeOptions, builder: BuffersBuilder,
                        widths=None, attributes=None) -> None:
        """`attributes`: the path's custom endpoint attributes, (num_points, A) f32 (rows of
        control points and of Close's repeated point are not read), as lyon's Path built with
        attributes carries them (stroke.rs:164-177 then takes tessellate_with_ids): the vertex
        constructor then receives `custom_vertex_dtype(A)` records, and
        `options.variable_line_width` names the attribute that scales the width.
        `widths`: one width factor per point for a variable width without other attributes;
        neither strokes with the fixed width."""
        if attributes is not None:
            _single_custom(self.ctx, path, options, builder, attributes)
            return
        if options.variable_line_width is not None and widths is None:
            # stroke.rs:127-131: a variable width needs the attributes to read it from.
            raise ValueError("variable line width requires custom attributes")
        _single("stroke", self.ctx, path, options, builder, widths)

    def tessellate_ellipse(self, center, radii, x_rotation: float, winding: int,
                           options: StrokeOptions, builder: BuffersBuilder) -> None:
        """stroke.rs:294-307: the path builder's ellipse (quadratic arcs), stroked."""
        b = PathBuilder()
        b.add_ellipse(center, radii, x_rotation, winding)
        self.tessellate_path(b.build(), options, builder)

    def tessellate_polygon(self, points, closed: bool, options: StrokeOptions,
                           builder: BuffersBuilder) -> None:
        """stroke.rs:255-263."""
        b = PathBuilder()
        b.add_polygon(points, closed)
        self.tessellate_path(b.build(), options, builder)

    def tessellate_rectangle(self, rect, options: StrokeOptions, builder: BuffersBuilder) -> None:
        """stroke.rs:265-278: the rectangle as a path (Winding::Positive)."""
        b = PathBuilder()
        b.add_rectangle(rect, 1)
        self.tessellate_path(b.build(), options, builder)

    def tessellate_circle(self, center, radius: float, options: StrokeOptions,
                          builder: BuffersBuilder) -> None:
        """stroke.rs:280-292: the circle as a path of four cubics (Winding::Positive)."""
        b = PathBuilder()
        b.add_circle(center, radius, 1)
        self.tessellate_path(b.build(), options, builder)

    tessellate = tessellate_path


class FillTessellator:
    """lyon's FillTessellator (`Positions` vertices)."""

    def __init__(self, ctx: Optional[Context] = None):
        self.ctx = ctx or Context.default()

    def tessellate_ellipse(self, center, radii, x_rotation: float, winding: int,
                           options: FillOptions, builder: BuffersBuilder) -> None:
        """fill.rs:675-690: the path builder's ellipse, filled without intersection handling."""
        b = PathBuilder()
        b.add_ellipse(center, radii, x_rotation, winding)
        self.tessellate_path(b.build(), options.with_intersections(False), builder)

    def tessellate_polygon(self, points, closed: bool, options: FillOptions,
                           builder: BuffersBuilder) -> None:
        """fill.rs:643-651."""
        b = PathBuilder()
        b.add_polygon(points, closed)
        self.tessellate_path(b.build(), options, builder)

    def _shape(self, kind, params, options, builder):
        import torch
        p = torch.tensor(np.asarray(params, np.float32).reshape(-1), device="cuda")
        od = upload_options(options.to_record())
        res = fill_shapes(kind, p, 1, od, 1, builder.buffers.index_bits, INDEX_PER_PATH,
                          builder.next_index(), self.ctx)
        self.ctx.synchronize()
        _append_result(res, builder)

    def tessellate_rectangle(self, rect, options: FillOptions, builder: BuffersBuilder) -> None:
        """fill.rs:653-661 (basic_shapes.rs:12-38); rect = (min_x, min_y, max_x, max_y)."""
        self._shape(SHAPE_RECTANGLE, rect, options, builder)

    def tessellate_circle(self, center, radius: float, options: FillOptions,
                          builder: BuffersBuilder) -> None:
        """fill.rs:663-672 (basic_shapes.rs:40-124)."""
        self._shape(SHAPE_CIRCLE, [center[0], center[1], radius], options, builder)

    def tessellate_path(self, path: Path, options: FillOptions, builder: BuffersBuilder,
                        attributes=None) -> None:
        """`attributes`: the path's custom endpoint attributes, (num_points, A) f32 (fill.rs:
        636-640 then takes tessellate_with_ids): a vertex constructor receives
        `fill_vertex_dtype(A)` records whose sources are ranges of `builder.sources`."""
        if attributes is not None:
            _single_fill_custom(self.ctx, path, options, builder, attributes)
            return
        _single("fill", self.ctx, path, options, builder)

    tessellate = tessellate_path


# ---------------------------------------------------------------------------------------------
# Batched API over device memory.
# ---------------------------------------------------------------------------------------------

class _CudaArray:
    """A view of library-owned device memory for torch.as_tensor (__cuda_array_interface__)."""

    def __init__(self, ptr: int, shape, typestr: str):
        self.__cuda_array_interface__ = {"data": (int(ptr), False), "shape": tuple(shape),
                                         "typestr": typestr, "version": 3, "strides": None}


@dataclass
class DeviceBatch:
    """A PathBatch uploaded to the GPU (torch tensors keep the memory alive)."""

    verbs: object
    points: object
    verb_offsets: object
    point_offsets: object
    num_paths: int

    @staticmethod
    def upload(batch: PathBatch, device: int = 0) -> "DeviceBatch":
        import torch
        dev = torch.device("cuda", device)

        def up(a):
            t = torch.from_numpy(np.ascontiguousarray(a))
            return t.to(dev, non_blocking=False) if t.numel() else torch.zeros(1, dtype=t.dtype,
                                                                               device=dev)
        d = DeviceBatch(up(batch.verbs), up(batch.points.reshape(-1)), up(batch.verb_offsets),
                        up(batch.point_offsets), batch.num_paths)
        torch.cuda.synchronize(dev)
        return d

    def c(self) -> _native.CPathBatch:
        return _native.CPathBatch(self.verbs.data_ptr(), self.points.data_ptr(),
                                  self.verb_offsets.data_ptr(), self.point_offsets.data_ptr(),
                                  self.num_paths)


def upload_options(records: np.ndarray, device: int = 0):
    import torch
    raw = np.ascontiguousarray(records).view(np.uint8)
    t = torch.from_numpy(raw.copy()).to(torch.device("cuda", device))
    torch.cuda.synchronize()
    return t


@dataclass
class BatchResult:
    status: int
    total_vertices: int
    total_indices: int
    num_failed_paths: int
    vertices_ptr: int
    indices_ptr: int
    status_ptr: int
    index_bits: int
    num_paths: int
    vertex_offsets_ptr: int = 0
    index_offsets_ptr: int = 0
    vertex_floats: int = 2  # 6 when the vertices are lyon_stroke_vertex records
    sources_ptr: int = 0          # lyon_vertex_source records (custom-attribute calls)
    custom_attributes_ptr: int = 0
    num_attributes: int = 0
    source_offsets_ptr: int = 0   # fills: total_vertices + 1 u64 (vertex v's sources)
    total_sources: int = 0

    def offsets(self):
        """(vertex_offsets, index_offsets) as int64 torch tensors of num_paths + 1 entries."""
        import torch
        v = torch.as_tensor(_CudaArray(self.vertex_offsets_ptr, (self.num_paths + 1,), "<i8"),
                            device="cuda")
        i = torch.as_tensor(_CudaArray(self.index_offsets_ptr, (self.num_paths + 1,), "<i8"),
                            device="cuda")
        return v, i

    def vertices(self):
        """Positions, (V, 2) f32 (a strided view when the output holds records)."""
        import torch
        t = torch.as_tensor(_CudaArray(self.vertices_ptr, (self.total_vertices, self.vertex_floats),
                                       "<f4"), device="cuda")
        return t if self.vertex_floats == 2 else t[:, :2]

    def records(self):
        """lyon_stroke_vertex records as a (V, 6) f32 tensor (column 5 holds the side's u32
        bits); `.cpu().numpy().view(STROKE_VERTEX_DTYPE)` gives the structured records."""
        import torch
        assert self.vertex_floats == 6, "not an attribute output"
        return torch.as_tensor(_CudaArray(self.vertices_ptr, (self.total_vertices, 6), "<f4"),
                               device="cuda")

    def sources(self):
        """Each vertex's lyon_vertex_source as a (V, 3) int32 tensor (from, to, t's f32 bits;
        `to` == -1 for an endpoint)."""
        import torch
        assert self.sources_ptr, "not a custom-attribute output"
        n = self.total_sources if self.source_offsets_ptr else self.total_vertices
        return torch.as_tensor(_CudaArray(self.sources_ptr, (n, 3), "<i4"), device="cuda")

    def source_offsets(self):
        """Fills: vertex v's sources are sources()[offsets[v]:offsets[v + 1]] (int64)."""
        import torch
        assert self.source_offsets_ptr, "not a fill custom-attribute output"
        return torch.as_tensor(_CudaArray(self.source_offsets_ptr, (self.total_vertices + 1,),
                                          "<i8"), device="cuda")

    def custom_attributes(self):
        """Each vertex's interpolated custom attributes, (V, A) f32."""
        import torch
        assert self.custom_attributes_ptr, "no custom attributes"
        return torch.as_tensor(_CudaArray(self.custom_attributes_ptr,
                                          (self.total_vertices, self.num_attributes), "<f4"),
                               device="cuda")

    def indices(self):
        import torch
        ts = "<u2" if self.index_bits == 16 else "<u4"
        arr = _CudaArray(self.indices_ptr, (self.total_indices,), ts)
        if self.index_bits == 32:
            # torch has no uint32 view support everywhere: read as int32 with the same bits.
            arr.__cuda_array_interface__["typestr"] = "<i4"
        else:
            arr.__cuda_array_interface__["typestr"] = "<i2"
        return torch.as_tensor(arr, device="cuda")

    def statuses(self):
        import torch
        return torch.as_tensor(_CudaArray(self.status_ptr, (self.num_paths,), "<i4"),
                               device="cuda")


def tessellate_paths(kind: str, dbatch: DeviceBatch, options_dev, num_options: int,
                     index_bits: int = 32, index_mode: int = INDEX_GLOBAL,
                     vertex_offset: int = 0, ctx: Optional[Context] = None,
                     attributes: bool = False, widths=None, custom_attributes=None,
                     width_attribute: int = -1) -> BatchResult:
    """Batched stroke or fill of every path of a DeviceBatch (results stay on the device,
    owned by the context until its next batched call). With `attributes` (strokes), the
    vertices are lyon_stroke_vertex records (BatchResult.records). `custom_attributes`, a (P, A)
    f32 device tensor of per-point endpoint attributes (A may be 0), selects
    lyon_gpu_stroke_paths_custom: every vertex's source and interpolated attributes
    (BatchResult.sources / custom_attributes); `width_attribute` >= 0 strokes with that
    attribute as the variable line width."""
    ctx = ctx or Context.default()
    out = _native.CBatchOutput()
    cb = dbatch.c()
    if (attributes or widths is not None) and kind != "stroke":
        raise ValueError("vertex attributes and variable widths are stroke options")
    if custom_attributes is not None and kind == "fill":
        na = int(custom_attributes.shape[1]) if custom_attributes.dim() == 2 else 0
        co = _native.CFillCustomOutput()
        r = ctx.lib.lyon_gpu_fill_paths_custom(
            ctx.h, ctypes.byref(cb), custom_attributes.data_ptr() if na else None, na,
            options_dev.data_ptr(), num_options, index_bits, index_mode, vertex_offset,
            ctypes.byref(out), ctypes.byref(co))
        if r != LYON_OK:
            raise TessellationError(r, ctx.last_error())
        return BatchResult(r, int(out.total_vertices), int(out.total_indices),
                           int(out.num_failed_paths), int(out.vertices or 0),
                           int(out.indices or 0), int(out.status or 0), index_bits,
                           dbatch.num_paths, int(out.vertex_offsets or 0),
                           int(out.index_offsets or 0), 2, int(co.sources or 0),
                           int(co.attributes or 0), na, int(co.source_offsets or 0),
                           int(co.total_sources))
    if custom_attributes is not None:
        na = int(custom_attributes.shape[1]) if custom_attributes.dim() == 2 else 0
        co = _native.CCustomOutput()
        r = ctx.lib.lyon_gpu_stroke_paths_custom(
            ctx.h, ctypes.byref(cb), custom_attributes.data_ptr() if na else None, na,
            width_attribute, options_dev.data_ptr(), num_options, index_bits, index_mode,
            vertex_offset, 1 if attributes else 0, ctypes.byref(out), ctypes.byref(co))
        if r != LYON_OK:
            raise TessellationError(r, ctx.last_error())
        return BatchResult(r, int(out.total_vertices), int(out.total_indices),
                           int(out.num_failed_paths), int(out.vertices or 0),
                           int(out.indices or 0), int(out.status or 0), index_bits,
                           dbatch.num_paths, int(out.vertex_offsets or 0),
                           int(out.index_offsets or 0), 6 if attributes else 2,
                           int(co.sources or 0), int(co.attributes or 0), na)
    if widths is not None:
        # Variable line width: `widths` is a device tensor of one f32 factor per point.
        r = ctx.lib.lyon_gpu_stroke_paths_variable_width(
            ctx.h, ctypes.byref(cb), widths.data_ptr(), options_dev.data_ptr(), num_options,
            index_bits, index_mode, vertex_offset, 1 if attributes else 0, ctypes.byref(out))
    else:
        if attributes:
            fn = ctx.lib.lyon_gpu_stroke_paths_attributes
        else:
            fn = ctx.lib.lyon_gpu_stroke_paths if kind == "stroke" else ctx.lib.lyon_gpu_fill_paths
        r = fn(ctx.h, ctypes.byref(cb), options_dev.data_ptr(), num_options, index_bits,
               index_mode, vertex_offset, ctypes.byref(out))
    if r != LYON_OK:
        raise TessellationError(r, ctx.last_error())
    return BatchResult(r, int(out.total_vertices), int(out.total_indices),
                       int(out.num_failed_paths), int(out.vertices or 0), int(out.indices or 0),
                       int(out.status or 0), index_bits, dbatch.num_paths,
                       int(out.vertex_offsets or 0), int(out.index_offsets or 0),
                       6 if attributes else 2)
