"""Hatching and dot patterns: lyon_algorithms' `hatching` module
(crates/algorithms/src/hatching.rs) on the GPU.

`Hatcher.hatch_path` / `dot_path` mirror lyon's with the regular patterns
(`RegularHatchingPattern`, `RegularDotPattern`): the segments or dots come back as structured
arrays instead of through a callback. `hatch_paths` / `dot_paths` run a whole device-resident
batch (lyon_gpu_hatch_paths / lyon_gpu_dot_paths).
"""

from __future__ import annotations

import ctypes
from dataclasses import dataclass, replace
from typing import Optional

import numpy as np

from . import _native
from .path import Path, PathBatch
from .tessellation import (Context, DeviceBatch, LYON_OK, TessellationError, _CudaArray)

HATCH_SEGMENT_DTYPE = np.dtype([("a_x", "<f4"), ("a_y", "<f4"), ("a_tangent_x", "<f4"),
                                ("a_tangent_y", "<f4"), ("a_u", "<f4"), ("b_x", "<f4"),
                                ("b_y", "<f4"), ("b_tangent_x", "<f4"), ("b_tangent_y", "<f4"),
                                ("b_u", "<f4"), ("row", "<u4"), ("v", "<f4")])
DOT_DTYPE = np.dtype([("x", "<f4"), ("y", "<f4"), ("u", "<f4"), ("v", "<f4"), ("column", "<u4"),
                      ("row", "<u4")])


@dataclass(frozen=True)
class HatchingOptions:
    """HatchingOptions (hatching.rs:44-118)."""
    tolerance: float = 0.1
    angle: float = 0.0
    compute_tangents: bool = True
    uv_origin: tuple = (0.0, 0.0)

    def with_tolerance(self, t: float) -> "HatchingOptions":
        return replace(self, tolerance=t)

    def with_angle(self, a: float) -> "HatchingOptions":
        return replace(self, angle=a)

    def with_tangents(self, b: bool) -> "HatchingOptions":
        return replace(self, compute_tangents=b)


@dataclass(frozen=True)
class DotOptions:
    """DotOptions (hatching.rs:120-179)."""
    tolerance: float = 0.1
    angle: float = 0.0
    uv_origin: tuple = (0.0, 0.0)


@dataclass
class HatchResult:
    """Device tensors (owned by the context until its next call): path i's records are
    records[offsets[i]:offsets[i + 1]] (uint8 rows of HATCH_SEGMENT_DTYPE / DOT_DTYPE size)."""
    records: object
    offsets: object
    status: object
    total: int
    dtype: np.dtype

    def to_numpy(self):
        if self.total == 0:
            return np.zeros(0, self.dtype)
        return self.records.cpu().numpy().view(self.dtype).reshape(-1)


def _run(fn, dbatch: DeviceBatch, o: _native.CHatchingOptions, dtype, ctx) -> HatchResult:
    import torch
    out = _native.CHatchOutput()
    cb = dbatch.c()
    r = fn(ctx.h, ctypes.byref(cb), ctypes.byref(o), ctypes.byref(out))
    if r != LYON_OK:
        raise TessellationError(r, ctx.last_error())
    n = dbatch.num_paths
    total = int(out.total)
    ptr = out.dots if dtype is DOT_DTYPE else out.segments
    rec = torch.as_tensor(_CudaArray(int(ptr or 0), (total, dtype.itemsize), "|u1"),
                          device="cuda")
    offs = torch.as_tensor(_CudaArray(int(out.offsets or 0), (n + 1,), "<i8"), device="cuda")
    st = torch.as_tensor(_CudaArray(int(out.status or 0), (n,), "<i4"), device="cuda")
    return HatchResult(rec, offs, st, total, dtype)


def hatch_paths(dbatch: DeviceBatch, options: HatchingOptions, interval: float,
                ctx: Optional[Context] = None) -> HatchResult:
    """Hatcher::hatch_path with RegularHatchingPattern { interval } for every path."""
    ctx = ctx or Context.default()
    o = _native.CHatchingOptions(options.tolerance, options.angle, options.uv_origin[0],
                                 options.uv_origin[1], interval, 0.0,
                                 1 if options.compute_tangents else 0)
    return _run(ctx.lib.lyon_gpu_hatch_paths, dbatch, o, HATCH_SEGMENT_DTYPE, ctx)


def dot_paths(dbatch: DeviceBatch, options: DotOptions, row_interval: float,
              column_interval: float, ctx: Optional[Context] = None) -> HatchResult:
    """Hatcher::dot_path with RegularDotPattern { column_interval, row_interval }."""
    ctx = ctx or Context.default()
    o = _native.CHatchingOptions(options.tolerance, options.angle, options.uv_origin[0],
                                 options.uv_origin[1], row_interval, column_interval, 0)
    return _run(ctx.lib.lyon_gpu_dot_paths, dbatch, o, DOT_DTYPE, ctx)


class Hatcher:
    """lyon's Hatcher (hatching.rs:243-298) for one path at a time."""

    def __init__(self, ctx: Optional[Context] = None):
        self.ctx = ctx or Context.default()

    def hatch_path(self, path: Path, options: HatchingOptions, interval: float) -> np.ndarray:
        db = DeviceBatch.upload(PathBatch.from_paths([path]), 0)
        res = hatch_paths(db, options, interval, self.ctx)
        self.ctx.synchronize()
        _check(res)
        return res.to_numpy()

    def dot_path(self, path: Path, options: DotOptions, row_interval: float,
                 column_interval: float) -> np.ndarray:
        db = DeviceBatch.upload(PathBatch.from_paths([path]), 0)
        res = dot_paths(db, options, row_interval, column_interval, self.ctx)
        self.ctx.synchronize()
        _check(res)
        return res.to_numpy()


def _check(res: HatchResult) -> None:
    st = int(res.status.cpu().numpy()[0])
    if st != LYON_OK:
        raise TessellationError(st)
