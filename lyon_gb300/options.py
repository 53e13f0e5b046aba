"""Tessellation options and enums mirroring lyon's.

LineCap / LineJoin / FillRule: crates/path/src/lib.rs:170-281.
StrokeOptions: crates/tessellation/src/lib.rs:315-433.
FillOptions:   crates/tessellation/src/lib.rs:445-537.
The ctypes structures match `lyon_stroke_options` / `lyon_fill_options` in include/lyon_gpu.h.
"""

from __future__ import annotations

import ctypes
from dataclasses import dataclass, replace
from typing import Optional

import numpy as np


class LineCap:
    Butt = 0
    Square = 1
    Round = 2


class LineJoin:
    Miter = 0
    MiterClip = 1
    Round = 2
    Bevel = 3


class FillRule:
    EvenOdd = 0
    NonZero = 1


class Orientation:
    Vertical = 0
    Horizontal = 1


class CStrokeOptions(ctypes.Structure):
    _fields_ = [("start_cap", ctypes.c_int32), ("end_cap", ctypes.c_int32),
                ("line_join", ctypes.c_int32), ("line_width", ctypes.c_float),
                ("miter_limit", ctypes.c_float), ("tolerance", ctypes.c_float)]


class CFillOptions(ctypes.Structure):
    _fields_ = [("tolerance", ctypes.c_float), ("fill_rule", ctypes.c_int32),
                ("sweep_orientation", ctypes.c_int32), ("handle_intersections", ctypes.c_int32)]


STROKE_OPTIONS_DTYPE = np.dtype([("start_cap", "<i4"), ("end_cap", "<i4"), ("line_join", "<i4"),
                                 ("line_width", "<f4"), ("miter_limit", "<f4"),
                                 ("tolerance", "<f4")])
FILL_OPTIONS_DTYPE = np.dtype([("tolerance", "<f4"), ("fill_rule", "<i4"),
                               ("sweep_orientation", "<i4"), ("handle_intersections", "<i4")])


@dataclass(frozen=True)
class StrokeOptions:
    start_cap: int = LineCap.Butt
    end_cap: int = LineCap.Butt
    line_join: int = LineJoin.Miter
    line_width: float = 1.0
    miter_limit: float = 4.0
    tolerance: float = 0.1
    # StrokeOptions::variable_line_width (lib.rs:340, 429-432): the index of the path's endpoint
    # attribute that scales line_width, or None. Passed beside the C record, which has no field
    # for it.
    variable_line_width: Optional[int] = None

    MINIMUM_MITER_LIMIT = 1.0

    @staticmethod
    def default() -> "StrokeOptions":
        return StrokeOptions()

    @staticmethod
    def with_tolerance_only(tolerance: float) -> "StrokeOptions":
        return StrokeOptions(tolerance=tolerance)

    def with_tolerance(self, tolerance: float) -> "StrokeOptions":
        return replace(self, tolerance=tolerance)

    def with_line_cap(self, cap: int) -> "StrokeOptions":
        return replace(self, start_cap=cap, end_cap=cap)

    def with_start_cap(self, cap: int) -> "StrokeOptions":
        return replace(self, start_cap=cap)

    def with_end_cap(self, cap: int) -> "StrokeOptions":
        return replace(self, end_cap=cap)

    def with_line_join(self, join: int) -> "StrokeOptions":
        return replace(self, line_join=join)

    def with_line_width(self, width: float) -> "StrokeOptions":
        return replace(self, line_width=width)

    def with_variable_line_width(self, index: int) -> "StrokeOptions":
        return replace(self, variable_line_width=index)

    def with_miter_limit(self, limit: float) -> "StrokeOptions":
        # lib.rs:423-427 asserts limit >= MINIMUM_MITER_LIMIT.
        assert limit >= self.MINIMUM_MITER_LIMIT
        return replace(self, miter_limit=limit)

    def to_c(self) -> CStrokeOptions:
        return CStrokeOptions(self.start_cap, self.end_cap, self.line_join, self.line_width,
                              self.miter_limit, self.tolerance)

    def to_record(self) -> np.ndarray:
        r = np.zeros(1, dtype=STROKE_OPTIONS_DTYPE)
        r[0] = (self.start_cap, self.end_cap, self.line_join, self.line_width, self.miter_limit,
                self.tolerance)
        return r


@dataclass(frozen=True)
class FillOptions:
    tolerance: float = 0.1
    fill_rule: int = FillRule.EvenOdd
    sweep_orientation: int = Orientation.Vertical
    handle_intersections: bool = True

    @staticmethod
    def default() -> "FillOptions":
        return FillOptions()

    @staticmethod
    def even_odd() -> "FillOptions":
        return FillOptions()

    @staticmethod
    def non_zero() -> "FillOptions":
        return FillOptions(fill_rule=FillRule.NonZero)

    def with_tolerance(self, tolerance: float) -> "FillOptions":
        return replace(self, tolerance=tolerance)

    def with_fill_rule(self, rule: int) -> "FillOptions":
        return replace(self, fill_rule=rule)

    def with_sweep_orientation(self, o: int) -> "FillOptions":
        return replace(self, sweep_orientation=o)

    def with_intersections(self, b: bool) -> "FillOptions":
        return replace(self, handle_intersections=b)

    def to_c(self) -> CFillOptions:
        return CFillOptions(self.tolerance, self.fill_rule, self.sweep_orientation,
                            1 if self.handle_intersections else 0)

    def to_record(self) -> np.ndarray:
        r = np.zeros(1, dtype=FILL_OPTIONS_DTYPE)
        r[0] = (self.tolerance, self.fill_rule, self.sweep_orientation,
                1 if self.handle_intersections else 0)
        return r


def stroke_options_array(records) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(records, dtype=STROKE_OPTIONS_DTYPE))


def fill_options_array(records) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(records, dtype=FILL_OPTIONS_DTYPE))
