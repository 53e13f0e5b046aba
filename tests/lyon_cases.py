"""Helpers shared by the tests: golden fixtures and lyon's test harness conventions."""

from __future__ import annotations

import json
import math
import os

import numpy as np

from lyon_gb300.path import Path, PathBuilder, Verb
from lyon_gb300.options import LineCap, LineJoin, StrokeOptions

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load(name):
    with open(os.path.join(GOLDEN, name)) as f:
        return json.load(f)


def case_path(case) -> Path:
    return Path.from_arrays(case["verbs"], case["points"] if case["points"] else np.zeros((0, 2)))


def rust_logo() -> Path:
    d = load("rust_logo.json")
    return Path.from_arrays(d["verbs"], d["points"])


def stroke_options_from_case(opts: dict) -> StrokeOptions:
    o = StrokeOptions()
    for k, v in opts.items():
        if k == "line_join":
            o = o.with_line_join(getattr(LineJoin, v))
        elif k == "line_cap":
            o = o.with_line_cap(getattr(LineCap, v))
        elif k == "tolerance":
            o = o.with_tolerance(float(v))
        elif k == "miter_limit":
            o = o.with_miter_limit(float(v))
        elif k == "line_width":
            o = o.with_line_width(float(v))
        elif k == "variable_line_width":
            pass  # the case's per-point `widths` carry the attribute
        else:
            raise KeyError(k)
    return o


def flatten_to_lines(path: Path, counts: np.ndarray, pts: np.ndarray) -> Path:
    """Rebuilds `path.iter().flattened(tol)` events as a line-only Path (the way
    crates/tessellation/src/fill_tests.rs:10-28 feeds its tessellator)."""
    b = PathBuilder()
    pi = 0  # index into the original points (for Begin)
    fi = 0  # index into the flattened points
    for vi, v in enumerate(path.verbs.tolist()):
        if v == Verb.BEGIN:
            b.begin(path.points[pi])
            pi += 1
        elif v in (Verb.LINE_TO, Verb.QUADRATIC_TO, Verb.CUBIC_TO):
            for _ in range(int(counts[vi])):
                b.line_to(pts[fi])
                fi += 1
            pi += {Verb.LINE_TO: 1, Verb.QUADRATIC_TO: 2, Verb.CUBIC_TO: 3}[v]
        elif v == Verb.CLOSE:
            b.end(True)
            pi += 1
        elif v == Verb.END:
            b.end(False)
    return b.build()


def rotation_angles(step: float):
    """The angles lyon's test_path_with_rotations visits (fill_tests.rs:134-150), in f32."""
    angle = np.float32(0.0)
    two_pi = np.float32(math.pi) * np.float32(2.0)
    step = np.float32(step)
    while angle < two_pi:
        yield float(angle)
        angle = np.float32(angle + step)
