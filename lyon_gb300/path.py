"""Path storage mirroring lyon's `Path` (crates/path/src/path.rs:75-79, 472-597).

A path is two arrays: one verb byte per event and the points in event order. `close` stores the
first point of the sub-path again, exactly as lyon's `BuilderImpl::end` does
(crates/path/src/path.rs:534-542). `PathBatch` concatenates many paths with offset arrays; it is
the input layout of the batched C ABI (`lyon_path_batch` in include/lyon_gpu.h).
"""

from __future__ import annotations

import ctypes
import ctypes.util
import math
from dataclasses import dataclass
from typing import Iterable, List, Sequence, Tuple

import numpy as np

# lyon takes f32 cos/sin/tan from the platform's libm; the builder's ellipses do the same.
_libm = ctypes.CDLL(ctypes.util.find_library("m") or "libm.so.6")
for _name in ("cosf", "sinf", "tanf"):
    getattr(_libm, _name).restype = ctypes.c_float
    getattr(_libm, _name).argtypes = [ctypes.c_float]
_F = np.float32


def _cosf(x) -> np.float32:
    return _F(_libm.cosf(float(x)))


def _sinf(x) -> np.float32:
    return _F(_libm.sinf(float(x)))


def _rotate(angle, x, y):
    """euclid's Rotation2D::transform_point / transform_vector, in f32."""
    c, s = _cosf(angle), _sinf(angle)
    return _F(x * c - y * s), _F(x * s + y * c)


def arc_quadratic_beziers(center, radii, start_angle, sweep_angle, x_rotation):
    """arc_to_quadratic_beziers_with_t (crates/geom/src/arc.rs:668-703), f32 arithmetic: the
    arc split into ceil(|sweep| / (pi/4)) equal steps, each one quadratic whose control point is
    on the tangent at its start (Maisonobe). Returns [(from, ctrl, to, t0, t1), ...]."""
    cx, cy = _F(center[0]), _F(center[1])
    rx, ry = _F(radii[0]), _F(radii[1])
    start, sweep, rot = _F(start_angle), _F(sweep_angle), _F(x_rotation)
    sign = _F(math.copysign(1.0, float(sweep))) if not math.isnan(float(sweep)) else _F(np.nan)
    two_pi = _F(np.pi) * _F(2.0)
    sw = min(_F(abs(sweep)), two_pi)
    n_steps = _F(np.ceil(sw / _F(np.pi / 4)))
    step = _F(sw / n_steps * sign)
    dt = _F(_F(1.0) / n_steps)
    alpha = _F(_libm.tanf(float(step * _F(0.5))))
    n = int(n_steps)
    out = []
    t0 = _F(0.0)

    def sample(a):
        ex, ey = _F(rx * _cosf(a)), _F(ry * _sinf(a))
        vx, vy = _rotate(rot, ex, ey)
        return _F(cx + vx), _F(cy + vy)
    for i in range(n):
        a1 = _F(start + _F(step * _F(i)))
        a2 = _F(start + _F(step * _F(i + 1)))
        frm = sample(a1)
        to = sample(a2)
        tx, ty = _rotate(rot, _F(-rx * _sinf(a1)), _F(ry * _cosf(a1)))
        ctrl = (_F(frm[0] + _F(tx * alpha)), _F(frm[1] + _F(ty * alpha)))
        t1 = _F(1.0) if i + 1 == n else _F(t0 + dt)
        out.append((frm, ctrl, to, t0, t1))
        t0 = t1
    return out


class Verb:
    """Same order as lyon's `Verb` (crates/path/src/path.rs:29-36)."""

    LINE_TO = 0
    QUADRATIC_TO = 1
    CUBIC_TO = 2
    BEGIN = 3
    CLOSE = 4
    END = 5


_POINTS_PER_VERB = np.array([1, 2, 3, 1, 1, 0], dtype=np.int64)


@dataclass
class Path:
    verbs: np.ndarray   # uint8 [num_verbs]
    points: np.ndarray  # float32 [num_points, 2]

    @staticmethod
    def builder() -> "PathBuilder":
        return PathBuilder()

    @staticmethod
    def from_arrays(verbs: Sequence[int], points: Sequence[Sequence[float]]) -> "Path":
        v = np.asarray(verbs, dtype=np.uint8).reshape(-1)
        p = np.asarray(points, dtype=np.float32).reshape(-1, 2)
        return Path(np.ascontiguousarray(v), np.ascontiguousarray(p))

    @property
    def num_verbs(self) -> int:
        return int(self.verbs.shape[0])

    @property
    def num_points(self) -> int:
        return int(self.points.shape[0])

    def transformed_rotation(self, angle: float) -> "Path":
        """Rotation about the origin, evaluated in f32 as euclid's Rotation2D applies it."""
        a = np.float32(angle)
        c = np.float32(math.cos(float(a)))
        s = np.float32(math.sin(float(a)))
        x = self.points[:, 0]
        y = self.points[:, 1]
        nx = (x * c - y * s).astype(np.float32)
        ny = (x * s + y * c).astype(np.float32)
        return Path(self.verbs.copy(), np.ascontiguousarray(np.stack([nx, ny], axis=1)))

    def scaled(self, scale: float) -> "Path":
        return Path(self.verbs.copy(), (self.points * np.float32(scale)).astype(np.float32))

    def iter_events(self):
        """Yields lyon PathEvents as tuples (crates/path/src/path.rs:843-909)."""
        pi = 0
        cur = first = None
        for v in self.verbs.tolist():
            if v == Verb.BEGIN:
                cur = first = tuple(self.points[pi])
                pi += 1
                yield ("begin", cur)
            elif v == Verb.LINE_TO:
                to = tuple(self.points[pi])
                pi += 1
                yield ("line", cur, to)
                cur = to
            elif v == Verb.QUADRATIC_TO:
                c, to = tuple(self.points[pi]), tuple(self.points[pi + 1])
                pi += 2
                yield ("quadratic", cur, c, to)
                cur = to
            elif v == Verb.CUBIC_TO:
                c1, c2, to = (tuple(self.points[pi]), tuple(self.points[pi + 1]),
                              tuple(self.points[pi + 2]))
                pi += 3
                yield ("cubic", cur, c1, c2, to)
                cur = to
            elif v == Verb.CLOSE:
                pi += 1
                yield ("end", cur, first, True)
            elif v == Verb.END:
                yield ("end", cur, first, False)
                cur = first


class PathBuilder:
    """lyon's `Path::builder()` (crates/path/src/path.rs:472-597)."""

    def __init__(self):
        self._verbs: List[int] = []
        self._points: List[Tuple[float, float]] = []
        self._first = (0.0, 0.0)
        self._open = False

    def begin(self, at) -> int:
        assert not self._open, "begin() while a sub-path is open"
        at = (float(at[0]), float(at[1]))
        idx = len(self._points)
        self._first = at
        self._points.append(at)
        self._verbs.append(Verb.BEGIN)
        self._open = True
        return idx

    def line_to(self, to) -> int:
        assert self._open
        idx = len(self._points)
        self._points.append((float(to[0]), float(to[1])))
        self._verbs.append(Verb.LINE_TO)
        return idx

    def quadratic_bezier_to(self, ctrl, to) -> int:
        assert self._open
        self._points.append((float(ctrl[0]), float(ctrl[1])))
        idx = len(self._points)
        self._points.append((float(to[0]), float(to[1])))
        self._verbs.append(Verb.QUADRATIC_TO)
        return idx

    def cubic_bezier_to(self, ctrl1, ctrl2, to) -> int:
        assert self._open
        self._points.append((float(ctrl1[0]), float(ctrl1[1])))
        self._points.append((float(ctrl2[0]), float(ctrl2[1])))
        idx = len(self._points)
        self._points.append((float(to[0]), float(to[1])))
        self._verbs.append(Verb.CUBIC_TO)
        return idx

    def end(self, close: bool) -> None:
        assert self._open
        if close:
            self._points.append(self._first)
        self._verbs.append(Verb.CLOSE if close else Verb.END)
        self._open = False

    def close(self) -> None:
        self.end(True)

    # ---- shapes (crates/path/src/builder.rs:560-680, 1508-1548, 1551-1660) ----------------
    # Arithmetic is f32, as in lyon; `winding` is +1 (Winding::Positive) or -1 (Negative).

    def add_polygon(self, points, closed: bool = True) -> None:
        """builder.rs:560-573: begin at the first point, a line to each next one."""
        pts = np.asarray(points, dtype=np.float32).reshape(-1, 2)
        if len(pts) == 0:
            return
        self.begin(pts[0])
        for p in pts[1:]:
            self.line_to(p)
        self.end(closed)

    def add_rectangle(self, rect, winding: int = 1) -> None:
        """builder.rs:649-675; rect = (min_x, min_y, max_x, max_y)."""
        x0, y0, x1, y1 = [np.float32(v) for v in rect]
        if winding >= 0:
            self.add_polygon([(x0, y0), (x1, y0), (x1, y1), (x0, y1)], True)
        else:
            self.add_polygon([(x0, y0), (x0, y1), (x1, y1), (x1, y0)], True)

    def add_circle(self, center, radius: float, winding: int = 1) -> None:
        """builder.rs:1508-1548: four cubic arcs with the 0.55191505 control factor."""
        f = np.float32
        r = abs(f(radius))
        d_dir = f(1.0) if winding >= 0 else f(-1.0)
        cx, cy = f(center[0]), f(center[1])
        d = r * f(0.55191505)

        def at(dx, dy):
            return (cx + f(dx), cy + f(dy))
        self.begin(at(-r, f(0.0)))
        self.cubic_bezier_to(at(-r, -d * d_dir), at(-d, -r * d_dir), at(f(0.0), -r * d_dir))
        self.cubic_bezier_to(at(d, -r * d_dir), at(r, -d * d_dir), at(r, f(0.0)))
        self.cubic_bezier_to(at(r, d * d_dir), at(d, r * d_dir), at(f(0.0), r * d_dir))
        self.cubic_bezier_to(at(-d, r * d_dir), at(-r, d * d_dir), at(-r, f(0.0)))
        self.close()

    def add_ellipse(self, center, radii, x_rotation: float = 0.0, winding: int = 1) -> None:
        """builder.rs:606-636: the full arc (start 0, sweep 2 pi in the winding's direction)
        as quadratic béziers, closed."""
        sweep = _F(_F(2.0) * _F(np.pi)) * (_F(1.0) if winding >= 0 else _F(-1.0))
        quads = arc_quadratic_beziers(center, radii, 0.0, sweep, x_rotation)
        # Arc::sample(0.0): the start angle is 0.
        cx, cy = _F(center[0]), _F(center[1])
        ex, ey = _F(_F(radii[0]) * _cosf(_F(0.0))), _F(_F(radii[1]) * _sinf(_F(0.0)))
        vx, vy = _rotate(_F(x_rotation), ex, ey)
        self.begin((_F(cx + vx), _F(cy + vy)))
        for _frm, ctrl, to, _t0, _t1 in quads:
            self.quadratic_bezier_to(ctrl, to)
        self.end(True)

    def add_rounded_rectangle(self, rect, radii, winding: int = 1) -> None:
        """builder.rs:1551-1660; radii = (top_left, top_right, bottom_left, bottom_right)."""
        f = np.float32
        x_min, y_min, x_max, y_max = [f(v) for v in rect]
        w = x_max - x_min
        h = y_max - y_min
        min_wh = min(w, h)
        tl, tr, bl, br = [min(abs(f(r)), min_wh) for r in radii]
        if tl + tr > w:
            x = (tl + tr - w) * f(0.5)
            tl, tr = tl - x, tr - x
        if bl + br > w:
            x = (bl + br - w) * f(0.5)
            bl, br = bl - x, br - x
        if tr + br > h:
            x = (tr + br - h) * f(0.5)
            tr, br = tr - x, br - x
        if tl + bl > h:
            x = (tl + bl - h) * f(0.5)
            tl, bl = tl - x, bl - x
        k = f(0.55191505)
        tl_d, tr_d, br_d, bl_d = tl * k, tr * k, br * k, bl * k
        z = f(0.0)
        pts = [
            (x_min, y_min + tl), (x_min + z, y_min + (tl - tl_d)), (x_min + (tl - tl_d), y_min + z),
            (x_min + tl, y_min + z),
            (x_max - tr, y_min), (x_max + (-tr + tr_d), y_min + z), (x_max + z, y_min + (tr - tr_d)),
            (x_max + z, y_min + tr),
            (x_max, y_max - br), (x_max + z, y_max + (-br + br_d)), (x_max + (-br + br_d), y_max + z),
            (x_max + -br, y_max + z),
            (x_min + bl, y_max), (x_min + (bl - bl_d), y_max + z), (x_min + z, y_max + (-bl + bl_d)),
            (x_min + z, y_max + -bl),
        ]
        if winding >= 0:
            self.begin(pts[0])
            if tl > 0:
                self.cubic_bezier_to(pts[1], pts[2], pts[3])
            self.line_to(pts[4])
            if tr > 0:
                self.cubic_bezier_to(pts[5], pts[6], pts[7])
            self.line_to(pts[8])
            if br > 0:
                self.cubic_bezier_to(pts[9], pts[10], pts[11])
            self.line_to(pts[12])
            if bl > 0:
                self.cubic_bezier_to(pts[13], pts[14], pts[15])
        else:
            self.begin(pts[15])
            if bl > 0:
                self.cubic_bezier_to(pts[14], pts[13], pts[12])
            self.line_to(pts[11])
            if br > 0:
                self.cubic_bezier_to(pts[10], pts[9], pts[8])
            self.line_to(pts[7])
            if tr > 0:
                self.cubic_bezier_to(pts[6], pts[5], pts[4])
            self.line_to(pts[3])
            if tl > 0:
                self.cubic_bezier_to(pts[2], pts[1], pts[0])
        self.end(True)

    def build(self) -> Path:
        if self._open:
            self.end(False)
        return Path.from_arrays(self._verbs, self._points if self._points else np.zeros((0, 2)))


@dataclass
class PathBatch:
    """Many paths in one SoA layout (the `lyon_path_batch` of include/lyon_gpu.h)."""

    verbs: np.ndarray          # uint8 [total_verbs]
    points: np.ndarray         # float32 [total_points, 2]
    verb_offsets: np.ndarray   # uint32 [num_paths + 1]
    point_offsets: np.ndarray  # uint32 [num_paths + 1]

    @property
    def num_paths(self) -> int:
        return int(self.verb_offsets.shape[0] - 1)

    @staticmethod
    def from_paths(paths: Iterable[Path]) -> "PathBatch":
        paths = list(paths)
        vo = np.zeros(len(paths) + 1, dtype=np.uint32)
        po = np.zeros(len(paths) + 1, dtype=np.uint32)
        vo[1:] = np.cumsum([p.num_verbs for p in paths])
        po[1:] = np.cumsum([p.num_points for p in paths])
        verbs = (np.concatenate([p.verbs for p in paths]).astype(np.uint8) if paths
                 else np.zeros(0, np.uint8))
        pts = (np.concatenate([p.points for p in paths]).astype(np.float32) if paths
               else np.zeros((0, 2), np.float32))
        return PathBatch(np.ascontiguousarray(verbs), np.ascontiguousarray(pts), vo, po)

    def path(self, i: int) -> Path:
        v0, v1 = int(self.verb_offsets[i]), int(self.verb_offsets[i + 1])
        p0, p1 = int(self.point_offsets[i]), int(self.point_offsets[i + 1])
        return Path(self.verbs[v0:v1], self.points[p0:p1])

    def head(self, n: int) -> "PathBatch":
        """The first n paths (array slices, offsets unchanged)."""
        n = min(n, self.num_paths)
        vo = self.verb_offsets[:n + 1]
        po = self.point_offsets[:n + 1]
        return PathBatch(self.verbs[:int(vo[-1])], self.points[:int(po[-1])], vo, po)

    def subset(self, idx: Sequence[int]) -> "PathBatch":
        return PathBatch.from_paths(self.path(int(i)) for i in idx)

    def input_bytes(self, options_bytes_per_path: int = 0) -> int:
        """Algorithmic bytes read: verbs + points + both offset arrays + per-path options."""
        n = self.num_paths
        return int(self.verbs.nbytes + self.points.nbytes + 8 * (n + 1)
                   + options_bytes_per_path * n)


def points_per_verb(verbs: np.ndarray) -> np.ndarray:
    return _POINTS_PER_VERB[verbs.astype(np.int64)]
