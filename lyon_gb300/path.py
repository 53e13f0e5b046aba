"""Path storage mirroring lyon's `Path` (crates/path/src/path.rs:75-79, 472-597).

A path is two arrays: one verb byte per event and the points in event order. `close` stores the
first point of the sub-path again, exactly as lyon's `BuilderImpl::end` does
(crates/path/src/path.rs:534-542). `PathBatch` concatenates many paths with offset arrays; it is
the input layout of the batched C ABI (`lyon_path_batch` in include/lyon_gpu.h).
"""

from __future__ import annotations

import math
from dataclasses import dataclass
from typing import Iterable, List, Sequence, Tuple

import numpy as np


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
