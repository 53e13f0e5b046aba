"""lyon's PathBuffer (crates/path/src/path_buffer.rs): many paths stored contiguously.

The buffer holds exactly the arrays of a PathBatch (verbs, points, per-path verb and point
ranges), so `as_batch()` is the batched C ABI's input without repacking, and a buffer built with
attributes gives the per-point attribute table the custom-attribute calls read
(`attribute_table`). Paths keep their own endpoint ids (builders return ids relative to the
path's first point, as lyon's `Builder::adjust_id` does).
"""

from __future__ import annotations

from typing import Iterable, Iterator, List, Optional, Sequence

import numpy as np

from .path import Path, PathBatch, PathBuilder, Verb


class PathBuffer:
    """PathBuffer (path_buffer.rs:14-130)."""

    def __init__(self):
        self._verbs: List[np.ndarray] = []
        self._points: List[np.ndarray] = []
        self._attrs: List[Optional[np.ndarray]] = []
        self._num_attributes: List[int] = []

    @staticmethod
    def with_capacity(endpoints: int = 0, ctrl_points: int = 0, paths: int = 0) -> "PathBuffer":
        return PathBuffer()

    @staticmethod
    def from_paths(paths: Iterable[Path]) -> "PathBuffer":
        """FromIterator<PathSlice> (path_buffer.rs:114-130)."""
        buf = PathBuffer()
        for p in paths:
            buf._push(p.verbs, p.points, None)
        return buf

    def _push(self, verbs, points, attrs) -> int:
        self._verbs.append(np.ascontiguousarray(verbs, np.uint8))
        self._points.append(np.ascontiguousarray(points, np.float32).reshape(-1, 2))
        self._attrs.append(attrs)
        self._num_attributes.append(0 if attrs is None else attrs.shape[1])
        return len(self._verbs) - 1

    def builder(self) -> "PathBufferBuilder":
        return PathBufferBuilder(self)

    def get(self, index: int) -> Path:
        return Path(self._verbs[index], self._points[index])

    def attributes(self, index: int) -> Optional[np.ndarray]:
        """The path's per-point attributes ((points, n) f32), or None."""
        return self._attrs[index]

    def num_attributes(self, index: int) -> int:
        return self._num_attributes[index]

    def indices(self) -> range:
        return range(len(self._verbs))

    def __len__(self) -> int:
        return len(self._verbs)

    def is_empty(self) -> bool:
        return len(self._verbs) == 0

    def __iter__(self) -> Iterator[Path]:
        return (self.get(i) for i in self.indices())

    def clear(self) -> None:
        self.__init__()

    def reserve(self, endpoints: int = 0, ctrl_points: int = 0, paths: int = 0) -> None:
        pass

    def as_batch(self) -> PathBatch:
        return PathBatch.from_paths(self)

    def attribute_table(self, num_attributes: Optional[int] = None) -> np.ndarray:
        """One row of `num_attributes` floats per point of `as_batch()` (zeros for paths built
        without attributes): the table lyon_gpu_stroke_paths_custom / fill_paths_custom read."""
        n = num_attributes if num_attributes is not None else max(self._num_attributes,
                                                                  default=0)
        rows = []
        for pts, a in zip(self._points, self._attrs):
            r = np.zeros((len(pts), n), np.float32)
            if a is not None and n:
                k = min(n, a.shape[1])
                r[:, :k] = a[:, :k]
            rows.append(r)
        return np.concatenate(rows) if rows else np.zeros((0, n), np.float32)


class PathBufferBuilder(PathBuilder):
    """path_buffer.rs:193-348: a path builder whose build() appends to the buffer and returns
    the path's index."""

    def __init__(self, buffer: PathBuffer):
        super().__init__()
        self._buffer = buffer

    def with_attributes(self, num_attributes: int) -> "PathBufferBuilderWithAttributes":
        assert not self._verbs, "with_attributes() before the first event"
        return PathBufferBuilderWithAttributes(self._buffer, num_attributes)

    def build(self) -> int:  # type: ignore[override]
        p = super().build()
        return self._buffer._push(p.verbs, p.points, None)


class PathBufferBuilderWithAttributes:
    """path_buffer.rs:350-500: endpoints carry `num_attributes` floats (rows of control points
    and of Close's repeated point hold the neighbouring endpoint's values)."""

    def __init__(self, buffer: PathBuffer, num_attributes: int):
        self._buffer = buffer
        self._b = PathBuilder()
        self._n = num_attributes
        self._rows: List[np.ndarray] = []
        self._first = np.zeros(num_attributes, np.float32)

    def _attrs(self, attributes: Sequence[float]) -> np.ndarray:
        a = np.asarray(attributes, np.float32).reshape(-1)
        assert len(a) == self._n, "one value per attribute"
        return a

    def begin(self, at, attributes) -> int:
        a = self._attrs(attributes)
        self._first = a
        self._rows.append(a)
        return self._b.begin(at)

    def line_to(self, to, attributes) -> int:
        self._rows.append(self._attrs(attributes))
        return self._b.line_to(to)

    def quadratic_bezier_to(self, ctrl, to, attributes) -> int:
        a = self._attrs(attributes)
        self._rows += [a, a]
        return self._b.quadratic_bezier_to(ctrl, to)

    def cubic_bezier_to(self, ctrl1, ctrl2, to, attributes) -> int:
        a = self._attrs(attributes)
        self._rows += [a, a, a]
        return self._b.cubic_bezier_to(ctrl1, ctrl2, to)

    def end(self, close: bool) -> None:
        if close:
            self._rows.append(self._first)
        self._b.end(close)

    def close(self) -> None:
        self.end(True)

    def build(self) -> int:
        p = self._b.build()
        attrs = (np.stack(self._rows).astype(np.float32) if self._rows
                 else np.zeros((0, self._n), np.float32))
        assert len(attrs) == len(p.points)
        return self._buffer._push(p.verbs, p.points, attrs)
