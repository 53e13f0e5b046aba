"""Hatching and dots on the CPU: the oracle's restatement of lyon_algorithms' Hatcher
(crates/algorithms/src/hatching.rs) on lyon's own `simple_hatching` case and on geometric
properties (segments run from outline to outline along rotated scan lines; dots on the regular
grid)."""

import ctypes
import ctypes.util
import math

import numpy as np

from oracle import lyon_oracle as orc
from lyon_gb300.path import Path, PathBatch, PathBuilder, Verb

_libm = ctypes.CDLL(ctypes.util.find_library("m") or "libm.so.6")
for _n in ("cosf", "sinf"):
    getattr(_libm, _n).restype = ctypes.c_float
    getattr(_libm, _n).argtypes = [ctypes.c_float]


def params(angle=0.0, interval=1.0, tangents=True, dots=False, column=1.0, tol=0.1,
           uv=(0.0, 0.0)):
    """The oracle's 11 parameters, cos/sin from the C library as the GPU library takes them."""
    return [tol, _libm.cosf(angle), _libm.sinf(angle), _libm.cosf(-angle), _libm.sinf(-angle),
            uv[0], uv[1], interval, 1.0 if tangents else 0.0, 1.0 if dots else 0.0, column]


SQUARE = Path.from_arrays([Verb.BEGIN, Verb.LINE_TO, Verb.LINE_TO, Verb.LINE_TO, Verb.CLOSE],
                          [[0, 0], [10, 0], [10, 10], [0, 10], [0, 0]])


def test_simple_hatching():
    # hatching.rs:725-756: a 10 x 10 square hatched every 1.0.
    out, offs, st = orc.hatch(PathBatch.from_paths([SQUARE]), params())
    assert list(st) == [0]
    assert len(out) == 9
    assert np.array_equal(out["a_x"], np.zeros(9, np.float32))
    assert np.array_equal(out["b_x"], np.full(9, 10.0, np.float32))
    assert np.array_equal(out["a_y"], np.arange(1, 10, dtype=np.float32))
    assert np.array_equal(out["row"], np.arange(9, dtype=np.uint32))
    assert np.allclose(out["a_tangent_y"], 1.0) and np.allclose(out["b_tangent_y"], 1.0)


def test_rotated_hatching_stays_inside():
    b = PathBuilder()
    b.add_circle((0.0, 0.0), 50.0)
    b.add_polygon([(100, 0), (140, 10), (120, 60)], True)
    batch = PathBatch.from_paths([b.build()])
    for angle in (0.3, 1.2, -2.0):
        out, offs, st = orc.hatch(batch, params(angle=angle, interval=3.0))
        assert st[0] == 0 and len(out) > 20
        # Segments are perpendicular to the rotated v axis: constant v along the row, and
        # a, b on the same scan line rotated back.
        d = np.stack([out["b_x"] - out["a_x"], out["b_y"] - out["a_y"]], axis=1)
        along = np.array([math.cos(angle), -math.sin(angle)])
        cross = d[:, 0] * along[1] - d[:, 1] * along[0]
        assert np.allclose(cross, 0, atol=1e-3)
        assert np.all(out["b_u"] >= out["a_u"])


def test_dots_grid():
    out, offs, st = orc.hatch(PathBatch.from_paths([SQUARE]),
                              params(dots=True, interval=2.0, column=2.5, tangents=False))
    assert st[0] == 0
    # Rows at y = 2, 4, 6, 8; columns at u = 0, 2.5, 5, 7.5.
    assert len(out) == 16
    assert np.array_equal(np.unique(out["y"]), np.array([2, 4, 6, 8], np.float32))
    assert np.array_equal(np.unique(out["x"]), np.array([0, 2.5, 5, 7.5], np.float32))
    assert np.array_equal(out["column"][:4], np.arange(4, dtype=np.uint32))


def test_empty_and_tiny_interval():
    empty = Path.from_arrays([], np.zeros((0, 2)))
    out, offs, st = orc.hatch(PathBatch.from_paths([empty, SQUARE]), params(interval=0.0))
    # An interval of 0 draws one row and stops (next_offset <= 0 ends the sweep).
    assert list(st) == [0, 0] and offs[1] == 0 and offs[2] - offs[1] == 1
