"""The path builder's shapes (crates/path/src/builder.rs): lyon's own test of a rounded
rectangle, and the layouts of rectangles, circles and polygons (CPU only)."""

import numpy as np

from lyon_gb300.path import PathBuilder, Verb


def _events(path):
    return list(path.iter_events())


def test_top_right_rounded_rect():
    # builder.rs:1807-1822: only the top-right corner rounded (radius 2); the third event is
    # its cubic from (98, 0) to (100, 2).
    b = PathBuilder()
    b.add_rounded_rectangle((0.0, 0.0, 100.0, 100.0), (0.0, 2.0, 0.0, 0.0), 1)
    ev = _events(b.build())
    kind, *args = ev[2]
    assert kind == "cubic"
    assert tuple(args[0]) == (98.0, 0.0) and tuple(args[-1]) == (100.0, 2.0)


def test_rectangle_windings():
    # builder.rs:649-675
    b = PathBuilder()
    b.add_rectangle((1.0, 2.0, 3.0, 5.0), 1)
    b.add_rectangle((1.0, 2.0, 3.0, 5.0), -1)
    p = b.build()
    assert p.verbs.tolist() == [Verb.BEGIN, Verb.LINE_TO, Verb.LINE_TO, Verb.LINE_TO, Verb.CLOSE] * 2
    assert p.points[:4].tolist() == [[1, 2], [3, 2], [3, 5], [1, 5]]
    assert p.points[5:9].tolist() == [[1, 2], [1, 5], [3, 5], [3, 2]]


def test_circle_layout():
    # builder.rs:1508-1548: starts at (cx - r, cy), four cubics, closed; the control points sit
    # at 0.55191505 r along the tangents.
    b = PathBuilder()
    b.add_circle((10.0, 20.0), 4.0, 1)
    p = b.build()
    assert p.verbs.tolist() == [Verb.BEGIN] + [Verb.CUBIC_TO] * 4 + [Verb.CLOSE]
    assert p.points[0].tolist() == [6.0, 20.0]
    d = np.float32(4.0) * np.float32(0.55191505)
    assert p.points[1].tolist() == [6.0, float(np.float32(20.0) + -d)]
    assert p.points[3].tolist() == [10.0, 16.0]
    assert p.points[12].tolist() == [6.0, 20.0]


def test_polygon_open_and_closed():
    b = PathBuilder()
    b.add_polygon([(0, 0), (1, 0), (1, 1)], False)
    b.add_polygon([(0, 0), (1, 0), (1, 1)], True)
    b.add_polygon([], True)
    p = b.build()
    assert p.verbs.tolist() == [Verb.BEGIN, Verb.LINE_TO, Verb.LINE_TO, Verb.END,
                                Verb.BEGIN, Verb.LINE_TO, Verb.LINE_TO, Verb.CLOSE]
