"""Elliptic arcs on the CPU: the oracle's Arc::for_each_flattened_with_t
(crates/geom/src/arc.rs:339-389) against lyon's own arc tests, the path builder's quadratic
approximation (arc.rs:668-703, lyon's test_to_quadratics_and_cubics) and its ellipses
(crates/path/src/builder.rs:606-636)."""

import math

import numpy as np

from oracle import lyon_oracle as orc
from lyon_gb300.options import FillOptions, StrokeOptions
from lyon_gb300.path import PathBuilder, Verb, arc_quadratic_beziers


def _arcs(rows):
    a = np.zeros(len(rows), orc.ARC_DTYPE)
    for i, r in enumerate(rows):
        a[i] = r
    return a


def test_negative_flattening_step():
    # arc.rs:1207-1236: the first arc once never converged (sweep -898 rad); the second, with a
    # negative sweep, was flattened to a single segment.
    a = _arcs([(-100.0, -150.0, 50.0, 50.0, 0.982944787, -898.0, 0.0),
               (0.0, 0.0, 100.0, 10.0, 0.2, -2.0, 0.0)])
    pts, ts, offs, st = orc.flatten_arcs(a, 0.100000001)
    assert list(st) == [0, 0]
    assert offs[1] - offs[0] > 2
    assert offs[2] - offs[1] - 1 > 1  # segments after the start point


def test_flattening_properties_circles():
    rng = np.random.default_rng(3)
    n = 300
    a = np.zeros(n, orc.ARC_DTYPE)
    a["center_x"] = rng.uniform(-100, 100, n)
    a["center_y"] = rng.uniform(-100, 100, n)
    r = rng.uniform(0.5, 200, n).astype(np.float32)
    a["radius_x"] = r
    a["radius_y"] = r
    a["start_angle"] = rng.uniform(-7, 7, n)
    a["sweep_angle"] = rng.uniform(-12, 12, n)
    a["x_rotation"] = rng.uniform(-3, 3, n)
    tol = 0.05
    pts, ts, offs, st = orc.flatten_arcs(a, tol)
    assert np.all(st == 0)
    for i in range(n):
        p = pts[offs[i]:offs[i + 1]].astype(np.float64)
        t = ts[offs[i]:offs[i + 1]]
        assert t[0] == 0.0 and t[-1] == 1.0 and np.all(np.diff(t) > 0)
        c = np.array([a["center_x"][i], a["center_y"][i]], np.float64)
        d = np.linalg.norm(p - c, axis=1)
        assert np.allclose(d, r[i], rtol=1e-5, atol=1e-3)
        # Every chord stays within the tolerance of the circle (its sagitta).
        chord = np.linalg.norm(np.diff(p, axis=0), axis=1)
        sag = r[i] - np.sqrt(np.maximum(r[i] ** 2 - (chord / 2) ** 2, 0))
        assert np.all(sag <= tol * 1.01 + 1e-4)


def test_arc_to_quadratics_counts():
    # arc.rs:941-1016 (quadratic counts 4, 4, 1, 1), with the segments joined end to end.
    cases = [(((2.0, 3.0), (10.0, 3.0), 0.1, 3.0, 0.5), 4),
             (((4.0, 5.0), (3.0, 5.0), 2.0, -3.0, 1.3), 4),
             (((0.0, 0.0), (100.0, 0.01), -1.0, 0.1, 0.3), 1),
             (((0.0, 0.0), (1.0, 1.0), 3.0, -0.1, -0.3), 1)]
    for args, count in cases:
        q = arc_quadratic_beziers(*args)
        assert len(q) == count
        for (_, _, to, _, t1), (frm, _, _, t0, _) in zip(q, q[1:]):
            assert np.allclose(to, frm, atol=1e-5) and t1 == t0
        assert q[-1][4] == 1.0


def test_add_ellipse_layout():
    b = PathBuilder()
    b.add_ellipse((10.0, 20.0), (30.0, 5.0), 0.3, 1)
    b.add_ellipse((-5.0, 2.0), (4.0, 9.0), -1.0, -1)
    p = b.build()
    quad = [Verb.BEGIN] + [Verb.QUADRATIC_TO] * 8 + [Verb.CLOSE]
    assert list(p.verbs) == quad + quad
    first = p.points[0]
    last_to = p.points[16]  # the eighth quadratic's end point
    assert np.allclose(first, last_to, atol=1e-4)
    # Every endpoint lies on the rotated ellipse.
    c, s = math.cos(0.3), math.sin(0.3)
    for k in range(2, 17, 2):
        x, y = p.points[k] - np.array([10.0, 20.0], np.float32)
        u, v = x * c + y * s, -x * s + y * c
        assert abs((u / 30.0) ** 2 + (v / 5.0) ** 2 - 1.0) < 1e-4


def test_ellipse_tessellates_on_the_oracle():
    b = PathBuilder()
    b.add_ellipse((0.0, 0.0), (50.0, 20.0), 0.25, 1)
    p = b.build()
    f = orc.fill(p, FillOptions(handle_intersections=False), 32)
    s = orc.stroke(p, StrokeOptions(line_width=2.0), 32)
    assert f.status == 0 and f.num_triangles > 0
    assert s.status == 0 and s.num_triangles > 0
