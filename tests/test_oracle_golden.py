"""Pins the oracle (CPU restatement of lyon) against lyon's own known-answer tests.

Every expectation comes from the reference test sources, extracted into tests/golden/ by
tests/golden/make_golden.py: fill triangle counts (crates/tessellation/src/fill_tests.rs),
stroke triangle counts and properties (crates/tessellation/src/stroke.rs tests), flattening
properties (crates/geom/src/quadratic_bezier.rs, cubic_bezier.rs tests).
"""

import math
import os

import numpy as np
import pytest

from oracle import lyon_oracle as orc
from lyon_gb300.options import FillOptions, FillRule, LineCap, LineJoin, StrokeOptions
from lyon_gb300.path import Path, PathBuilder

from lyon_cases import (case_path, flatten_to_lines, load, rotation_angles, rust_logo,
                        stroke_options_from_case)

FULL = os.environ.get("LYON_FULL_ROTATIONS") == "1"


def lyon_fill_test(path: Path, rule: int):
    """crates/tessellation/src/fill_tests.rs:10-28: flatten at 0.05, fill at 0.05, u16."""
    counts, pts = orc.flatten(path, 0.05)
    flat = flatten_to_lines(path, counts, pts)
    r = orc.fill(flat, FillOptions(tolerance=0.05, fill_rule=rule), index_bits=16)
    return r


FILL_CASES = load("lyon_fill_cases.json")


@pytest.mark.parametrize("case", FILL_CASES, ids=[c["name"] for c in FILL_CASES])
def test_fill_kat(case):
    path = case_path(case)
    expect = case["expect_even_odd_triangles"]
    if case["rotation_step"] is None:
        paths = [path]
    else:
        angles = list(rotation_angles(case["rotation_step"]))
        if not FULL and len(angles) > 400:
            angles = angles[::max(1, len(angles) // 400)]
        paths = [path.transformed_rotation(a) for a in angles]
    for p in paths:
        r = lyon_fill_test(p, FillRule.EvenOdd)
        assert r.status == 0, f"{case['src']}: even-odd failed with status {r.status}"
        if expect is not None:
            assert r.num_triangles == expect, f"{case['src']}: {r.num_triangles} != {expect}"
        r = lyon_fill_test(p, FillRule.NonZero)
        assert r.status == 0, f"{case['src']}: non-zero failed with status {r.status}"


def test_fill_empty_path():
    # fill_tests.rs test_empty_path: 0 triangles.
    r = lyon_fill_test(Path.from_arrays([], np.zeros((0, 2))), FillRule.EvenOdd)
    assert r.status == 0 and r.num_triangles == 0


@pytest.mark.parametrize("scale", [None, 260.0, 0.005, 0.0000001])
def test_fill_rust_logo(scale):
    # fill_tests.rs test_rust_logo_no_intersection / _scale_up / _scale_down(2).
    logo = rust_logo()
    if scale == 260.0:
        paths = [logo.scaled(scale)]
    else:
        counts, pts = orc.flatten(logo, 0.011)
        flat = flatten_to_lines(logo, counts, pts)
        if scale is not None:
            paths = [flat.scaled(scale)]
        else:
            angles = list(rotation_angles(0.011))
            if not FULL:
                angles = angles[::8]
            paths = [flat.transformed_rotation(a) for a in angles]
    for p in paths:
        for rule in (FillRule.EvenOdd, FillRule.NonZero):
            r = lyon_fill_test(p, rule)
            assert r.status == 0


def test_fill_rust_logo_with_intersection():
    # fill_tests.rs test_rust_logo_with_intersection.
    logo = rust_logo()
    counts, pts = orc.flatten(logo, 0.011)
    flat = flatten_to_lines(logo, counts, pts)
    verbs = list(flat.verbs) + [3, 0, 0, 0, 4]
    points = list(map(tuple, flat.points)) + [(10.0, 30.0), (130.0, 30.0), (130.0, 60.0),
                                              (10.0, 60.0), (10.0, 30.0)]
    p = Path.from_arrays(verbs, points)
    angles = list(rotation_angles(0.011))
    if not FULL:
        angles = angles[::8]
    for a in angles:
        q = p.transformed_rotation(a)
        for rule in (FillRule.EvenOdd, FillRule.NonZero):
            assert lyon_fill_test(q, rule).status == 0


def test_fill_triangle_winding():
    # fill_tests.rs test_triangle_winding: every triangle has (b - a) x (c - b) <= 0.
    r = orc.fill(rust_logo(), FillOptions(tolerance=0.05))
    assert r.status == 0 and r.num_triangles > 0
    v = r.vertices.astype(np.float32)
    t = r.indices32.reshape(-1, 3)
    a, b, c = v[t[:, 0]], v[t[:, 1]], v[t[:, 2]]
    ba = (b - a).astype(np.float32)
    cb = (c - b).astype(np.float32)
    cross = (ba[:, 0] * cb[:, 1] - ba[:, 1] * cb[:, 0]).astype(np.float32)
    assert (cross <= 0).all()


def test_fill_too_many_vertices():
    # fill_tests.rs test_too_many_vertices: a builder that runs out of ids after 0/10/100
    # vertices returns TooManyVertices. A u16 builder whose offset leaves that many ids free
    # behaves the same way.
    for free in (0, 10, 100):
        r = orc.fill(rust_logo(), FillOptions(tolerance=0.05), index_bits=16,
                     vertex_offset=65536 - free)
        assert r.status == 3 and len(r.vertices) == 0 and len(r.indices) == 0


def test_fill_overflow_with_vertex_offset():
    # geometry_builder.rs overflow_with_vertex_offset: ids 65534 and 65535 fit, the third fails.
    b = PathBuilder()
    b.begin((0, 0))
    b.line_to((1, 0))
    b.line_to((0, 1))
    b.end(True)
    r = orc.fill(b.build(), FillOptions(), index_bits=16, vertex_offset=65534)
    assert r.status == 3 and len(r.vertices) == 0


STROKE_CASES = load("lyon_stroke_cases.json")


def check_stroke_builder_asserts(r):
    """The TestBuilder of stroke.rs:2787-2849: distinct indices, cross >= -0.035, no NaN; with
    attributes, no NaN normal or advancement and no zero normal (stroke.rs:2817-2826)."""
    v = r.vertices.astype(np.float32)
    assert not np.isnan(v).any()
    if r.attributes is not None:
        f = r.attributes[:, :3].copy().view(np.float32)
        assert not np.isnan(f).any()
        assert ((f[:, 0] * f[:, 0] + f[:, 1] * f[:, 1]) != 0.0).all()
    t = r.indices32.reshape(-1, 3).astype(np.int64)
    assert (t[:, 0] != t[:, 1]).all() and (t[:, 0] != t[:, 2]).all() and (t[:, 1] != t[:, 2]).all()
    pa, pb, pc = v[t[:, 0]], v[t[:, 1]], v[t[:, 2]]
    ab = (pa - pb).astype(np.float32)
    cb = (pc - pb).astype(np.float32)
    cross = (ab[:, 0] * cb[:, 1] - ab[:, 1] * cb[:, 0]).astype(np.float32)
    assert (cross >= -0.035).all()


@pytest.mark.parametrize("case", STROKE_CASES,
                         ids=[f"{c['name']}-{i}" for i, c in enumerate(STROKE_CASES)])
def test_stroke_kat(case):
    path = case_path(case)
    opts = stroke_options_from_case(case["options"])
    widths = case.get("widths") if case["options"].get("variable_line_width") else None
    r = orc.stroke(path, opts, index_bits=16, attributes=True, widths=widths)
    if case.get("no_internal_error"):
        # The test only requires that lyon does not panic (the result is discarded).
        assert r.status != 5, case["src"]
        return
    assert r.status == 0, case["src"]
    if case["name"] in ("test_square", "test_empty_caps", "test_empty_path"):
        # These go through stroke.rs `test_path`, whose TestBuilder asserts per triangle.
        check_stroke_builder_asserts(r)
    if case["expect_triangles"] is not None:
        assert r.num_triangles == case["expect_triangles"], case["src"]
    if case.get("nonempty"):
        assert len(r.indices) > 0
    if case.get("winding_nonpositive"):
        v = r.vertices
        t = r.indices32.reshape(-1, 3)
        a, b, c = v[t[:, 0]], v[t[:, 1]], v[t[:, 2]]
        ba = (b - a).astype(np.float32)
        cb = (c - b).astype(np.float32)
        assert ((ba[:, 0] * cb[:, 1] - ba[:, 1] * cb[:, 0]).astype(np.float32) <= 0).all()
    if "vertices_in" in case:
        allowed = np.array(case["vertices_in"], np.float32)
        for p in r.vertices:
            assert np.min(np.abs(allowed - p).max(axis=1)) < 1e-5
    if "max_y" in case:
        assert float(r.vertices[:, 1].max()) == case["max_y"]


def _adv(r):
    return r.attributes[:, 2].copy().view(np.float32)


def test_stroke_attributes_advancement_and_sides():
    # A right angle, miter join within the limit, butt caps: the join's two vertices at
    # advancement 10, the end's at 20, the start's at 0; one vertex per side each time.
    p = Path.builder()
    p.begin((0.0, 0.0))
    p.line_to((10.0, 0.0))
    p.line_to((10.0, 10.0))
    p.end(False)
    r = orc.stroke(p.build(), StrokeOptions(line_width=2.0), attributes=True)
    assert r.status == 0
    assert sorted(_adv(r).tolist()) == [0.0, 0.0, 10.0, 10.0, 20.0, 20.0]
    for a in (0.0, 10.0, 20.0):
        assert sorted(r.attributes[_adv(r) == a, 3].tolist()) == [0, 1]
    # Positions are position_on_path + normal * half_width.
    n = r.attributes[:, :2].copy().view(np.float32)
    on_path = {0.0: (0.0, 0.0), 10.0: (10.0, 0.0), 20.0: (10.0, 10.0)}
    for k in range(len(r.vertices)):
        c = np.array(on_path[float(_adv(r)[k])], np.float32)
        assert np.allclose(r.vertices[k], c + n[k] * np.float32(1.0), atol=1e-6)


def test_stroke_attributes_advancement_across_sub_paths():
    # end_with_caps carries the end advancement into the next sub-path (stroke.rs:1359); a
    # closed sub-path does not (close() leaves sub_path_start_advancement alone).
    p = Path.builder()
    p.begin((0.0, 0.0))
    p.line_to((10.0, 0.0))
    p.end(False)
    p.begin((0.0, 5.0))
    p.line_to((0.0, 8.0))
    p.end(False)
    r = orc.stroke(p.build(), StrokeOptions(line_width=2.0), attributes=True)
    assert sorted(set(_adv(r).tolist())) == [0.0, 10.0, 13.0]
    p = Path.builder()
    p.begin((0.0, 0.0))
    p.line_to((10.0, 0.0))
    p.line_to((10.0, 10.0))
    p.end(True)
    p.begin((0.0, 20.0))
    p.line_to((5.0, 20.0))
    p.end(False)
    r = orc.stroke(p.build(), StrokeOptions(line_width=2.0), attributes=True)
    a = _adv(r)
    # The closed triangle: 0, 10, 20 and the closing join at 20 + 10*sqrt(2); then 0 and 5.
    tail = a[-4:]
    assert sorted(tail.tolist()) == [0.0, 0.0, 5.0, 5.0]
    assert np.isclose(a.max(), 20.0 + 10.0 * math.sqrt(2.0), atol=1e-4)


def test_stroke_too_many_vertices():
    # stroke.rs test_too_many_vertices: the logo at tolerance 0.05 with 0/10/100 free ids.
    for free in (0, 10, 100):
        r = orc.stroke(rust_logo(), StrokeOptions(tolerance=0.05), index_bits=16,
                       vertex_offset=65536 - free)
        assert r.status == 3 and len(r.vertices) == 0 and len(r.indices) == 0


def test_stroke_logo_all_joins_and_caps():
    # Not a lyon assertion by itself: the logo through every join/cap combination must succeed
    # and satisfy the stroke TestBuilder assertions.
    logo = rust_logo()
    for join in (LineJoin.Miter, LineJoin.MiterClip, LineJoin.Round, LineJoin.Bevel):
        for cap in (LineCap.Butt, LineCap.Square, LineCap.Round):
            r = orc.stroke(logo, StrokeOptions(line_join=join, tolerance=0.05).with_line_cap(cap))
            assert r.status == 0
            assert r.num_triangles > 0
            assert not np.isnan(r.vertices).any()


FLATTEN_CASES = load("lyon_flatten_cases.json")


def _flatten_curve(case):
    pts = case["points"]
    b = PathBuilder()
    b.begin(pts[0])
    if case["kind"] == "quadratic":
        b.quadratic_bezier_to(pts[1], pts[2])
    else:
        b.cubic_bezier_to(pts[1], pts[2], pts[3])
    b.end(False)
    counts, out = orc.flatten(b.build(), case["tolerance"])
    return int(counts[1]), out


def _sample(case, t):
    p = [np.array(x, np.float64) for x in case["points"]]
    if case["kind"] == "quadratic":
        return (1 - t) ** 2 * p[0] + 2 * (1 - t) * t * p[1] + t * t * p[2]
    return ((1 - t) ** 3 * p[0] + 3 * (1 - t) ** 2 * t * p[1] + 3 * (1 - t) * t * t * p[2]
            + t ** 3 * p[3])


@pytest.mark.parametrize("case", FLATTEN_CASES,
                         ids=[f"{c['name']}-{c['tolerance']}" for c in FLATTEN_CASES])
def test_flatten_kat(case):
    n, out = _flatten_curve(case)
    if "expect_count" in case:
        assert n == case["expect_count"]
    if "expect_min_count" in case:
        assert n >= case["expect_min_count"]
    prop = case.get("property")
    if prop == "more_than_2":
        assert n > 2
    if prop == "ends_at_to":
        assert tuple(out[-1]) == tuple(np.float32(case["points"][-1]))
    if prop == "within_tolerance":
        # cubic_bezier.rs flatten_with_t: every point lies within tolerance of the curve sample
        # at its t (t accumulated as lyon does).
        w = orc.wang(case["points"], case["tolerance"])
        step = np.float32(1.0) / np.float32(w)
        t = np.float32(0.0)
        for k in range(n - 1):
            t = np.float32(t + step)
            d = np.linalg.norm(_sample(case, float(t)) - out[k].astype(np.float64))
            assert d <= case["tolerance"] + 1e-4


def test_wang_lut_matches_ceil_fourth_root():
    # quadratic_bezier.rs:943-974: within the LUT range, n = ceil(err4^(1/4)) (clamped >= 1);
    # beyond it, the fractional fourth root. Checked over a sweep of control-point distances.
    rng = np.random.default_rng(0)
    for _ in range(2000):
        pts = rng.uniform(-50, 50, size=(3, 2)).astype(np.float32)
        tol = np.float32(rng.choice([0.01, 0.1, 1.0]))
        n = orc.wang(pts, float(tol))
        l = (pts[0] - np.float32(2) * pts[1] + pts[2]) * np.float32(2)
        d = np.float32(1) / (np.float32(8) * tol)
        err4 = np.float32(np.float32(np.float32(l[0] * l[0] + l[1] * l[1]) * d) * d)
        r = float(err4) ** 0.25
        if err4 <= 331776:
            assert n == max(1, math.ceil(r - 1e-9)) or abs(r - round(r)) < 1e-4
        else:
            assert abs(n - r) <= 1e-3 * r


# ---- euclid's angle helpers (euclid 0.22.9, the version lyon's Cargo.lock pins) -------------

def _fast_atan2_f32(y, x):
    """euclid's Trig::fast_atan2 for f32, evaluated with numpy float32 scalars: the published
    polynomial of math.stackexchange question 1098487 (answer 1105038)."""
    f = np.float32
    y, x = f(y), f(x)
    xa, ya = abs(x), abs(y)
    a = f(min(xa, ya) / max(xa, ya))
    s = a * a
    r = ((f(-0.0464964749) * s + f(0.15931422)) * s - f(0.327622764)) * s * a + a
    if ya > xa:
        r = f(math.pi / 2) - r
    if x < 0:
        r = f(math.pi) - r
    if y < 0:
        r = -r
    return f(r)


def test_fast_atan2_is_euclids_polynomial():
    # lyon's join, cap and sharp-turn angles come from Vector2D::angle_from_x_axis, which is
    # euclid's fast_atan2 (stroke.rs:1986-1987, 2482-2483, 3204). The oracle must return that
    # polynomial's f32 value bit for bit, not the libm arctangent.
    L = orc.lib()
    rng = np.random.default_rng(12)
    v = rng.normal(size=(4000, 2)).astype(np.float32) * np.float32(100.0)
    worst = 0.0
    for x, y in v:
        got = np.float32(L.lyon_oracle_fast_atan2(float(y), float(x)))
        assert got == _fast_atan2_f32(y, x)
        worst = max(worst, abs(float(got) - math.atan2(float(y), float(x))))
    # The published method's error (about 2e-4 rad at a = 1); a libm atan2 would be ~1e-7.
    assert 1e-4 < worst < 2.1e-4
    # Axis directions are exact.
    f = lambda y, x: np.float32(L.lyon_oracle_fast_atan2(y, x))
    assert f(0.0, 1.0) == 0.0
    assert f(1.0, 0.0) == np.float32(math.pi / 2)
    assert f(0.0, -1.0) == np.float32(math.pi)
    assert f(-1.0, 0.0) == -np.float32(math.pi / 2)
    assert math.isnan(f(0.0, 0.0))  # 0 / 0, as euclid's


def test_angle_to_is_euclids_remainder_form():
    # Angle::angle_to: d = (to - from) % 2pi; (2 d) % 2pi - d, with exact float remainders.
    L = orc.lib()
    f32 = np.float32
    pi = f32(math.pi)
    two_pi = pi * f32(2)
    cases = [(0.0, 3.0), (0.0, 4.0), (3.0, -3.0), (0.0, float(pi)), (1.0, -2.5), (-3.1, 3.1)]
    for a, b in cases:
        d = f32(math.fmod(f32(f32(b) - f32(a)), two_pi))
        want = f32(f32(math.fmod(f32(2) * d, two_pi)) - d)
        assert np.float32(L.lyon_oracle_angle_to(a, b)) == want
    # Hand-derived values: 4 - 2pi for a turn of 4 rad, and -pi (not +pi) at exactly pi.
    assert np.float32(L.lyon_oracle_angle_to(0.0, 4.0)) == f32(f32(8.0) - two_pi) - f32(4.0)
    assert np.float32(L.lyon_oracle_angle_to(0.0, float(pi))) == -pi


@pytest.mark.parametrize("vw,expect", [(False, (200, 204)), (True, (104, 108))])
def test_square_round_joins_and_caps_counts(vw, expect):
    # stroke.rs test_square, Round joins and Round caps at tolerance 0.001 (lyon asserts only the
    # TestBuilder's per-triangle checks there). Counts derived by hand from stroke.rs:
    # circle_flattening_step(r, 0.001) = 2 acos((r - 0.001) / r); every turn and cap half is a
    # quarter turn (the normals are axis aligned, so fast_atan2 is exact there).
    #   fixed width, r = 0.5: pi/2 / 0.12652 = 12.4 -> 13 segments -> depth round(log2 13) = 4,
    #     15 arc vertices per arc. Per sub-path: 3 edges x 2 triangles; 2 joins x (1 interior
    #     triangle + 15); 2 caps x (1 + 2 x 15) = 6 + 32 + 62 = 100 triangles; 2 sub-paths.
    #     Vertices: 4 end vertices + 2 joins x (3 + 15) + 2 caps x (1 + 30) = 102 per sub-path.
    #   variable width 0.3 (r = 0.15): pi/2 / 0.23112 = 6.8 -> 7 -> depth 3, 7 per arc:
    #     6 + 2 x 8 + 2 x 15 = 52 triangles and 4 + 2 x 10 + 2 x 15 = 54 vertices per sub-path.
    case = next(c for c in STROKE_CASES if c["name"] == "test_square"
                and c["options"].get("line_join") == "Round"
                and bool(c["options"].get("variable_line_width")) == vw)
    opts = stroke_options_from_case(case["options"])
    widths = case.get("widths") if vw else None
    r = orc.stroke(case_path(case), opts, index_bits=16, attributes=True, widths=widths)
    assert r.status == 0
    assert (r.num_triangles, len(r.vertices)) == expect
    assert r.near_ties == 0
    check_stroke_builder_asserts(r)


@pytest.mark.parametrize("vw", [False, True])
def test_empty_round_caps_counts(vw):
    # stroke.rs test_empty_caps with Round caps (default tolerance 0.1, radius 0.5): a quarter
    # turn is pi/2 / (2 acos(0.8)) = 1.22 -> 2 segments -> depth 1, one vertex per arc. Each
    # empty cap: 2 vertices + 2 half caps x (1 mid vertex + 2 arc vertices) = 8 vertices and
    # 2 x (1 + 2) = 6 triangles; the test path has 4 empty sub-paths.
    case = next(c for c in STROKE_CASES if c["name"] == "test_empty_caps"
                and c["options"].get("line_cap") == "Round"
                and bool(c["options"].get("variable_line_width")) == vw)
    opts = stroke_options_from_case(case["options"])
    widths = case.get("widths") if vw else None
    r = orc.stroke(case_path(case), opts, index_bits=16, attributes=True, widths=widths)
    assert r.status == 0
    assert (r.num_triangles, len(r.vertices)) == (24, 32)
    check_stroke_builder_asserts(r)

