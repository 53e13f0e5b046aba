"""Generates the golden fixtures under tests/golden/ from lyon's own test sources.

Run where a checkout of the lyon repository is available (its location given by
``--reference``). The script reads lyon's Rust test files as text, extracts the paths they build
with `Path::builder()` calls together with the results those tests assert (triangle counts, "must
not fail"), and writes them as JSON. Nothing of lyon is executed: the expectations are the ones
written in the reference tests.

Outputs:
  lyon_fill_cases.json    paths + expected even-odd triangle counts from
                          crates/tessellation/src/fill_tests.rs
  lyon_stroke_cases.json  paths from the stroke tests in crates/tessellation/src/stroke.rs with
                          their asserted triangle counts / properties
  lyon_flatten_cases.json curves and asserted counts from crates/geom/src/quadratic_bezier.rs and
                          crates/geom/src/cubic_bezier.rs
  lyon_fuzz_cases.json    the polygons of crates/tessellation/src/fuzz_tests.rs (lyon's own
                          regression cases: the fill must succeed with both fill rules)
  rust_logo.json          the rust logo path of crates/extra/src/rust_logo.rs (lyon's own test
                          data), converted from its SVG-builder calls to absolute verbs/points
                          with f32 arithmetic (crates/path/src/builder.rs:1193-1480 semantics)

Usage: python tests/golden/make_golden.py --reference PATH  (a checkout of lyon's sources)
"""

import argparse
import json
import os
import re
from fractions import Fraction

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))

VERB_LINE, VERB_QUAD, VERB_CUBIC, VERB_BEGIN, VERB_CLOSE, VERB_END = 0, 1, 2, 3, 4, 5


def f32(lit):
    """Correctly rounded float32 value of a decimal literal (as rustc parses `1.5` into f32)."""
    lit = lit.strip().replace("_", "")
    lit = re.sub(r"f32$|f64$", "", lit)
    exact = Fraction(lit)
    approx = np.float32(float(exact))
    best = approx
    for cand in (np.nextafter(approx, np.float32(-np.inf)), np.nextafter(approx, np.float32(np.inf))):
        d_best = abs(Fraction(float(best)) - exact)
        d_cand = abs(Fraction(float(cand)) - exact)
        if d_cand < d_best or (d_cand == d_best and (int(cand.view(np.uint32)) & 1) == 0):
            best = cand
    return float(best)


NUM = r"-?\d[\d_]*(?:\.\d*)?(?:[eE][-+]?\d+)?(?:f32|f64)?"
POINT = rf"point\(\s*({NUM})\s*,\s*({NUM})\s*\)"


class PathBuild:
    """Collects verbs/points in lyon's Path layout (crates/path/src/path.rs:472-597)."""

    def __init__(self):
        self.verbs = []
        self.points = []
        # The first endpoint attribute of every point (lyon stores attributes per endpoint;
        # control points get 0.0, which nothing reads).
        self.widths = []
        self.first = None
        self.first_w = 0.0
        self.open = False

    def begin(self, p, w=0.0):
        self.first = p
        self.first_w = w
        self.points.append(p)
        self.widths.append(w)
        self.verbs.append(VERB_BEGIN)
        self.open = True

    def line_to(self, p, w=0.0):
        self.points.append(p)
        self.widths.append(w)
        self.verbs.append(VERB_LINE)

    def quad_to(self, c, p, w=0.0):
        self.points += [c, p]
        self.widths += [0.0, w]
        self.verbs.append(VERB_QUAD)

    def cubic_to(self, c1, c2, p, w=0.0):
        self.points += [c1, c2, p]
        self.widths += [0.0, 0.0, w]
        self.verbs.append(VERB_CUBIC)

    def end(self, close):
        if close:
            self.points.append(self.first)
            self.widths.append(self.first_w)
        self.verbs.append(VERB_CLOSE if close else VERB_END)
        self.open = False


def split_tests(src):
    """Yields (name, line, body) for every `#[test] fn name()` in a Rust source."""
    lines = src.split("\n")
    starts = [i for i, l in enumerate(lines) if l.strip() == "#[test]"]
    for k, s in enumerate(starts):
        m = None
        for j in range(s + 1, min(s + 4, len(lines))):
            m = re.match(r"\s*fn\s+(\w+)\s*\(", lines[j])
            if m:
                break
        if not m:
            continue
        end = starts[k + 1] if k + 1 < len(starts) else len(lines)
        body = "\n".join(lines[s:end])
        yield m.group(1), s + 1, body


CALL_RE = re.compile(
    r"\b(\w+)\.(begin|line_to|quadratic_bezier_to|cubic_bezier_to|end|close|move_to)\s*\(")


def parse_builder_calls(body):
    """Parses builder calls in order. Returns a PathBuild or None if something is unsupported."""
    pb = PathBuild()
    svg_open = False
    pos = 0
    for m in CALL_RE.finditer(body):
        if m.start() < pos:
            continue
        method = m.group(2)
        # Grab the argument text up to the matching parenthesis.
        depth, i = 1, m.end()
        while i < len(body) and depth:
            if body[i] == "(":
                depth += 1
            elif body[i] == ")":
                depth -= 1
            i += 1
        args = body[m.end():i - 1]
        pos = i
        pts = [(f32(a), f32(b)) for a, b in re.findall(POINT, args)]
        attr = re.search(r"&\[\s*(" + NUM + r")", args)
        w = f32(attr.group(1)) if attr else 0.0
        if method == "begin":
            if len(pts) != 1:
                return None
            pb.begin(pts[0], w)
        elif method == "move_to":
            if len(pts) != 1:
                return None
            if svg_open:
                pb.end(False)
            pb.begin(pts[0])
            svg_open = True
        elif method == "line_to":
            if len(pts) != 1 or not pb.open:
                return None
            pb.line_to(pts[0], w)
        elif method == "quadratic_bezier_to":
            if len(pts) != 2 or not pb.open:
                return None
            pb.quad_to(*pts, w)
        elif method == "cubic_bezier_to":
            if len(pts) != 3 or not pb.open:
                return None
            pb.cubic_to(*pts, w)
        elif method == "end":
            a = args.strip()
            if a not in ("true", "false"):
                return None
            pb.end(a == "true")
        elif method == "close":
            if not pb.open:
                return None
            pb.end(True)
            svg_open = False
    if svg_open and pb.open:
        pb.end(False)
    return pb


def fill_cases(ref):
    path = os.path.join(ref, "crates/tessellation/src/fill_tests.rs")
    src = open(path).read()
    cases = []
    unsupported = ("build_logo_path", "for ", "transformed", "catch_unwind", "with_svg()",
                   "flattened(", "builder_with_attributes", "arc(", "add_", "Box2D")
    for name, line, body in split_tests(src):
        calls = re.findall(r"(test_path_and_count_triangles|test_path_with_rotations|test_path)\(",
                           body)
        if not calls or any(u in body for u in unsupported):
            continue
        pb = parse_builder_calls(body)
        if pb is None or not pb.verbs or pb.open:
            continue
        expect = None
        rot = None
        m = re.search(r"test_path_and_count_triangles\([^,]+,\s*(\d+)\s*\)", body)
        if m:
            expect = int(m.group(1))
        m = re.search(rf"test_path_with_rotations\([^,]+,\s*({NUM})\s*,\s*(Some\((\d+)\)|None)",
                      body)
        if m:
            rot = float(m.group(1))
            expect = int(m.group(3)) if m.group(3) else None
        cases.append({
            "name": name,
            "src": f"crates/tessellation/src/fill_tests.rs:{line}",
            "verbs": pb.verbs,
            "points": pb.points,
            "expect_even_odd_triangles": expect,
            "rotation_step": rot,
        })
    # The empty path (fill_tests.rs: test_empty_path) asserts 0 triangles.
    return cases


def stroke_cases(ref):
    """Stroke tests of crates/tessellation/src/stroke.rs that the fixed-width path covers."""
    path = os.path.join(ref, "crates/tessellation/src/stroke.rs")
    src = open(path).read()
    tests = {name: (line, body) for name, line, body in split_tests(src)}
    out = []

    def add(name, pb, options, expect, **extra):
        line = tests[name][0]
        d = {"name": name, "src": f"crates/tessellation/src/stroke.rs:{line}",
             "verbs": pb.verbs, "points": pb.points, "options": options,
             "expect_triangles": expect}
        d.update(extra)
        out.append(d)

    # test_square: expected counts are literal in the test.
    line, body = tests["test_square"]
    pb = parse_builder_calls(body)
    counts = [int(x) for x in re.findall(r"Some\((\d+)\)", body)]
    assert counts == [12, 16], counts
    add("test_square", pb, {"line_join": "Miter", "line_cap": "Butt"}, counts[0])
    add("test_square", pb, {"line_join": "Bevel", "line_cap": "Square"}, counts[1])
    add("test_square", pb, {"line_join": "MiterClip", "miter_limit": 1.0, "line_cap": "Round"},
        None)
    add("test_square", pb, {"tolerance": 0.001, "line_join": "Round", "line_cap": "Round"}, None)

    line, body = tests["test_empty_caps"]
    pb = parse_builder_calls(body)
    m = re.findall(r"with_line_cap\(LineCap::(\w+)\),\s*(Some\((\d+)\)|None)", body)
    for cap, _, n in m:
        add("test_empty_caps", pb, {"line_cap": cap}, int(n) if n else None)

    add("test_empty_path", PathBuild(), {}, 0)

    for name in ("single_segment_closed", "issue_819"):
        line, body = tests[name]
        # Only the first path of each test (the fixed-width one).
        first = body.split("let path = path.build()")[0] if name == "single_segment_closed" \
            else body.split("let mut tess")[0]
        pb = parse_builder_calls(first)
        tol = re.search(rf"StrokeOptions::tolerance\(({NUM})\)", body).group(1)
        add(name, pb, {"tolerance": f32(tol)}, None, must_succeed=True,
            nonempty=(name == "single_segment_closed"))

    line, body = tests["test_triangle_winding"]
    pb = parse_builder_calls(body)
    add("test_triangle_winding", pb, {"tolerance": 0.05}, None, winding_nonpositive=True)

    line, body = tests["test_line_width"]
    pb = parse_builder_calls(body)
    add("test_line_width", pb, {"line_width": 2.0}, None,
        vertices_in=[[0.0, 0.0], [0.0, 2.0], [2.0, 0.0], [2.0, 2.0]])

    # The variable-line-width runs of test_square and test_empty_caps (the same expectations,
    # StrokeOptions::default().with_variable_line_width(0)) and the variable-width regressions.
    for name in ("test_square", "test_empty_caps"):
        line, body = tests[name]
        assert "with_variable_line_width(0)" in body
        pb = parse_builder_calls(body)
        for c in [c for c in out if c["name"] == name]:
            d = dict(c)
            d["options"] = dict(c["options"], variable_line_width=True)
            d["widths"] = pb.widths
            out.append(d)
    for name, tol_re in (("issue_821", r"with_tolerance\((" + NUM + r")\)"),
                         ("issue_894", r"StrokeOptions::tolerance\((" + NUM + r")\)")):
        line, body = tests[name]
        assert "with_variable_line_width" in body and "LineCap::Round" in body
        pb = parse_builder_calls(body)
        tol = re.search(tol_re, body).group(1)
        add(name, pb, {"tolerance": f32(tol), "line_cap": "Round",
                       "variable_line_width": True}, None,
            widths=pb.widths, must_succeed=(name == "issue_821"), no_internal_error=True)

    line, body = tests["correct_miter_clip_length"]
    pb = PathBuild()
    pb.begin((-70.0, -200.0))
    pb.line_to((0.0, 300.0))
    pb.line_to((70.0, -200.0))
    pb.end(False)
    assert "point(-70.0, -200.0)" in body and "path_max_y = 300.0" in body
    add("correct_miter_clip_length", pb,
        {"line_width": 30.0, "line_join": "MiterClip", "miter_limit": 3.0}, None,
        max_y=300.0 + 30.0 * 3.0 * 0.5)
    return out


def flatten_cases(ref):
    q = os.path.join(ref, "crates/geom/src/quadratic_bezier.rs")
    c = os.path.join(ref, "crates/geom/src/cubic_bezier.rs")
    qs = {n: (l, b) for n, l, b in split_tests(open(q).read())}
    cs = {n: (l, b) for n, l, b in split_tests(open(c).read())}
    out = []

    def pts(body):
        return [(f32(a), f32(b)) for a, b in re.findall(POINT.replace("point", r"(?:point|Point::new)"),
                                                        body)]

    for name in ("test_flattening_empty_curve", "test_flattening_straight_line"):
        line, body = qs[name]
        p = pts(body)[:3]
        out.append({"name": name, "src": f"crates/geom/src/quadratic_bezier.rs:{line}",
                    "kind": "quadratic", "points": p, "tolerance": 0.1, "expect_count": 1})
    line, body = qs["test_flattened_t_values_are_monotonic"]
    out.append({"name": "test_flattened_t_values_are_monotonic",
                "src": f"crates/geom/src/quadratic_bezier.rs:{line}", "kind": "quadratic",
                "points": pts(body)[:3], "tolerance": 0.01, "expect_min_count": 3})
    for name, tols, prop in (("test_issue_194", [0.1], "more_than_2"),
                             ("flatten_with_t", [0.1, 0.01, 0.001, 0.0001], "within_tolerance"),
                             ("test_flatten_end", [0.0001], "ends_at_to"),
                             ("test_flatten_point", [0.0001], "ends_at_to"),
                             ("issue_652", [1.0, 0.1, 0.01], "terminates")):
        line, body = cs[name]
        p = pts(body)[:4]
        for t in tols:
            out.append({"name": name, "src": f"crates/geom/src/cubic_bezier.rs:{line}",
                        "kind": "cubic", "points": p, "tolerance": t, "property": prop})
    return out


def rust_logo(ref):
    """Replays crates/extra/src/rust_logo.rs through the WithSvg semantics in f32."""
    src = open(os.path.join(ref, "crates/extra/src/rust_logo.rs")).read()
    calls = re.findall(r"path\.(\w+)\(([^;]*?)\);", src, flags=re.S)
    F = np.float32
    pb = PathBuild()
    cur = (F(0), F(0))
    first = cur
    last_cmd = None
    last_ctrl = cur
    need_moveto = True

    def vec(args):
        return [(F(f32(a)), F(f32(b))) for a, b in
                re.findall(rf"(?:vector|point)\(\s*({NUM})\s*,\s*({NUM})\s*\)", args)]

    def rel(v):
        return (F(cur[0] + v[0]), F(cur[1] + v[1]))

    def emit_line(to):
        nonlocal cur, last_cmd, need_moveto
        if need_moveto:
            moveto(first)
        cur = to
        last_cmd = "line"
        pb.line_to((float(to[0]), float(to[1])))

    def emit_cubic(c1, c2, to):
        nonlocal cur, last_cmd, last_ctrl, need_moveto
        if need_moveto:
            moveto(first)
        cur = to
        last_cmd = "cubic"
        last_ctrl = c2
        pb.cubic_to((float(c1[0]), float(c1[1])), (float(c2[0]), float(c2[1])),
                    (float(to[0]), float(to[1])))

    def moveto(p):
        nonlocal cur, first, last_cmd, need_moveto
        if last_cmd in ("line", "cubic", "begin"):
            pb.end(False)
        pb.begin((float(p[0]), float(p[1])))
        need_moveto = False
        first = p
        cur = p
        last_cmd = "begin"

    for name, args in calls:
        if name == "move_to":
            moveto(vec(args)[0])
        elif name == "close":
            if need_moveto:
                continue
            cur = first
            need_moveto = True
            last_cmd = "close"
            pb.end(True)
        elif name == "line_to":
            emit_line(vec(args)[0])
        elif name == "relative_line_to":
            emit_line(rel(vec(args)[0]))
        elif name == "horizontal_line_to":
            emit_line((F(f32(args)), cur[1]))
        elif name == "relative_horizontal_line_to":
            emit_line((F(cur[0] + F(f32(args))), cur[1]))
        elif name == "vertical_line_to":
            emit_line((cur[0], F(f32(args))))
        elif name == "relative_vertical_line_to":
            emit_line((cur[0], F(cur[1] + F(f32(args)))))
        elif name == "cubic_bezier_to":
            c1, c2, to = vec(args)
            emit_cubic(c1, c2, to)
        elif name == "relative_cubic_bezier_to":
            c1, c2, to = vec(args)
            to_a = rel(to)
            emit_cubic(rel(c1), rel(c2), to_a)
        elif name in ("smooth_cubic_bezier_to", "smooth_relative_cubic_bezier_to"):
            c2, to = vec(args)
            if last_cmd == "cubic":
                c1 = (F(cur[0] + F(cur[0] - last_ctrl[0])), F(cur[1] + F(cur[1] - last_ctrl[1])))
            else:
                c1 = cur
            if name == "smooth_relative_cubic_bezier_to":
                c2 = rel(c2)
                to = rel(to)
            emit_cubic(c1, c2, to)
        else:
            raise ValueError(f"unsupported logo command {name}")
    if last_cmd in ("line", "cubic", "begin"):
        pb.end(False)
    return {"src": "crates/extra/src/rust_logo.rs:5", "verbs": pb.verbs, "points": pb.points}


def fuzz_cases(ref):
    """crates/tessellation/src/fuzz_tests.rs: every test builds a polygon path with builder calls
    and asserts that filling it (after flattening at 0.05) succeeds with both fill rules."""
    path = os.path.join(ref, "crates/tessellation/src/fuzz_tests.rs")
    src = open(path).read()
    out = []
    for name, line, body in split_tests(src):
        if "test_path(" not in body:
            continue
        pb = parse_builder_calls(body)
        if pb is None or not pb.verbs or pb.open:
            continue
        out.append({"name": name, "src": f"crates/tessellation/src/fuzz_tests.rs:{line}",
                    "verbs": pb.verbs, "points": pb.points})
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", required=True, help="a checkout of lyon's sources")
    a = ap.parse_args()
    outputs = {
        "lyon_fill_cases.json": fill_cases(a.reference),
        "lyon_stroke_cases.json": stroke_cases(a.reference),
        "lyon_flatten_cases.json": flatten_cases(a.reference),
        "lyon_fuzz_cases.json": fuzz_cases(a.reference),
        "rust_logo.json": rust_logo(a.reference),
    }
    for fname, data in outputs.items():
        with open(os.path.join(HERE, fname), "w") as f:
            json.dump(data, f, indent=None, separators=(",", ":"))
        n = len(data) if isinstance(data, list) else len(data["verbs"])
        print(f"wrote {fname}: {n} entries")


if __name__ == "__main__":
    main()
