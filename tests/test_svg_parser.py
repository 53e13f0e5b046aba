"""The library's SVG path parser (lyon_svg_parse_paths) against lyon_extra's own parser tests
(crates/extra/src/parser.rs:494-769) and, on random path data, against a Python restatement of
the parser (oracle/svg_oracle.py). Host code only: runs without a GPU."""

import numpy as np
import pytest

from lyon_gb300 import svg
from oracle import svg_oracle

KIND = {"number": svg.SVG_ERR_NUMBER, "flag": svg.SVG_ERR_FLAG,
        "command": svg.SVG_ERR_COMMAND, "missing_move_to": svg.SVG_ERR_MISSING_MOVE_TO}


def _one(src, **kw):
    r = svg.parse_paths([src], **kw)
    b = r.batch
    return (b.verbs[b.verb_offsets[0]:b.verb_offsets[1]],
            b.points[b.point_offsets[0]:b.point_offsets[1]], int(r.status[0]),
            int(r.error_line[0]), int(r.error_column[0]),
            r.widths[b.point_offsets[0]:b.point_offsets[1]] if r.widths is not None else None)


def test_empty_square_attr_polyline():
    # parser.rs:495-552 (empty, simple_square, simple_attr, implicit_polyline)
    for s in ("", " "):
        v, p, st, *_ = _one(s)
        assert st == 0 and len(v) == 0
    v, p, st, *_ = _one("M 0 0 L 1 0 L 1 1 L 0 1 Z")
    assert st == 0 and v.tolist() == [3, 0, 0, 0, 4]
    v, p, st, _, _, w = _one("M 0 0 1.0 L 1 0 2.0 L 1 1 3.0 L 0 1 4.0 Z", num_attributes=1)
    assert st == 0 and w.tolist() == [1.0, 2.0, 3.0, 4.0, 1.0]
    v, p, st, _, _, w = _one("0 0 0 1 1 1.0 2 2 2.0 3 3 3", num_attributes=1)
    assert st == 0 and v.tolist() == [3, 0, 0, 0, 5] and w.tolist() == [0.0, 1.0, 2.0, 3.0]


def test_invalid_command_positions():
    # parser.rs:555-592
    _, _, st, line, col, _ = _one("x 0 0 0", num_attributes=1)
    assert (st, line, col) == (svg.SVG_ERR_COMMAND, 0, 0)
    _, _, st, line, col, _ = _one("\n M 0 \n0 1 x 1 1 1", num_attributes=1)
    assert (st, line, col) == (svg.SVG_ERR_COMMAND, 2, 4)


def test_numbers():
    # parser.rs:595-671 (number_01, number_scientific_notation, bad_numbers)
    v, p, st, *_ = _one("M 0.6.5")
    assert st == 0 and v.tolist() == [3, 5]
    assert p.tolist() == [[np.float32(0.6), 0.5]]
    v, p, st, *_ = _one("M 1e-2 -1E3")
    assert st == 0 and p.tolist() == [[np.float32(1e-2), -1000.0]]
    for s in ("M 0 --1", "M 0 1ee2", "M 0 1e--1", "M 0 *2", "M 0 e", "M 0 1e", "M 0 +1"):
        assert _one(s)[2] == svg.SVG_ERR_NUMBER, s


def test_stop_and_need_start():
    # parser.rs:674-737 (stop, need_start)
    for s in ("M 0 0 | xxxxxx", "M 0 0| xxxxxx", "| xxxxxx", "    | xxxxxx"):
        assert _one(s, stop_at="|")[2] == 0, s
    v1, p1, st, *_ = _one("M 0 0 Z L 1 1 2 2 L 3 3 Z M 4 4", stop_at="|")
    assert st == svg.SVG_ERR_MISSING_MOVE_TO
    v2, p2, st2, *_ = _one("M 0 0 Z", stop_at="|")
    assert st2 == 0 and v1.tolist() == v2.tolist() and p1.tolist() == p2.tolist()


def test_issues_895_919():
    # parser.rs:740-769
    for s in ("M 1e-9 0", "M -1e-9 0", "M -1e11 0", "M 1.e-9 1.4e-4z", "M 1.6e-9 1.4e-4 z",
              "M0 1.6e-9L0 1.4e-4"):
        assert _one(s)[2] == 0, s
    _one("0 0M")  # must not crash


def _random_path(rng):
    cmds = []
    for _ in range(int(rng.integers(1, 12))):
        c = rng.choice(list("MmLlHhVvCcSsQqTtAaZz"))
        nums = {"M": 2, "L": 2, "H": 1, "V": 1, "C": 6, "S": 4, "Q": 4, "T": 2, "A": 7, "Z": 0}
        k = nums[c.upper()]
        vals = [f"{x:.3f}" for x in rng.uniform(-100, 100, size=k)]
        if c.upper() == "A":
            vals[0] = f"{abs(rng.uniform(0, 60)):.2f}"
            vals[1] = f"{abs(rng.uniform(0, 60)):.2f}"
            vals[3] = str(int(rng.integers(0, 2)))
            vals[4] = str(int(rng.integers(0, 2)))
        sep = rng.choice([" ", ",", "  ", "\n"])
        cmds.append(c + sep + sep.join(vals))
    return " ".join(cmds)


def test_random_paths_match_restatement():
    rng = np.random.default_rng(71)
    strings = [_random_path(rng) for _ in range(3000)]
    strings[0] = "M 10 10 a 5 5 0 0 1 10 0 A 30 20 45 1 0 50 50 z"
    r = svg.parse_paths(strings, num_threads=4)
    b = r.batch
    for i, s in enumerate(strings):
        v = b.verbs[b.verb_offsets[i]:b.verb_offsets[i + 1]]
        p = b.points[b.point_offsets[i]:b.point_offsets[i + 1]]
        ov, op, ow, err = svg_oracle.parse(s)
        ek = KIND[err[0]] if err else 0
        assert int(r.status[i]) == ek, (s, err)
        if err:
            assert (int(r.error_line[i]), int(r.error_column[i])) == (err[1], err[2]), s
        assert v.tolist() == ov.tolist(), s
        # Lines and curves are exact; points derived from arcs go through trigonometry.
        scale = max(1.0, float(np.abs(op).max()) if len(op) else 1.0)
        assert np.allclose(p, op, rtol=0, atol=1e-5 * scale, equal_nan=True), s


def test_parse_then_tessellate_batch_layout():
    r = svg.parse_paths(["M 0 0 L 10 0 L 10 10 Z", "M 5 5 Q 10 0 15 5 T 25 5"])
    b = r.batch
    assert b.num_paths == 2
    # Begin, 2 lines, Close (4 points with the closing one); Begin, 2 quadratics, End.
    assert b.verb_offsets.tolist() == [0, 4, 8]
    assert b.point_offsets.tolist() == [0, 4, 9]
    assert b.verbs.tolist() == [3, 0, 0, 4, 3, 1, 1, 5]
    # T reflects the previous control point: (15, 5) + ((15, 5) - (10, 0)) = (20, 10).
    assert b.points[7].tolist() == [20.0, 10.0]
