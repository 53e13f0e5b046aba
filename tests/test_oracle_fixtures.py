"""lyon's fill regression fixtures on the oracle (CPU).

* crates/tessellation/src/fuzz_tests.rs (lyon's own cases, extracted into
  tests/golden/lyon_fuzz_cases.json by tests/golden/make_golden.py): each polygon must fill
  without error with both fill rules at tolerance 0.05, u16 indices.
* crates/tessellation/src/earcut_tests.rs (Mapbox's earcut fixtures, ISC licensed): parsed in
  place from the lyon sources at test time and never copied into this repository; the test is
  skipped where those sources are absent. Each fixture must fill without error with both rules.
  The paths are built exactly as lyon's `earcut_test` builds them, including its
  `begin(point(start[0], start[0]))`.
"""

import json
import os
import re

import numpy as np
import pytest

from oracle import lyon_oracle as orc
from lyon_gb300.options import FillOptions, FillRule
from lyon_gb300.path import Path, Verb

from lyon_cases import GOLDEN


def _fill_ok(path):
    for rule in (FillRule.EvenOdd, FillRule.NonZero):
        r = orc.fill(path, FillOptions(tolerance=0.05, fill_rule=rule), 16)
        if r.status != 0:
            return False, rule, r.status
        if len(r.indices) and int(r.indices.max()) >= len(r.vertices):
            return False, rule, "index range"
    return True, None, None


def fuzz_paths():
    with open(os.path.join(GOLDEN, "lyon_fuzz_cases.json")) as f:
        cases = json.load(f)
    return [(c["src"], Path.from_arrays(c["verbs"], c["points"])) for c in cases]


def test_fuzz_cases_fill():
    cases = fuzz_paths()
    assert len(cases) >= 25
    for src, path in cases:
        ok, rule, why = _fill_ok(path)
        assert ok, (src, rule, why)


def _earcut_fixtures(text):
    """(name, [[(x, y), ...] per sub-path]) of every earcut_test / earcut_test_f32 call."""
    out = []
    for m in re.finditer(r"#\[test\]\s*fn (\w+)\(\)\s*\{\s*(earcut_test(?:_f32)?)\(&\[(.*?)\]\);",
                         text, re.S):
        name, fn, body = m.group(1), m.group(2), m.group(3)
        subs = []
        for sm in re.finditer(r"&\[(.*?)\]\s*,?\s*(?=&\[|$)", body, re.S):
            pts = re.findall(r"\[\s*(-?[\d.eE+-]+)\s*,\s*(-?[\d.eE+-]+)\s*\]", sm.group(1))
            subs.append([(np.float32(float(x)), np.float32(float(y))) for x, y in pts])
        out.append((name, subs))
    return out


def earcut_path(subs):
    verbs, points = [], []
    for sub in subs:
        if not sub:
            continue
        x0 = sub[0][0]
        verbs.append(Verb.BEGIN)
        points.append((x0, x0))  # as lyon's earcut_test builds it
        for p in sub:
            verbs.append(Verb.LINE_TO)
            points.append(p)
        verbs.append(Verb.CLOSE)
        points.append((x0, x0))
    return Path.from_arrays(verbs, points if points else np.zeros((0, 2)))


def test_earcut_fixtures_fill(reference_dir):
    text = open(os.path.join(reference_dir, "crates/tessellation/src/earcut_tests.rs")).read()
    fixtures = _earcut_fixtures(text)
    assert len(fixtures) >= 25, len(fixtures)
    for name, subs in fixtures:
        assert subs and all(len(s) >= 1 for s in subs), name
        ok, rule, why = _fill_ok(earcut_path(subs))
        assert ok, (name, rule, why)
