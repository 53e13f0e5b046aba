"""Fill correctness beyond parity: the triangles cover exactly the path's fill-rule interior.

For glyph paths (quadratic contours, holes, self-intersecting stars) and both fill rules, a grid
of samples over each path's bounding box is classified twice: by the winding number of the
flattened outline under the fill rule (FillRule::is_in, crates/path/src/lib.rs:267-281) and by
counting the output triangles that contain it. Inside samples must be covered exactly once and
outside samples not at all. Samples within the flattening tolerance of the outline are skipped
(the fill flattens curves from their downward end, so its outline differs from the forward
flattening by up to the tolerance). The GPU's fill output equals the oracle's bit for bit
(tests/test_gpu_fill.py), so the property holds for both.
"""

import numpy as np
import pytest

from oracle import lyon_oracle as orc
from lyon_gb300 import workloads
from lyon_gb300.options import FillOptions, FillRule
from lyon_gb300.path import Verb


def _outline(path, tol):
    """Closed polylines of the path's forward flattening: list of (k, 2) f64 arrays."""
    counts, pts = orc.flatten(path, tol)
    polys, cur, oi, pi = [], None, 0, 0
    for v, n in zip(path.verbs, counts):
        if v == Verb.BEGIN:
            cur = [path.points[pi].astype(np.float64)]
            pi += 1
            continue
        cur.extend(pts[oi:oi + n].astype(np.float64))
        oi += n
        pi += {Verb.LINE_TO: 1, Verb.QUADRATIC_TO: 2, Verb.CUBIC_TO: 3, Verb.CLOSE: 1}.get(v, 0)
        if v in (Verb.CLOSE, Verb.END):
            polys.append(np.array(cur))
            cur = None
    return polys


def _winding(samples, polys):
    w = np.zeros(len(samples), np.int64)
    for poly in polys:
        a = poly
        b = np.roll(poly, -1, axis=0)
        ax, ay, bx, by = a[:, 0][None], a[:, 1][None], b[:, 0][None], b[:, 1][None]
        px, py = samples[:, 0][:, None], samples[:, 1][:, None]
        cross = (bx - ax) * (py - ay) - (by - ay) * (px - ax)
        up = (ay <= py) & (by > py) & (cross > 0)
        down = (by <= py) & (ay > py) & (cross < 0)
        w += up.sum(axis=1) - down.sum(axis=1)
    return w


def _near_outline(samples, polys, eps):
    near = np.zeros(len(samples), bool)
    for poly in polys:
        a = poly
        b = np.roll(poly, -1, axis=0)
        ab = b - a
        l2 = np.maximum((ab * ab).sum(axis=1), 1e-30)
        ap = samples[:, None, :] - a[None]
        t = np.clip((ap * ab[None]).sum(axis=2) / l2[None], 0, 1)
        d = np.linalg.norm(ap - t[..., None] * ab[None], axis=2)
        near |= (d < eps).any(axis=1)
    return near


def _covered(samples, verts, idx):
    tri = verts[idx.reshape(-1, 3).astype(np.int64)].astype(np.float64)
    a, b, c = tri[:, 0][None], tri[:, 1][None], tri[:, 2][None]
    p = samples[:, None, :]

    def cr(u, v, w):
        return (v[..., 0] - u[..., 0]) * (w[..., 1] - u[..., 1]) - \
               (v[..., 1] - u[..., 1]) * (w[..., 0] - u[..., 0])
    d1, d2, d3 = cr(a, b, p), cr(b, c, p), cr(c, a, p)
    inside = ((d1 > 0) & (d2 > 0) & (d3 > 0)) | ((d1 < 0) & (d2 < 0) & (d3 < 0))
    return inside.sum(axis=1)


@pytest.mark.parametrize("rule", [FillRule.NonZero, FillRule.EvenOdd])
def test_glyph_coverage(rule):
    tol = 0.1
    batch, _ = workloads.glyph_fill(60, seed=171, fill_rule=rule)
    rng = np.random.default_rng(172)
    checked = 0
    for p in range(batch.num_paths):
        path = batch.path(p)
        r = orc.fill(path, FillOptions(tolerance=tol, fill_rule=rule), 32)
        assert r.status == 0
        polys = _outline(path, tol)
        lo, hi = path.points.min(axis=0), path.points.max(axis=0)
        samples = rng.uniform(lo, hi, size=(1500, 2))
        keep = ~_near_outline(samples, polys, 2 * tol + 1e-3)
        samples = samples[keep]
        w = _winding(samples, polys)
        inside = (w != 0) if rule == FillRule.NonZero else (w % 2 != 0)
        cov = _covered(samples, r.vertices, r.indices)
        assert np.array_equal(cov, inside.astype(np.int64)), (p, int((cov != inside).sum()))
        checked += len(samples)
    assert checked > 40000
