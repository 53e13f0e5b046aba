"""Flattening accuracy of lyon's scheme (quadratic_bezier.rs:943-974, cubic_bezier.rs:1369-1403),
measured in f64: t advances by 1/w for the fractional Wang count w, so every segment but the last
spans 1/w and stays within the tolerance of its curve; the last one ends at t = 1 and spans up to
2/w, so its distance is bounded by 4 x the tolerance (the deviation grows with the square of the
span). The oracle's flattening is the GPU's bit for bit
(tests/test_gpu_stroke.py::test_flatten_counts_and_points), so the bounds hold for both."""

import numpy as np
import pytest

from oracle import lyon_oracle as orc
from lyon_gb300 import workloads
from lyon_gb300.path import Verb


def _curve(ctrl, t):
    """Bézier of degree len(ctrl) - 1 at t (f64, de Casteljau)."""
    pts = [np.asarray(c, np.float64) for c in ctrl]
    t = t[:, None]
    while len(pts) > 1:
        pts = [a * (1 - t) + b * t for a, b in zip(pts, pts[1:])]
    return pts[0]


def _seg_dist(p, a, b):
    ab = b - a
    l2 = float(ab @ ab)
    if l2 == 0.0:
        return np.linalg.norm(p - a, axis=1)
    s = np.clip(((p - a) @ ab) / l2, 0.0, 1.0)
    return np.linalg.norm(p - (a + s[:, None] * ab), axis=1)


@pytest.mark.parametrize("tol", [0.01, 0.1, 1.0])
def test_flattened_segments_within_tolerance(tol):
    batch, _ = workloads.batched_stroke(100, seed=161)
    worst, worst_last = 0.0, 0.0
    for p in range(batch.num_paths):
        path = batch.path(p)
        counts, pts = orc.flatten(path, tol)
        pts = pts.astype(np.float64)
        pi = 0  # index into the path's points
        oi = 0  # index into the flattened points
        cur = None
        for v, n in zip(path.verbs, counts):
            if v == Verb.BEGIN:
                cur = path.points[pi].astype(np.float64)
                pi += 1
                continue
            if v in (Verb.QUADRATIC_TO, Verb.CUBIC_TO):
                k = 2 if v == Verb.QUADRATIC_TO else 3
                ctrl = [cur] + [path.points[pi + j].astype(np.float64) for j in range(k)]
                seg = np.vstack([cur[None, :], pts[oi:oi + n]])
                # lyon's parameters: t advances by 1/w (w = the fractional Wang count, in
                # f32), the last segment ends at t = 1.
                w = np.float32(orc.wang(np.array(ctrl, np.float32), tol))
                step = np.float32(1.0) / w
                ts = [np.float32(0.0)]
                for _ in range(n - 1):
                    ts.append(np.float32(ts[-1] + step))
                ts.append(np.float32(1.0))
                for s in range(n):
                    t = np.linspace(float(ts[s]), float(ts[s + 1]), 17)
                    d = float(_seg_dist(_curve(ctrl, t), seg[s], seg[s + 1]).max())
                    if s + 1 < n:
                        worst = max(worst, d)
                    else:
                        worst_last = max(worst_last, d)
                cur = ctrl[-1]
                pi += k
            elif v == Verb.LINE_TO:
                cur = path.points[pi].astype(np.float64)
                pi += 1
            elif v == Verb.CLOSE:
                pi += 1
            oi += n
    # The f32 evaluation of the points adds rounding on coordinates up to 1024.
    assert worst <= tol * 1.001 + 1e-3, worst
    assert worst_last <= 4 * tol * 1.001 + 1e-3, worst_last
