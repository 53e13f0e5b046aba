"""Seeded synthetic path workloads (vectorised numpy generators).

Five workload families, each parameterised by its size:
  plain_stroke   1,000 paths of one sub-path with 16 segments (line/quadratic/cubic thirds,
                 shuffled per path), f32 points uniform in [0, 1024]^2, half of them closed;
                 tolerance 0.1, width 4, miter join (limit 4), butt caps, u16 indices.
  batched_stroke 1,000,000 paths, segment count log-normal (median 12, sigma 1, clamp 1..4096),
                 same segment mix, coordinates and closed fraction; round joins and caps,
                 tolerance 0.05, per-path width uniform in [0.5, 8], u32 indices.
  glyph_fill     200,000 closed paths of 1-6 contours of 8-40 quadratic segments around random
                 centres (radius 5-200, +-30 % radial noise), 30 % of inner contours reversed
                 (holes), 10 % of paths replaced by self-intersecting star polygons of 5-50
                 points; non-zero and even-odd; tolerance 0.1; u32 indices.
  map_polylines  2,000,000 open polylines, lengths Pareto (alpha 1.2, min 2, max 20,000 points),
                 random-walk vertices (N(0, 3) px steps) from a start in [0, 65536]^2, widths
                 1-8, joins miter/bevel/round equally likely; tolerances {0.01, 0.1, 1.0}.
  serving        Poisson arrivals of scenes of 1-5,000 paths (log-uniform), 70 % plain_stroke
                 paths and 30 % glyph_fill paths.
All generators return a PathBatch plus per-path option records.
"""

from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

from .options import (FILL_OPTIONS_DTYPE, STROKE_OPTIONS_DTYPE, FillRule, LineCap, LineJoin,
                      Orientation)
from .path import PathBatch, Verb

PTS_PER_KIND = np.array([1, 2, 3], dtype=np.int64)  # line, quadratic, cubic


def _segment_paths(rng, seg_counts: np.ndarray, closed: np.ndarray, lo: float = 0.0,
                   hi: float = 1024.0) -> PathBatch:
    """One sub-path per path: Begin, `n` segments whose kinds are k mod 3 shuffled per path,
    then Close (with the first point repeated) or End."""
    n_paths = int(seg_counts.shape[0])
    seg_counts = seg_counts.astype(np.int64)
    total_segs = int(seg_counts.sum())
    path_of_seg = np.repeat(np.arange(n_paths, dtype=np.int64), seg_counts)
    seg_start = np.zeros(n_paths + 1, dtype=np.int64)
    seg_start[1:] = np.cumsum(seg_counts)
    k_in_path = np.arange(total_segs, dtype=np.int64) - seg_start[path_of_seg]
    kinds_sorted = (k_in_path % 3).astype(np.int64)
    # Shuffle kinds within each path: order segments by (path, random key).
    keys = rng.random(total_segs)
    order = np.lexsort((keys, path_of_seg))
    kinds = kinds_sorted[order]

    closed = closed.astype(bool)
    verbs_per_path = seg_counts + 2
    seg_pts = PTS_PER_KIND[kinds]
    pts_per_path = np.zeros(n_paths, dtype=np.int64)
    np.add.at(pts_per_path, path_of_seg, seg_pts)
    pts_per_path += 1 + closed.astype(np.int64)

    vo = np.zeros(n_paths + 1, dtype=np.int64)
    vo[1:] = np.cumsum(verbs_per_path)
    po = np.zeros(n_paths + 1, dtype=np.int64)
    po[1:] = np.cumsum(pts_per_path)

    verbs = np.empty(int(vo[-1]), dtype=np.uint8)
    verbs[vo[:-1]] = Verb.BEGIN
    verbs[vo[1:] - 1] = np.where(closed, Verb.CLOSE, Verb.END).astype(np.uint8)
    seg_verb_pos = vo[path_of_seg] + 1 + k_in_path
    verbs[seg_verb_pos] = kinds.astype(np.uint8)  # LINE_TO=0, QUADRATIC_TO=1, CUBIC_TO=2

    points = rng.uniform(lo, hi, size=(int(po[-1]), 2)).astype(np.float32)
    # Close repeats the sub-path's first point.
    closing = np.nonzero(closed)[0]
    points[po[closing + 1] - 1] = points[po[closing]]
    return PathBatch(verbs, points, vo.astype(np.uint32), po.astype(np.uint32))


def plain_stroke(n_paths: int = 1000, seed: int = 1):
    rng = np.random.default_rng(seed)
    seg_counts = np.full(n_paths, 16, dtype=np.int64)
    closed = rng.random(n_paths) < 0.5
    batch = _segment_paths(rng, seg_counts, closed)
    opts = np.zeros(1, dtype=STROKE_OPTIONS_DTYPE)
    opts[0] = (LineCap.Butt, LineCap.Butt, LineJoin.Miter, 4.0, 4.0, 0.1)
    return batch, opts


def batched_stroke_segment_counts(rng, n_paths: int) -> np.ndarray:
    z = rng.standard_normal(n_paths)
    return np.clip(np.rint(np.exp(math.log(12.0) + 1.0 * z)), 1, 4096).astype(np.int64)


def batched_stroke(n_paths: int = 1_000_000, seed: int = 2):
    rng = np.random.default_rng(seed)
    seg_counts = batched_stroke_segment_counts(rng, n_paths)
    closed = rng.random(n_paths) < 0.5
    batch = _segment_paths(rng, seg_counts, closed)
    opts = np.zeros(n_paths, dtype=STROKE_OPTIONS_DTYPE)
    opts["start_cap"] = LineCap.Round
    opts["end_cap"] = LineCap.Round
    opts["line_join"] = LineJoin.Round
    opts["line_width"] = rng.uniform(0.5, 8.0, size=n_paths).astype(np.float32)
    opts["miter_limit"] = 4.0
    opts["tolerance"] = 0.05
    return batch, opts


def _star_step(m: int) -> int:
    """k of the star polygon {m/k}: coprime to m, so the outline visits every vertex."""
    if m <= 4:
        return 1
    k = max(2, m // 2 - (1 if m % 2 == 0 else 0))
    while math.gcd(m, k) != 1:
        k -= 1
    return max(k, 2)


def glyph_fill(n_paths: int = 200_000, seed: int = 3, fill_rule: int = FillRule.NonZero):
    """Closed glyph-like paths; see the module docstring."""
    rng = np.random.default_rng(seed)
    is_star = rng.random(n_paths) < 0.10
    n_contours = np.where(is_star, 1, rng.integers(1, 7, size=n_paths)).astype(np.int64)
    centre = rng.uniform(0, 1024, size=(n_paths, 2))
    R = rng.uniform(5, 200, size=n_paths)
    # One row per contour (a star path is one contour of lines).
    n_c = int(n_contours.sum())
    cpath = np.repeat(np.arange(n_paths, dtype=np.int64), n_contours)
    cfirst = np.zeros(n_paths + 1, dtype=np.int64)
    cfirst[1:] = np.cumsum(n_contours)
    cidx = np.arange(n_c, dtype=np.int64) - cfirst[cpath]
    cstar = is_star[cpath]
    inner = cidx > 0
    cR = R[cpath]
    off = rng.uniform(-0.3, 0.3, size=(n_c, 2)) * cR[:, None]
    ox = centre[cpath, 0] + np.where(inner, off[:, 0], 0.0)
    oy = centre[cpath, 1] + np.where(inner, off[:, 1], 0.0)
    r = np.where(inner, cR * rng.uniform(0.1, 0.45, size=n_c), cR)
    reverse = inner & (rng.random(n_c) < 0.30)
    m = np.where(cstar, rng.integers(5, 51, size=n_c), rng.integers(8, 41, size=n_c))
    k = np.array([_star_step(int(x)) for x in range(51)], dtype=np.int64)[m]
    # Raw outline points: m star vertices, or 2m alternating on-curve / control points.
    n_raw = np.where(cstar, m, 2 * m)
    raw_first = np.zeros(n_c + 1, dtype=np.int64)
    raw_first[1:] = np.cumsum(n_raw)
    rc = np.repeat(np.arange(n_c, dtype=np.int64), n_raw)
    j = np.arange(int(raw_first[-1]), dtype=np.int64) - raw_first[rc]
    ang = np.where(cstar[rc], 2 * math.pi * ((j * k[rc]) % m[rc]) / m[rc],
                   2 * math.pi * j / (2 * m[rc]))
    ang = np.where(reverse[rc], -ang, ang)
    rad = r[rc] * (1 + rng.uniform(-0.3, 0.3, size=rc.shape[0]))
    raw = np.stack([ox[rc] + rad * np.cos(ang), oy[rc] + rad * np.sin(ang)], axis=1)
    # Emitted points: the raw points, then the first point again (the end of the last quadratic
    # of a curved contour, and the point Close stores).
    extra = np.where(cstar, 1, 2)
    n_out = n_raw + extra
    out_first = np.zeros(n_c + 1, dtype=np.int64)
    out_first[1:] = np.cumsum(n_out)
    oc = np.repeat(np.arange(n_c, dtype=np.int64), n_out)
    oj = np.arange(int(out_first[-1]), dtype=np.int64) - out_first[oc]
    src = raw_first[oc] + np.where(oj < n_raw[oc], oj, 0)
    points = raw[src].astype(np.float32)
    # Verbs: Begin, m - 1 lines (star) or m quadratics, Close.
    n_verbs = np.where(cstar, m + 1, m + 2)
    verb_first = np.zeros(n_c + 1, dtype=np.int64)
    verb_first[1:] = np.cumsum(n_verbs)
    vc = np.repeat(np.arange(n_c, dtype=np.int64), n_verbs)
    vj = np.arange(int(verb_first[-1]), dtype=np.int64) - verb_first[vc]
    body = np.where(cstar[vc], Verb.LINE_TO, Verb.QUADRATIC_TO)
    verbs = np.where(vj == 0, Verb.BEGIN,
                     np.where(vj == n_verbs[vc] - 1, Verb.CLOSE, body)).astype(np.uint8)
    vo = verb_first[cfirst].astype(np.uint32)
    po = out_first[cfirst].astype(np.uint32)
    batch = PathBatch(verbs, points, vo, po)
    opts = np.zeros(1, dtype=FILL_OPTIONS_DTYPE)
    opts[0] = (0.1, fill_rule, Orientation.Vertical, 1)
    return batch, opts


def map_polylines(n_paths: int = 2_000_000, seed: int = 4, tolerance: float = 0.1,
                  max_len: int = 20000):
    rng = np.random.default_rng(seed)
    u = rng.random(n_paths)
    lengths = np.minimum(max_len, np.floor(2.0 * np.power(1.0 - u, -1.0 / 1.2))).astype(np.int64)
    lengths = np.maximum(lengths, 2)
    n_pts = int(lengths.sum())
    po = np.zeros(n_paths + 1, dtype=np.int64)
    po[1:] = np.cumsum(lengths)
    steps = rng.normal(0.0, 3.0, size=(n_pts, 2))
    starts = rng.uniform(0, 65536, size=(n_paths, 2))
    first = po[:-1]
    steps[first] = starts
    # Random walk: cumulative sum restarted at every path start.
    cs = np.cumsum(steps, axis=0)
    base = np.repeat(cs[first] - starts, lengths, axis=0)
    points = (cs - base).astype(np.float32)
    vo = np.zeros(n_paths + 1, dtype=np.int64)
    vo[1:] = np.cumsum(lengths + 1)
    verbs = np.full(int(vo[-1]), Verb.LINE_TO, dtype=np.uint8)
    verbs[vo[:-1]] = Verb.BEGIN
    verbs[vo[1:] - 1] = Verb.END
    batch = PathBatch(verbs, points, vo.astype(np.uint32), po.astype(np.uint32))
    opts = np.zeros(n_paths, dtype=STROKE_OPTIONS_DTYPE)
    opts["start_cap"] = LineCap.Butt
    opts["end_cap"] = LineCap.Butt
    joins = np.array([LineJoin.Miter, LineJoin.Bevel, LineJoin.Round], np.int32)
    opts["line_join"] = joins[rng.integers(0, 3, size=n_paths)]
    opts["line_width"] = rng.uniform(1.0, 8.0, size=n_paths).astype(np.float32)
    opts["miter_limit"] = 4.0
    opts["tolerance"] = tolerance
    return batch, opts


@dataclass
class Request:
    arrival_s: float
    kind: str          # "stroke" or "fill"
    batch: PathBatch
    options: np.ndarray


def serving_requests(rate_per_s: float = 50_000.0, duration_s: float = 60.0, seed: int = 5,
                     max_requests: int | None = None, max_paths: int = 5000):
    """Poisson arrivals; each request a scene of 1..max_paths paths (log-uniform)."""
    rng = np.random.default_rng(seed)
    n = rng.poisson(rate_per_s * duration_s)
    if max_requests is not None:
        n = min(n, max_requests)
    arrivals = np.sort(rng.uniform(0.0, duration_s, size=n))
    sizes = np.rint(np.exp(rng.uniform(0.0, math.log(max_paths), size=n))).astype(np.int64)
    sizes = np.maximum(sizes, 1)
    is_stroke = rng.random(n) < 0.70
    # Pools of pre-generated paths that scenes sample from.
    stroke_pool, stroke_opts = plain_stroke(4096, seed=seed * 10 + 1)
    fill_pool, fill_opts = glyph_fill(2048, seed=seed * 10 + 2)
    reqs = []
    for i in range(n):
        if is_stroke[i]:
            idx = rng.integers(0, stroke_pool.num_paths, size=int(sizes[i]))
            reqs.append(Request(float(arrivals[i]), "stroke", stroke_pool.subset(idx),
                                stroke_opts))
        else:
            idx = rng.integers(0, fill_pool.num_paths, size=int(sizes[i]))
            reqs.append(Request(float(arrivals[i]), "fill", fill_pool.subset(idx), fill_opts))
    return reqs
