"""GPU parity for the one-thread-per-path stroke phase.

Line-only paths of at most `short_path_points` points (32 by default) are stroked one path per
thread after the warp items of a launch. Their outputs are checked against the oracle, and the
whole batch byte for byte against the warp walk alone (short_path_points = 0), failing paths
included.
"""

import ctypes

import numpy as np
import pytest

from lyon_gb300 import _native, workloads
from lyon_gb300 import tessellation as T
from lyon_gb300.options import STROKE_OPTIONS_DTYPE, LineCap, LineJoin
from lyon_gb300.path import Path, PathBatch, Verb

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gpu():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import gpu_helpers
    c = gpu_helpers.ctx()
    saved = _native.CStrokeTuning()
    assert c.lib.lyon_gpu_get_stroke_tuning(c.h, ctypes.byref(saved)) == 0
    yield gpu_helpers
    c.lib.lyon_gpu_set_stroke_tuning(c.h, ctypes.byref(saved))


def _tune(gpu, long_points, short_points, blocks=0):
    c = gpu.ctx()
    t = _native.CStrokeTuning(long_points, blocks, short_points)
    assert c.lib.lyon_gpu_set_stroke_tuning(c.h, ctypes.byref(t)) == 0


def short_polylines(n, seed):
    """Line-only paths of 1-3 sub-paths and at most about 32 points: repeated and nearly
    repeated points (merge filter, empty caps), closed and open sub-paths."""
    rng = np.random.default_rng(seed)
    paths = []
    for _ in range(n):
        nsub = 1 if rng.random() < 0.8 else int(rng.integers(2, 4))
        budget = int(rng.integers(1, 34))
        verbs, pts = [], []
        for _ in range(nsub):
            m = int(rng.integers(1, max(1, budget // nsub) + 1))
            steps = rng.normal(0.0, 10.0, size=(m, 2))
            steps[0] = 0.0
            steps[rng.random(m) < 0.15] = 0.0
            steps[rng.random(m) < 0.05] *= 1e-4
            p = rng.uniform(0.0, 1000.0, size=2) + np.cumsum(steps, axis=0)
            verbs.append(Verb.BEGIN)
            pts.append(p[0])
            for q in p[1:]:
                verbs.append(Verb.LINE_TO)
                pts.append(q)
            if rng.random() < 0.3:
                verbs.append(Verb.CLOSE)
                pts.append(p[0])
            else:
                verbs.append(Verb.END)
        paths.append(Path.from_arrays(verbs, pts))
    return PathBatch.from_paths(paths)


def random_options(n, seed):
    rng = np.random.default_rng(seed)
    o = np.zeros(n, dtype=STROKE_OPTIONS_DTYPE)
    o["line_join"] = rng.choice([LineJoin.Miter, LineJoin.MiterClip, LineJoin.Round,
                                 LineJoin.Bevel], size=n)
    caps = rng.choice([LineCap.Butt, LineCap.Square, LineCap.Round], size=(n, 2))
    o["start_cap"] = caps[:, 0]
    o["end_cap"] = caps[:, 1]
    o["line_width"] = rng.uniform(0.5, 8.0, size=n).astype(np.float32)
    o["miter_limit"] = rng.choice(np.array([1.0, 4.0, 10.0], np.float32), size=n)
    o["tolerance"] = rng.choice(np.array([0.01, 0.1, 1.0], np.float32), size=n)
    return o


def failing_paths():
    """Paths that fail: points missing for their verbs, a Begin inside a sub-path, a sub-path
    without Begin; and one that ends without End (stroked, no tail)."""
    return [
        Path.from_arrays([Verb.BEGIN, Verb.LINE_TO, Verb.LINE_TO, Verb.END], [[0, 0], [5, 0]]),
        Path.from_arrays([Verb.BEGIN, Verb.LINE_TO, Verb.BEGIN, Verb.LINE_TO, Verb.END],
                         [[0, 0], [5, 0], [9, 9], [9, 12]]),
        Path.from_arrays([Verb.LINE_TO, Verb.LINE_TO, Verb.END], [[0, 0], [5, 0]]),
        Path.from_arrays([Verb.BEGIN, Verb.LINE_TO, Verb.LINE_TO], [[0, 0], [5, 0], [5, 5]]),
        Path.from_arrays([Verb.BEGIN, Verb.LINE_TO, Verb.CLOSE], [[0, 0], [5, 0]]),
    ]


def _same(a, b):
    for k in ("status", "vtx_offsets", "idx_offsets", "indices", "vertices"):
        assert np.array_equal(a[k], b[k]), k


def test_short_paths_match_oracle(gpu):
    batch = short_polylines(6000, seed=91)
    opts = random_options(batch.num_paths, seed=92)
    _tune(gpu, 1024, 32)
    s = gpu.compare_per_path("stroke", batch, opts, index_bits=32)
    print(f"paths={s['paths']} mismatches={len(s['mismatches'])} "
          f"near_tie_mismatches={s['near_tie_mismatches']}")
    assert not s["mismatches"], s["mismatches"][:10]
    assert s["near_tie_mismatches"] <= max(2, batch.num_paths // 1000)


@pytest.mark.parametrize("index_bits,index_mode", [(16, T.INDEX_PER_PATH),
                                                   (32, T.INDEX_GLOBAL)])
def test_short_phase_equals_warp_walk(gpu, index_bits, index_mode):
    short = short_polylines(3000, seed=93)
    paths = [short.path(i) for i in range(short.num_paths)]
    rng = np.random.default_rng(94)
    for k, p in enumerate(failing_paths()):
        paths.insert(int(rng.integers(0, len(paths))), p)
    batch = PathBatch.from_paths(paths)
    opts = random_options(batch.num_paths, seed=95)
    _tune(gpu, 1024, 0)
    warp = gpu.gpu_batch("stroke", batch, opts, index_bits=index_bits, index_mode=index_mode)
    _tune(gpu, 1024, 32)
    seq = gpu.gpu_batch("stroke", batch, opts, index_bits=index_bits, index_mode=index_mode)
    assert int((warp["status"] != 0).sum()) >= 4
    _same(warp, seq)


def test_mixed_classes_equal_across_settings(gpu):
    # Long polylines, curves and short line-only paths in one batch; every class non-empty.
    poly, popts = workloads.map_polylines(4000, seed=96, max_len=400)
    curves, copts = workloads.batched_stroke(1500, seed=97)
    short = short_polylines(2500, seed=98)
    paths = ([poly.path(i) for i in range(poly.num_paths)] +
             [curves.path(i) for i in range(curves.num_paths)] +
             [short.path(i) for i in range(short.num_paths)])
    order = np.random.default_rng(99).permutation(len(paths))
    batch = PathBatch.from_paths([paths[i] for i in order])
    opts = np.concatenate([popts, copts, random_options(short.num_paths, seed=100)])[order]
    results = []
    for long_points, short_points, blocks in [(0, 0, 0), (64, 32, 0), (64, 32, 1), (0, 64, 0),
                                              (256, 8, 0)]:
        _tune(gpu, long_points, short_points, blocks)
        results.append(gpu.gpu_batch("stroke", batch, opts, index_bits=32,
                                     index_mode=T.INDEX_GLOBAL))
    for r in results[1:]:
        _same(results[0], r)
    _tune(gpu, 64, 32)
    s = gpu.compare_per_path("stroke", batch, opts, index_bits=32)
    assert not s["mismatches"], s["mismatches"][:10]
    assert s["near_tie_mismatches"] <= max(2, batch.num_paths // 1000)


def test_short_path_points_bound(gpu):
    c = gpu.ctx()
    t = _native.CStrokeTuning(1024, 0, 65)
    assert c.lib.lyon_gpu_set_stroke_tuning(c.h, ctypes.byref(t)) != 0
