"""GPU parity of hatching and dots (lyon_gpu_hatch_paths / lyon_gpu_dot_paths: lyon_algorithms'
Hatcher with the regular patterns, crates/algorithms/src/hatching.rs) against the oracle: per
path the status and the records, bit for bit (NaN tangents equal)."""

import numpy as np
import pytest

from lyon_gb300 import hatching as H
from lyon_gb300 import tessellation as T
from lyon_gb300 import workloads
from lyon_gb300.path import PathBatch
from oracle import lyon_oracle as orc

from test_hatching import SQUARE, params

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gpu():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import gpu_helpers
    return gpu_helpers


def _compare(gpu, batch, angle, interval, dots=False, column=1.0, tangents=True, tol=0.1,
             uv=(0.0, 0.0)):
    c = gpu.ctx()
    db = T.DeviceBatch.upload(batch, 0)
    if dots:
        res = H.dot_paths(db, H.DotOptions(tol, angle, uv), interval, column, c)
    else:
        res = H.hatch_paths(db, H.HatchingOptions(tol, angle, tangents, uv), interval, c)
    c.synchronize()
    g = res.to_numpy()
    go = res.offsets.cpu().numpy()
    gs = res.status.cpu().numpy()
    o, oo, os_ = orc.hatch(batch, params(angle, interval, tangents, dots, column, tol, uv))
    assert np.array_equal(gs, os_)
    bad = []
    for p in range(batch.num_paths):
        a = g[go[p]:go[p + 1]].view(np.uint8)
        b = o[oo[p]:oo[p + 1]].view(np.uint8)
        if not np.array_equal(a, b):
            # Bit patterns may differ only in NaN payloads.
            fa = g[go[p]:go[p + 1]]
            fb = o[oo[p]:oo[p + 1]]
            same = len(fa) == len(fb) and all(
                np.array_equal(fa[n], fb[n], equal_nan=fa.dtype[n].kind == "f")
                for n in fa.dtype.names)
            if not same:
                bad.append(p)
    return bad, len(g)


@pytest.mark.parametrize("angle,interval", [(0.0, 2.0), (0.7, 1.5), (-2.2, 4.0)])
def test_hatch_glyphs(gpu, angle, interval):
    batch, _ = workloads.glyph_fill(1500, seed=131)
    bad, n = _compare(gpu, batch, angle, interval, uv=(3.0, -7.0))
    print(f"segments={n} bad={len(bad)}")
    assert not bad, bad[:10]


def test_hatch_strokes_no_tangents(gpu):
    # Open paths with cubics (the closing edge is added all the same, as lyon does).
    batch, _ = workloads.batched_stroke(800, seed=132)
    bad, _ = _compare(gpu, batch, 0.3, 5.0, tangents=False)
    assert not bad, bad[:10]


def test_dots_glyphs(gpu):
    batch, _ = workloads.glyph_fill(1000, seed=133)
    bad, n = _compare(gpu, batch, 0.5, 3.0, dots=True, column=2.0)
    assert n > 0 and not bad, bad[:10]


def test_simple_hatching_single_path(gpu):
    segs = H.Hatcher(gpu.ctx()).hatch_path(SQUARE, H.HatchingOptions(), 1.0)
    assert len(segs) == 9
    assert np.array_equal(segs["a_y"], np.arange(1, 10, dtype=np.float32))
    dots = H.Hatcher(gpu.ctx()).dot_path(SQUARE, H.DotOptions(), 2.0, 2.5)
    assert len(dots) == 16


def test_hatch_empty_batch_and_paths(gpu):
    from lyon_gb300.path import Path
    empty = Path.from_arrays([], np.zeros((0, 2)))
    batch = PathBatch.from_paths([empty, SQUARE, empty])
    bad, n = _compare(gpu, batch, 0.0, 1.0)
    assert not bad and n == 9
