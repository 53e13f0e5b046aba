"""Per-sample coverage on a 4096 x 4096 grid: the fill output of the CUDA sweep and the oracle's
on the same glyph paths, rasterised by the same kernel (lyon_gpu_coverage_compare: samples
strictly inside a triangle, ties on shared edges given to exactly one of the two triangles), must
cover exactly the same samples with the same counts, for both fill rules. Also checks the
rasteriser itself on shapes whose coverage is known."""

import ctypes

import numpy as np
import pytest

from lyon_gb300 import _native, workloads
from lyon_gb300.options import FillRule
from oracle import lyon_oracle as orc

pytestmark = pytest.mark.gpu

GRID = 4096


@pytest.fixture(scope="module")
def gpu():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import gpu_helpers
    return gpu_helpers


def _dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def _compare(boxes, a, b, grid=GRID):
    """a, b: (vertices (V, 2) f32, indices u32 relative to each path's first vertex, vertex
    offsets (P + 1), index offsets (P + 1)). Returns (P, 3): samples covered by a, by b, and
    samples whose counts differ."""
    import torch
    lib = _native.load()
    n = len(boxes)
    keep = [_dev(np.asarray(boxes, np.float32))]
    for v, i, vo, io in (a, b):
        v = np.asarray(v, np.float32).reshape(-1, 2)
        i = np.asarray(i, np.uint32)
        keep += [_dev(v if len(v) else np.zeros((1, 2), np.float32)),
                 _dev(i if len(i) else np.zeros(1, np.uint32)),
                 _dev(np.asarray(vo, np.uint64)), _dev(np.asarray(io, np.uint64))]
    out = torch.zeros(3 * n, dtype=torch.int64, device="cuda")
    f = lib.lyon_gpu_coverage_compare
    f.restype = ctypes.c_int
    r = f(ctypes.c_void_p(keep[0].data_ptr()), ctypes.c_uint32(n), ctypes.c_uint32(grid),
          *[ctypes.c_void_p(t.data_ptr()) for t in keep[1:]], ctypes.c_void_p(out.data_ptr()),
          None)
    assert r == 0
    torch.cuda.synchronize()
    return out.cpu().numpy().reshape(n, 3)


def test_rasteriser_counts_a_square_once_however_it_is_cut(gpu):
    # The square [0.25, 0.75]^2 in the box [0, 1]^2, cut along either diagonal (the second cut's
    # triangles in the opposite orientation): every sample inside is covered exactly once, the
    # counts agree, and the covered samples are the grid points inside.
    v = np.array([[0.25, 0.25], [0.75, 0.25], [0.75, 0.75], [0.25, 0.75]], np.float32)
    cut1 = np.array([0, 1, 2, 0, 2, 3], np.uint32)
    cut2 = np.array([1, 3, 0, 1, 2, 3], np.uint32)
    offs_v = np.array([0, 4], np.uint64)
    offs_i = np.array([0, 6], np.uint64)
    c = _compare([[0, 0, 1, 1]], (v, cut1, offs_v, offs_i), (v, cut2, offs_v, offs_i),
                 grid=1024)
    # Sample centres (i + 0.5) / 1024 in [0.25, 0.75]: i = 256 .. 767 (512 columns).
    assert c[0, 2] == 0
    assert c[0, 0] == c[0, 1] == 512 * 512


def test_rasteriser_sees_a_missing_triangle(gpu):
    v = np.array([[0.1, 0.1], [0.9, 0.1], [0.9, 0.9], [0.1, 0.9]], np.float32)
    full = np.array([0, 1, 2, 0, 2, 3], np.uint32)
    half = np.array([0, 1, 2], np.uint32)
    c = _compare([[0, 0, 1, 1]],
                 (v, full, np.array([0, 4], np.uint64), np.array([0, 6], np.uint64)),
                 (v, half, np.array([0, 4], np.uint64), np.array([0, 3], np.uint64)), grid=512)
    assert c[0, 2] > 0 and c[0, 2] == c[0, 0] - c[0, 1]


@pytest.mark.parametrize("rule", [FillRule.NonZero, FillRule.EvenOdd])
def test_glyph_fill_coverage_matches_oracle(gpu, rule):
    # 200 glyph paths of the fill workload (contours of quadratics, holes, self-intersecting
    # stars) per rule, each on a 4096^2 grid over its input box.
    batch, opts = workloads.glyph_fill(200, seed=41, fill_rule=rule)
    g = gpu.gpu_batch("fill", batch, opts, index_bits=32)
    r = orc.batch("fill", batch, opts, 32, 8)
    boxes = []
    for p in range(batch.num_paths):
        pts = batch.points[batch.point_offsets[p]:batch.point_offsets[p + 1]]
        lo, hi = pts.min(axis=0), pts.max(axis=0)
        pad = 0.01 * float(max(hi - lo))
        boxes.append([lo[0] - pad, lo[1] - pad, hi[0] + pad, hi[1] + pad])
    assert ((g["status"] == 0) & (r["status"] == 0)).all()
    c = _compare(boxes, (g["vertices"], g["indices"], g["vtx_offsets"], g["idx_offsets"]),
                 (r["vertices"], r["indices"], r["vtx_offsets"], r["idx_offsets"]))
    assert (c[:, 2] == 0).all(), np.nonzero(c[:, 2])[0][:10]
    assert (c[:, 0] == c[:, 1]).all()
    assert (c[:, 0] > 0).all()
