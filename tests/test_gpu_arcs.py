"""GPU parity of arc flattening (lyon_gpu_flatten_arcs: Arc::for_each_flattened_with_t,
crates/geom/src/arc.rs:339-389) and of ellipse tessellation (stroke.rs:294-307,
fill.rs:675-690) against the oracle.

Both sides evaluate cos, sin and acos in f64 and round once, so points and t agree bit for bit
except where the two f64 libraries round a value to different sides of an f32 midpoint (rare):
per arc the counts must be equal and the points equal within 1e-5 of the arc's scale."""

import numpy as np
import pytest

from lyon_gb300 import tessellation as T
from lyon_gb300.options import FillOptions, LineCap, LineJoin, StrokeOptions
from oracle import lyon_oracle as orc

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gpu():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import gpu_helpers
    return gpu_helpers


def _gpu_arcs(gpu, arcs, tol):
    import torch
    c = gpu.ctx()
    d = torch.from_numpy(np.ascontiguousarray(arcs).view(np.uint8).copy()).cuda()
    res = T.flatten_arcs(d, len(arcs), tol, c)
    c.synchronize()
    pts = res.points.cpu().numpy() if res.total_points else np.zeros((0, 2), np.float32)
    ts = res.t.cpu().numpy() if res.total_points else np.zeros(0, np.float32)
    return pts, ts, res.offsets.cpu().numpy(), res.status.cpu().numpy()


def _random_arcs(n, seed):
    rng = np.random.default_rng(seed)
    a = np.zeros(n, T.ARC_DTYPE)
    a["center_x"] = rng.uniform(-1000, 1000, n)
    a["center_y"] = rng.uniform(-1000, 1000, n)
    a["radius_x"] = np.exp(rng.uniform(-3, 7, n))
    a["radius_y"] = np.where(rng.random(n) < 0.3, a["radius_x"], np.exp(rng.uniform(-3, 7, n)))
    a["start_angle"] = rng.uniform(-10, 10, n)
    a["sweep_angle"] = rng.uniform(-20, 20, n)
    a["x_rotation"] = rng.uniform(-4, 4, n)
    return a


def compare_arcs(gpu, arcs, tol):
    gp, gt, go, gs = _gpu_arcs(gpu, arcs, tol)
    op, ot, oo, os_ = orc.flatten_arcs(arcs.view(orc.ARC_DTYPE), tol)
    assert np.array_equal(gs, os_)
    bad, exact = [], 0
    for i in range(len(arcs)):
        g0, g1, o0, o1 = int(go[i]), int(go[i + 1]), int(oo[i]), int(oo[i + 1])
        if g1 - g0 != o1 - o0:
            bad.append((i, "count", g1 - g0, o1 - o0))
            continue
        if np.array_equal(gp[g0:g1], op[o0:o1]) and np.array_equal(gt[g0:g1], ot[o0:o1]):
            exact += 1
            continue
        scale = float(max(abs(arcs["center_x"][i]), abs(arcs["center_y"][i]), 1.0) +
                      max(arcs["radius_x"][i], arcs["radius_y"][i]))
        if not (np.allclose(gp[g0:g1], op[o0:o1], rtol=0, atol=1e-5 * scale) and
                np.allclose(gt[g0:g1], ot[o0:o1], rtol=0, atol=1e-6)):
            bad.append((i, "values"))
    return bad, exact


def test_flatten_arcs_random(gpu):
    arcs = _random_arcs(20000, 121)
    bad, exact = compare_arcs(gpu, arcs, 0.1)
    print(f"arcs={len(arcs)} exact={exact} bad={len(bad)}")
    assert len(bad) <= 2, bad[:10]
    assert exact >= len(arcs) - 50


def test_flatten_arcs_lyon_cases_and_edges(gpu):
    rows = [(-100.0, -150.0, 50.0, 50.0, 0.982944787, -898.0, 0.0),  # arc.rs:1212-1218
            (0.0, 0.0, 100.0, 10.0, 0.2, -2.0, 0.0),                   # arc.rs:1225-1231
            (0.0, 0.0, 0.0, 0.0, 0.0, 1.0, 0.0),                       # zero radius
            (5.0, 5.0, 1.0, 1.0, 0.0, 0.0, 0.0),                       # zero sweep
            (0.0, 0.0, 0.01, 0.01, 0.0, 6.0, 0.0),                     # radius below tolerance
            (0.0, 0.0, 1e6, 1e6, 0.0, 0.5, 0.0)]                       # long arc
    arcs = np.zeros(len(rows), T.ARC_DTYPE)
    for i, r in enumerate(rows):
        arcs[i] = r
    bad, _ = compare_arcs(gpu, arcs, 0.1)
    assert not bad, bad
    bad, _ = compare_arcs(gpu, arcs, 0.001)
    assert not bad, bad


def test_flatten_arcs_empty(gpu):
    pts, ts, offs, st = _gpu_arcs(gpu, np.zeros(0, T.ARC_DTYPE), 0.1)
    assert len(pts) == 0 and list(offs) == [0]


def test_tessellate_ellipse_stroke_and_fill(gpu):
    from lyon_gb300.path import PathBuilder
    for center, radii, rot, winding in [((10.0, 20.0), (30.0, 5.0), 0.3, 1),
                                        ((-50.0, 7.0), (8.0, 40.0), -1.2, -1)]:
        b = PathBuilder()
        b.add_ellipse(center, radii, rot, winding)
        path = b.build()
        so = StrokeOptions(line_width=3.0, line_join=LineJoin.Round, start_cap=LineCap.Round,
                           end_cap=LineCap.Round, tolerance=0.05)
        buf = T.VertexBuffers(32)
        T.StrokeTessellator(gpu.ctx()).tessellate_ellipse(center, radii, rot, winding, so,
                                                          T.BuffersBuilder(buf))
        ref = orc.stroke(path, so, 32)
        assert np.array_equal(buf.indices, ref.indices)
        assert np.allclose(buf.vertices, ref.vertices, rtol=0, atol=1e-4)
        fo = FillOptions(tolerance=0.05)
        buf = T.VertexBuffers(16)
        T.FillTessellator(gpu.ctx()).tessellate_ellipse(center, radii, rot, winding, fo,
                                                        T.BuffersBuilder(buf))
        ref = orc.fill(path, fo.with_intersections(False), 16)
        assert np.array_equal(buf.indices, ref.indices)
        assert np.array_equal(buf.vertices, ref.vertices)
