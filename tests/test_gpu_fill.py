"""GPU fill parity: the CUDA sweep (through the C ABI) against the oracle on the same inputs.

Fill output is compared exactly: vertex and index counts, index topology and vertex positions
(the sweep performs lyon's f32/f64 operations in lyon's order). The covered area of every path
is also checked against the oracle's within 1e-4 relative.
"""

import json
import os

import numpy as np
import pytest

from lyon_gb300 import workloads
from lyon_gb300 import tessellation as T
from lyon_gb300.options import FillOptions, FillRule, fill_options_array
from lyon_gb300.path import Path, PathBatch
from oracle import lyon_oracle as orc

from lyon_cases import GOLDEN, case_path, flatten_to_lines, load, rotation_angles, rust_logo

pytestmark = pytest.mark.gpu

AREA_RTOL = 1e-4


@pytest.fixture(scope="module")
def gpu():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import gpu_helpers
    return gpu_helpers


def _check(gpu, batch, opts, index_bits=32):
    s = gpu.compare_per_path("fill", batch, opts, index_bits=index_bits, rtol=0.0,
                             allow_near_ties=False)
    assert not s["mismatches"], s["mismatches"][:10]
    g, r = s["gpu"], s["oracle"]
    # Covered area per path (vertices are path-relative in per-path mode).
    gv = g["vertices"].astype(np.float64)
    rv = r["vertices"].astype(np.float64)
    for p in range(batch.num_paths):
        if g["status"][p] != 0:
            continue
        vg = gv[g["vtx_offsets"][p]:g["vtx_offsets"][p + 1]]
        vr = rv[r["vtx_offsets"][p]:r["vtx_offsets"][p + 1]]
        ig = g["indices"][g["idx_offsets"][p]:g["idx_offsets"][p + 1]].astype(np.int64)
        ir = r["indices"][r["idx_offsets"][p]:r["idx_offsets"][p + 1]].astype(np.int64)
        if index_bits == 16:
            ir = ir & 0xFFFF
        ag = _area(vg, ig)
        ar = _area(vr, ir)
        assert abs(ag - ar) <= AREA_RTOL * max(ar, 1e-30), (p, ag, ar)
    return s


def _area(v, idx):
    t = idx.reshape(-1, 3)
    if len(t) == 0:
        return 0.0
    a, b, c = v[t[:, 0]], v[t[:, 1]], v[t[:, 2]]
    u, w = b - a, c - a
    return float(np.abs(u[:, 0] * w[:, 1] - u[:, 1] * w[:, 0]).sum() * 0.5)


@pytest.mark.parametrize("rule", [FillRule.NonZero, FillRule.EvenOdd])
def test_glyph_fill_workload_subset(gpu, rule):
    # The glyph fill generator (contours of quadratics, holes, self-intersecting stars).
    batch, opts = workloads.glyph_fill(3000, seed=3, fill_rule=rule)
    s = _check(gpu, batch, opts)
    assert s["gpu"]["total_vertices"] > 0


def _lyon_fill_paths(paths):
    """fill_tests.rs:10-28 inputs: every path flattened at 0.05 first."""
    out = []
    for p in paths:
        counts, pts = orc.flatten(p, 0.05)
        out.append(flatten_to_lines(p, counts, pts))
    return out


def test_lyon_fill_fixtures(gpu):
    # Every fill fixture of lyon's tests (a subset of each rotation sweep), both fill rules,
    # tolerance 0.05, u16: the same triangles as the oracle.
    paths, expect = [], []
    for case in load("lyon_fill_cases.json"):
        path = case_path(case)
        if case["rotation_step"] is None:
            ps = [path]
        else:
            angles = list(rotation_angles(case["rotation_step"]))
            ps = [path.transformed_rotation(a) for a in angles[::max(1, len(angles) // 24)]]
        paths += ps
        expect += [case["expect_even_odd_triangles"]] * len(ps)
    flat = _lyon_fill_paths(paths)
    batch = PathBatch.from_paths(flat + flat)
    recs = ([FillOptions(tolerance=0.05, fill_rule=FillRule.EvenOdd).to_record()[0]] * len(flat)
            + [FillOptions(tolerance=0.05, fill_rule=FillRule.NonZero).to_record()[0]]
            * len(flat))
    s = _check(gpu, batch, fill_options_array(recs), index_bits=16)
    g = s["gpu"]
    for i, e in enumerate(expect):
        assert g["status"][i] == 0
        if e is not None:
            assert (g["idx_offsets"][i + 1] - g["idx_offsets"][i]) // 3 == e


def test_lyon_fuzz_fixtures(gpu):
    # crates/tessellation/src/fuzz_tests.rs polygons (lyon's regression cases), both fill rules,
    # tolerance 0.05, u16: every path succeeds, with the oracle's triangles.
    with open(os.path.join(GOLDEN, "lyon_fuzz_cases.json")) as f:
        cases = json.load(f)
    flat = _lyon_fill_paths([case_path(c) for c in cases])
    batch = PathBatch.from_paths(flat + flat)
    recs = ([FillOptions(tolerance=0.05, fill_rule=FillRule.EvenOdd).to_record()[0]] * len(flat)
            + [FillOptions(tolerance=0.05, fill_rule=FillRule.NonZero).to_record()[0]]
            * len(flat))
    s = _check(gpu, batch, fill_options_array(recs), index_bits=16)
    assert np.all(s["gpu"]["status"] == 0)


def test_rust_logo_variants(gpu):
    # fill_tests.rs: the logo scaled up and down, rotated, and with an intersecting rectangle;
    # both fill rules, both sweep orientations, intersections handled or not.
    logo = rust_logo()
    counts, pts = orc.flatten(logo, 0.011)
    flat = flatten_to_lines(logo, counts, pts)
    verbs = list(flat.verbs) + [3, 0, 0, 0, 4]
    points = list(map(tuple, flat.points)) + [(10.0, 30.0), (130.0, 30.0), (130.0, 60.0),
                                              (10.0, 60.0), (10.0, 30.0)]
    inter = Path.from_arrays(verbs, points)
    angles = list(rotation_angles(0.011))[::40]
    paths = [logo, logo.scaled(260.0), flat.scaled(0.005), flat.scaled(0.0000001)]
    paths += [flat.transformed_rotation(a) for a in angles]
    paths += [inter.transformed_rotation(a) for a in angles]
    all_paths, recs = [], []
    for rule in (FillRule.EvenOdd, FillRule.NonZero):
        for orient in (0, 1):
            for inter_on in (True, False):
                o = FillOptions(tolerance=0.05, fill_rule=rule, sweep_orientation=orient,
                                handle_intersections=inter_on)
                all_paths += paths
                recs += [o.to_record()[0]] * len(paths)
    _check(gpu, PathBatch.from_paths(all_paths), fill_options_array(recs))


def test_fill_tolerances_and_quadratic_glyphs(gpu):
    # Glyph paths at tolerances 0.01, 0.1 and 1.0 (curves flattened inside the event queue).
    batch, _ = workloads.glyph_fill(600, seed=11)
    rng = np.random.default_rng(5)
    recs = [FillOptions(tolerance=float(rng.choice([0.01, 0.1, 1.0])),
                        fill_rule=int(rng.integers(0, 2))).to_record()[0]
            for _ in range(batch.num_paths)]
    _check(gpu, batch, fill_options_array(recs))


def test_fill_too_many_vertices_single_path(gpu):
    # fill_tests.rs test_too_many_vertices through the single-path drop-in.
    for free in (0, 10, 100):
        buf = T.VertexBuffers(16)
        b = T.BuffersBuilder(buf, vertex_offset=65536 - free)
        with pytest.raises(T.TessellationError) as e:
            T.FillTessellator(gpu.ctx()).tessellate_path(rust_logo(), FillOptions(tolerance=0.05),
                                                         b)
        assert e.value.code == T.LYON_ERR_TOO_MANY_VERTICES
        assert len(buf.vertices) == 0 and len(buf.indices) == 0


def test_fill_single_path_matches_oracle(gpu):
    for rule in (FillRule.EvenOdd, FillRule.NonZero):
        opts = FillOptions(tolerance=0.05, fill_rule=rule)
        ref = orc.fill(rust_logo(), opts, index_bits=32)
        buf = T.VertexBuffers(32)
        T.FillTessellator(gpu.ctx()).tessellate_path(rust_logo(), opts, T.BuffersBuilder(buf))
        assert np.array_equal(buf.indices, ref.indices32)
        assert np.array_equal(buf.vertices, ref.vertices)


def test_fill_global_index_mode(gpu):
    # LYON_INDEX_GLOBAL: the batch equals tessellate_path called path by path on one builder.
    batch, opts = workloads.glyph_fill(300, seed=13)
    g = gpu.gpu_batch("fill", batch, opts, index_bits=32, index_mode=T.INDEX_GLOBAL)
    out = orc.Output(32)
    o = FillOptions(*[opts[0][k].item() for k in opts.dtype.names])
    for p in range(batch.num_paths):
        assert out.fill(batch.path(p), o) == 0
    ref = out.snapshot(0)
    assert np.array_equal(g["indices"], ref.indices32)
    assert np.array_equal(g["vertices"], ref.vertices)


def test_fill_autotuner_picks_a_setting_and_keeps_outputs(gpu):
    # lyon_gpu_autotune_fill times 10 settings (blocks per SM x sweepers per warp) on a sample,
    # keeps the fastest; outputs are the same under every setting.
    import ctypes
    from lyon_gb300 import _native
    batch, opts = workloads.glyph_fill(1500, seed=47)
    before = gpu.gpu_batch("fill", batch, opts, index_bits=32)
    c = gpu.ctx()
    db = T.DeviceBatch.upload(batch, 0)
    od = T.upload_options(opts, 0)
    cb = db.c()
    saved = _native.CFillTuning()
    assert c.lib.lyon_gpu_get_fill_tuning(c.h, ctypes.byref(saved)) == 0
    best = _native.CFillTuning()
    times = (ctypes.c_float * 10)()
    nc = ctypes.c_uint32()
    try:
        r = c.lib.lyon_gpu_autotune_fill(c.h, ctypes.byref(cb), od.data_ptr(), len(opts), 1000,
                                         ctypes.byref(best), times, ctypes.byref(nc))
        assert r == 0 and nc.value == 10
        assert all(t > 0.0 for t in times)
        assert best.blocks_per_sm in (16, 8) and best.lanes in (1, 4, 8, 12, 16)
        for lanes in (1, 16):
            t = _native.CFillTuning(8, lanes)
            assert c.lib.lyon_gpu_set_fill_tuning(c.h, ctypes.byref(t)) == 0
            after = gpu.gpu_batch("fill", batch, opts, index_bits=32)
            assert np.array_equal(after["indices"], before["indices"])
            assert np.array_equal(after["vertices"], before["vertices"])
    finally:
        c.lib.lyon_gpu_set_fill_tuning(c.h, ctypes.byref(saved))
