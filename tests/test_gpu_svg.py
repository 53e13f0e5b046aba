"""SVG path data parsed by the library (lyon_svg_parse_paths) and tessellated on the GPU, against
the oracle on the same parsed batch: the ingestion path end to end."""

import numpy as np
import pytest

from lyon_gb300 import svg
from lyon_gb300.options import FillOptions, StrokeOptions, LineJoin
from lyon_gb300.path import PathBatch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gpu():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import gpu_helpers
    return gpu_helpers


def _valid_strings(n, seed):
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        parts = [f"M {rng.uniform(0, 500):.2f} {rng.uniform(0, 500):.2f}"]
        for _ in range(int(rng.integers(1, 10))):
            c = rng.choice(list("LlHhVvCcSsQqTtAa"))
            k = {"L": 2, "H": 1, "V": 1, "C": 6, "S": 4, "Q": 4, "T": 2, "A": 7}[c.upper()]
            v = [f"{x:.2f}" for x in rng.uniform(-60, 60, size=k)]
            if c.upper() == "A":
                v[0], v[1] = f"{rng.uniform(1, 40):.2f}", f"{rng.uniform(1, 40):.2f}"
                v[3], v[4] = str(int(rng.integers(0, 2))), str(int(rng.integers(0, 2)))
            parts.append(c + " " + " ".join(v))
        if rng.random() < 0.5:
            parts.append("Z")
        out.append(" ".join(parts))
    return out


def test_svg_parsed_paths_stroke_and_fill(gpu):
    strings = _valid_strings(2000, 91)
    r = svg.parse_paths(strings)
    assert (r.status == 0).all()
    batch = r.batch
    so = StrokeOptions(line_width=3.0, tolerance=0.05, line_join=LineJoin.Round)
    s = gpu.compare_per_path("stroke", batch, so.to_record(), index_bits=32)
    assert not s["mismatches"], s["mismatches"][:10]
    fo = FillOptions(tolerance=0.05)
    s = gpu.compare_per_path("fill", batch, fo.to_record(), index_bits=32)
    assert not s["mismatches"], s["mismatches"][:10]


def _random_path(rng):
    cmds = []
    for _ in range(int(rng.integers(1, 12))):
        c = rng.choice(list("MmLlHhVvCcSsQqTtAaZz"))
        nums = {"M": 2, "L": 2, "H": 1, "V": 1, "C": 6, "S": 4, "Q": 4, "T": 2, "A": 7, "Z": 0}
        k = nums[c.upper()]
        vals = [f"{x:.{int(rng.integers(0, 9))}f}" for x in rng.uniform(-100, 100, size=k)]
        if c.upper() == "A":
            vals[0] = f"{abs(rng.uniform(0, 60)):.2f}"
            vals[1] = f"{abs(rng.uniform(0, 60)):.2f}"
            vals[3] = str(int(rng.integers(0, 2)))
            vals[4] = str(int(rng.integers(0, 2)))
        sep = rng.choice([" ", ",", "  ", "\n"])
        cmds.append(c + sep + sep.join(vals))
    return " ".join(cmds)


def test_device_parser_matches_host_parser(gpu):
    # lyon_gpu_svg_parse_paths (one string per thread) against lyon_svg_parse_paths (host
    # threads) on the same strings: verbs, offsets, statuses and error positions identical;
    # points identical except those derived from arcs (device cosf/sinf/tanf), within 1e-5.
    # The strings mix random commands, lyon's parser test cases and hard decimals.
    from test_svg_decimal import _cases
    rng = np.random.default_rng(93)
    strings = [_random_path(rng) for _ in range(3000)]
    strings += ["", " ", "M 0 0 L 1 0 L 1 1 L 0 1 Z", "x 0 0 0", "\n M 0 \n0 1 x 1 1 1",
                "M 0.6.5", "M 1e-2 -1E3", "M 0 --1", "M 0 1ee2", "M 0 +1", "M 0 0 Z L 1 1",
                "M 1.e-9 1.4e-4z", "0 0M", "M 10 10 a 5 5 0 0 1 10 0 A 30 20 45 1 0 50 50 z"]
    strings += [f"M {x} {x} L 1 {x}" for x in _cases()]
    host = svg.parse_paths(strings)
    dev = svg.parse_paths_device(gpu.ctx(), strings)
    hb = host.batch
    db = dev.host_batch()
    assert np.array_equal(dev.status, host.status)
    assert np.array_equal(dev.error_line, host.error_line)
    assert np.array_equal(dev.error_column, host.error_column)
    assert dev.num_failed == int((host.status != 0).sum())
    assert np.array_equal(db.verb_offsets, hb.verb_offsets)
    assert np.array_equal(db.point_offsets, hb.point_offsets)
    assert np.array_equal(db.verbs, hb.verbs)
    hp, dp = hb.points, db.points
    exact = (hp.view(np.uint32) == dp.view(np.uint32)).all(axis=1) | (np.isnan(hp) & np.isnan(dp)).all(axis=1)
    scale = max(1.0, float(np.nanmax(np.abs(hp))))
    assert np.allclose(dp, hp, rtol=0, atol=1e-5 * scale, equal_nan=True)
    # Everything that is not an arc's output is bit-identical: the hard-decimal strings have no
    # arcs, so all their points must be.
    first_hard = len(strings) - len(_cases())
    k0 = int(hb.point_offsets[first_hard])
    assert exact[k0:].all()
    assert exact.mean() > 0.9


def test_device_parsed_batch_strokes_like_host_parsed(gpu):
    # The device-parsed batch goes straight to the batched stroke call.
    from lyon_gb300 import tessellation as T
    strings = _valid_strings(1500, 94)
    dev = svg.parse_paths_device(gpu.ctx(), strings)
    assert dev.num_failed == 0
    so = StrokeOptions(line_width=2.0, tolerance=0.1, line_join=LineJoin.Round)
    od = T.upload_options(so.to_record(), 0)
    c = gpu.ctx()
    res = T.tessellate_paths("stroke", dev.batch, od, 1, 32, T.INDEX_PER_PATH, 0, c)
    c.synchronize()
    g = gpu.gpu_batch("stroke", dev.host_batch(), so.to_record(), index_bits=32)
    assert res.total_vertices == g["total_vertices"]
    assert res.total_indices == g["total_indices"]
