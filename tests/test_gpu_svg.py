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
