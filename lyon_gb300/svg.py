"""SVG path data to path batches (lyon_svg_parse_paths in include/lyon_gpu.h): lyon_extra's
PathParser (crates/extra/src/parser.rs) over many strings at once, on the host's threads, into
the batch layout the tessellation kernels read."""

from __future__ import annotations

import ctypes
from dataclasses import dataclass
from typing import Optional, Sequence

import numpy as np

from . import _native
from .path import PathBatch

SVG_ERR_NUMBER = 110
SVG_ERR_FLAG = 111
SVG_ERR_COMMAND = 112
SVG_ERR_MISSING_MOVE_TO = 113


@dataclass
class ParsedPaths:
    batch: PathBatch
    widths: Optional[np.ndarray]  # one endpoint attribute per point (num_attributes == 1)
    status: np.ndarray            # per string: 0 or a SVG_ERR_* code
    error_line: np.ndarray
    error_column: np.ndarray


def parse_paths(strings: Sequence[str], num_attributes: int = 0, stop_at: Optional[str] = None,
                num_threads: int = 0) -> ParsedPaths:
    """Parses every string as lyon's PathParser::parse would into its own path."""
    L = _native.load()
    enc = [s.encode("utf-8") for s in strings]
    n = len(enc)
    offs = np.zeros(n + 1, np.uint64)
    offs[1:] = np.cumsum([len(e) for e in enc], dtype=np.uint64)
    text = b"".join(enc) + b"\0"
    opts = _native.CSvgParseOptions(num_attributes, -1 if stop_at is None else ord(stop_at),
                                    num_threads)
    status = np.zeros(max(n, 1), np.int32)
    eline = np.zeros(max(n, 1), np.int32)
    ecol = np.zeros(max(n, 1), np.int32)
    tv = ctypes.c_uint64()
    tp = ctypes.c_uint64()
    r = L.lyon_svg_parse_paths(text, offs.ctypes.data, n, ctypes.byref(opts), None, 0, None, 0,
                               None, None, None, status.ctypes.data, eline.ctypes.data,
                               ecol.ctypes.data, ctypes.byref(tv), ctypes.byref(tp))
    if r not in (0, 103):  # LYON_OK or LYON_ERR_CAPACITY (the sizing call)
        raise RuntimeError(f"lyon_svg_parse_paths: status {r}")
    verbs = np.zeros(max(tv.value, 1), np.uint8)
    points = np.zeros((max(tp.value, 1), 2), np.float32)
    widths = np.zeros(max(tp.value, 1), np.float32) if num_attributes else None
    vo = np.zeros(n + 1, np.uint32)
    po = np.zeros(n + 1, np.uint32)
    r = L.lyon_svg_parse_paths(text, offs.ctypes.data, n, ctypes.byref(opts), verbs.ctypes.data,
                               len(verbs), points.ctypes.data, len(points),
                               widths.ctypes.data if widths is not None else None,
                               vo.ctypes.data, po.ctypes.data, None, None, None,
                               ctypes.byref(tv), ctypes.byref(tp))
    if r != 0:
        raise RuntimeError(f"lyon_svg_parse_paths: status {r}")
    batch = PathBatch(verbs[:tv.value], points[:tp.value], vo, po)
    return ParsedPaths(batch, widths[:tp.value] if widths is not None else None, status[:n],
                       eline[:n], ecol[:n])
