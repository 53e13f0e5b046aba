"""SVG path data to path batches: lyon_extra's PathParser (crates/extra/src/parser.rs) over many
strings at once into the batch layout the tessellation kernels read, on the host's threads
(lyon_svg_parse_paths) or on the device (lyon_gpu_svg_parse_paths, one thread per string)."""

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


@dataclass
class RawDeviceBatch:
    """Device pointers of a path batch the library owns (the layout of lyon_path_batch)."""
    verbs_ptr: int
    points_ptr: int
    verb_offsets_ptr: int
    point_offsets_ptr: int
    num_paths: int

    def c(self) -> _native.CPathBatch:
        return _native.CPathBatch(self.verbs_ptr, self.points_ptr, self.verb_offsets_ptr,
                                  self.point_offsets_ptr, self.num_paths)


@dataclass
class DeviceParsedPaths:
    """A batch parsed on the device; its arrays belong to the context until its next parse."""
    batch: "RawDeviceBatch"       # the parsed arrays (tessellate_paths reads it)
    widths_ptr: int
    status: np.ndarray            # host copies of the per-string diagnostics
    error_line: np.ndarray
    error_column: np.ndarray
    total_verbs: int
    total_points: int
    num_failed: int

    def host_batch(self) -> PathBatch:
        """The parsed batch copied to the host."""
        import torch
        from .tessellation import _CudaArray

        def get(ptr, n, typestr, dtype):
            if n == 0:
                return np.zeros(0, dtype)
            return torch.as_tensor(_CudaArray(ptr, (n,), typestr), device="cuda").cpu().numpy()

        b = self.batch
        verbs = get(b.verbs_ptr, self.total_verbs, "|u1", np.uint8)
        pts = get(b.points_ptr, 2 * self.total_points, "<f4", np.float32).reshape(-1, 2)
        vo = get(b.verb_offsets_ptr, b.num_paths + 1, "<u4", np.uint32)
        po = get(b.point_offsets_ptr, b.num_paths + 1, "<u4", np.uint32)
        return PathBatch(verbs, pts, vo, po)


def parse_paths_device(ctx, strings: Sequence[str], num_attributes: int = 0,
                       stop_at: Optional[str] = None) -> DeviceParsedPaths:
    """Parses every string on the device (the text goes up once, nothing comes back but the
    diagnostics)."""
    import torch
    enc = [s.encode("utf-8") for s in strings]
    n = len(enc)
    offs = np.zeros(n + 1, np.uint64)
    offs[1:] = np.cumsum([len(e) for e in enc], dtype=np.uint64)
    text = np.frombuffer(b"".join(enc) + b"\0", np.uint8)
    dev = torch.device("cuda", ctx.device) if hasattr(ctx, "device") else torch.device("cuda")
    dtext = torch.from_numpy(text.copy()).to(dev)
    doffs = torch.from_numpy(offs.view(np.int64).copy()).to(dev)
    opts = _native.CSvgParseOptions(num_attributes, -1 if stop_at is None else ord(stop_at), 0)
    out = _native.CSvgOutput()
    r = ctx.lib.lyon_gpu_svg_parse_paths(ctx.h, dtext.data_ptr(), doffs.data_ptr(), n,
                                         ctypes.byref(opts), ctypes.byref(out))
    if r != 0:
        raise RuntimeError(f"lyon_gpu_svg_parse_paths: status {r}")
    ctx.synchronize()

    def diag(ptr):
        if n == 0:
            return np.zeros(0, np.int32)
        from .tessellation import _CudaArray
        return torch.as_tensor(_CudaArray(ptr, (n,), "<i4"), device=dev).cpu().numpy()

    b = RawDeviceBatch(int(out.batch.verbs or 0), int(out.batch.points or 0),
                       int(out.batch.verb_offsets or 0), int(out.batch.point_offsets or 0), n)
    return DeviceParsedPaths(b, int(out.widths or 0), diag(out.status), diag(out.error_line),
                             diag(out.error_column), int(out.total_verbs),
                             int(out.total_points), int(out.num_failed))
