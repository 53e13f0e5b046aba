"""The serving loop of liblyon_gb300 (lyon_srv_* in include/lyon_gpu.h) from Python.

A request is a range of paths of a host PathBatch (borrowed: the arrays must outlive the
request) with 1 or per-path option records. Results stay in device memory until released.
"""

from __future__ import annotations

import ctypes
from dataclasses import dataclass
from typing import List, Optional, Sequence

import numpy as np

from . import _native
from .path import PathBatch
from .tessellation import TessellationError

KIND_STROKE = 0
KIND_FILL = 1


def batch_view(batch: PathBatch, start: int, count: int) -> _native.CPathBatch:
    """Paths [start, start + count) of a host batch, without copying (offsets stay absolute)."""
    vo = batch.verb_offsets
    po = batch.point_offsets
    assert vo.dtype == np.uint32 and po.dtype == np.uint32
    assert 0 <= start and start + count <= batch.num_paths
    return _native.CPathBatch(batch.verbs.ctypes.data, batch.points.ctypes.data,
                              vo.ctypes.data + 4 * start, po.ctypes.data + 4 * start, count)


@dataclass
class Request:
    kind: int
    batch: PathBatch
    start: int
    count: int
    options: np.ndarray  # 1 record, or one per path of the range

    def c_batch(self) -> _native.CPathBatch:
        return batch_view(self.batch, self.start, self.count)


@dataclass
class Result:
    status: int
    num_paths: int
    num_failed_paths: int
    vertices_ptr: int
    num_vertices: int
    indices_ptr: int
    num_indices: int
    path_vertex_offsets_ptr: int
    path_index_offsets_ptr: int
    path_status_ptr: int
    vertex_base: int
    index_base: int
    queue_ms: float
    latency_ms: float

    def host_copy(self):
        """(vertices (V, 2) f32, indices u32, per-path vertex offsets, per-path statuses)."""
        import torch
        from .tessellation import _CudaArray

        def get(ptr, shape, typestr, dtype):
            if int(np.prod(shape)) == 0:
                return np.zeros(shape, dtype)
            return torch.as_tensor(_CudaArray(ptr, shape, typestr), device="cuda").cpu().numpy()

        v = get(self.vertices_ptr, (self.num_vertices, 2), "<f4", np.float32)
        i = get(self.indices_ptr, (self.num_indices,), "<u4", np.uint32)
        vo = get(self.path_vertex_offsets_ptr, (self.num_paths + 1,), "<u8", np.uint64)
        st = get(self.path_status_ptr, (self.num_paths,), "<i4", np.int32)
        return v, i, vo - np.uint64(self.vertex_base), st


def _result(r: _native.CSrvResult) -> Result:
    return Result(r.status, r.num_paths, r.num_failed_paths, int(r.vertices or 0),
                  int(r.num_vertices), int(r.indices or 0), int(r.num_indices),
                  int(r.path_vertex_offsets or 0), int(r.path_index_offsets or 0),
                  int(r.path_status or 0), int(r.vertex_base), int(r.index_base),
                  float(r.queue_ms), float(r.latency_ms))


class Server:
    """lyon_srv_*: `num_workers` workers take any request (fill requests only when
    `num_stroke_workers` > 0, whose workers take the strokes on high-priority streams)."""

    def __init__(self, device: int = 0, num_workers: int = 2, max_batch_paths: int = 65536,
                 device_budget_bytes: int = 40 << 30, num_stroke_workers: int = 0,
                 fill_blocks_per_sm: int = 0, max_stroke_batch_paths: int = 0):
        self.lib = _native.load()
        cfg = _native.CSrvConfig(device, num_workers, max_batch_paths, device_budget_bytes,
                                 num_stroke_workers, fill_blocks_per_sm, max_stroke_batch_paths)
        self.h = self.lib.lyon_srv_create(ctypes.byref(cfg))
        if not self.h:
            raise RuntimeError("lyon_srv_create failed")
        self._keep = {}

    def submit(self, req: Request) -> int:
        cb = req.c_batch()
        opts = np.ascontiguousarray(req.options)
        t = self.lib.lyon_srv_submit(self.h, req.kind, ctypes.byref(cb), opts.ctypes.data,
                                     len(opts))
        if t == 0:
            raise ValueError("invalid request")
        self._keep[t] = (cb, opts)
        return int(t)

    def wait(self, ticket: int) -> Result:
        r = _native.CSrvResult()
        rc = self.lib.lyon_srv_wait(self.h, ticket, ctypes.byref(r))
        if rc != 0:
            raise TessellationError(rc, "lyon_srv_wait")
        return _result(r)

    def poll(self, ticket: int) -> Optional[Result]:
        r = _native.CSrvResult()
        rc = self.lib.lyon_srv_poll(self.h, ticket, ctypes.byref(r))
        return None if rc == 1 else _result(r)

    def release(self, ticket: int) -> None:
        self.lib.lyon_srv_release(self.h, ticket)
        self._keep.pop(ticket, None)

    def run_load(self, requests: Sequence[Request], rate_per_s: float, duration_s: float,
                 seed: int = 5, want_latencies: bool = False):
        items = (_native.CSrvLoadItem * len(requests))()
        keep: List = []
        for k, r in enumerate(requests):
            opts = np.ascontiguousarray(r.options)
            keep.append(opts)
            items[k] = _native.CSrvLoadItem(r.kind, r.c_batch(), opts.ctypes.data, len(opts))
        stats = _native.CSrvLoadStats()
        cap = int(rate_per_s * duration_s * 2 + 1024) if want_latencies else 0
        lat = np.zeros(cap, np.float64)
        rc = self.lib.lyon_srv_run_load(self.h, items, len(requests), float(rate_per_s),
                                        float(duration_s), seed, ctypes.byref(stats),
                                        lat.ctypes.data if cap else None, cap)
        if rc != 0:
            raise TessellationError(rc, "lyon_srv_run_load")
        out = {f: getattr(stats, f) for f, _ in _native.CSrvLoadStats._fields_}
        if want_latencies:
            out["latencies_ms"] = lat[:stats.completed]
        return out

    def config(self) -> dict:
        """The configuration the loop runs with, defaults resolved (lyon_srv_get_config)."""
        c = _native.CSrvConfig()
        rc = self.lib.lyon_srv_get_config(self.h, ctypes.byref(c))
        if rc != 0:
            raise TessellationError(rc, "lyon_srv_get_config")
        return {name: getattr(c, name) for name, _ in c._fields_}

    def close(self) -> None:
        if self.h:
            self.lib.lyon_srv_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:  # noqa: BLE001
            pass


def mixed_requests(stroke_pool: PathBatch, stroke_opts: np.ndarray, fill_pool: PathBatch,
                   fill_opts: np.ndarray, count: int, seed: int = 5, max_paths: int = 5000,
                   stroke_share: float = 0.7) -> List[Request]:
    """Requests of 1..max_paths paths (log-uniform), `stroke_share` of them strokes; each a
    range of the stroke or fill pool."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        stroke = rng.random() < stroke_share
        pool = stroke_pool if stroke else fill_pool
        opts = stroke_opts if stroke else fill_opts
        n = int(round(float(np.exp(rng.uniform(0.0, np.log(max_paths))))))
        n = max(1, min(n, pool.num_paths))
        start = int(rng.integers(0, pool.num_paths - n + 1))
        o = opts if len(opts) == 1 else opts[start:start + n]
        out.append(Request(KIND_STROKE if stroke else KIND_FILL, pool, start, n, o))
    return out
