"""ctypes binding of liblyon_gb300.so (C ABI in include/lyon_gpu.h).

The library is the only compute path: when it is missing or no CUDA device is present, loading
raises instead of falling back to anything else.
"""

from __future__ import annotations

import ctypes
import os
import threading

from . import build as _build

_lib = None
_lock = threading.Lock()

c_p = ctypes.c_void_p
u32 = ctypes.c_uint32
u64 = ctypes.c_uint64
i32 = ctypes.c_int32


class CPathBatch(ctypes.Structure):
    _fields_ = [("verbs", c_p), ("points", c_p), ("verb_offsets", c_p),
                ("point_offsets", c_p), ("num_paths", u32)]


class CResult(ctypes.Structure):
    _fields_ = [("vertices", c_p), ("num_vertices", u32), ("indices", c_p),
                ("num_indices", u32), ("status", i32)]


class CBatchOutput(ctypes.Structure):
    _fields_ = [("vertices", c_p), ("indices", c_p), ("vertex_offsets", c_p),
                ("index_offsets", c_p), ("status", c_p),
                ("total_vertices", u64), ("total_indices", u64), ("num_failed_paths", u32)]


class CVertexSource(ctypes.Structure):
    _fields_ = [("from_", u32), ("to", u32), ("t", ctypes.c_float)]


class CCustomOutput(ctypes.Structure):
    _fields_ = [("sources", c_p), ("attributes", c_p)]


class CFillCustomOutput(ctypes.Structure):
    _fields_ = [("sources", c_p), ("source_offsets", c_p), ("total_sources", u64),
                ("attributes", c_p)]


class CArcOutput(ctypes.Structure):
    _fields_ = [("points", c_p), ("t", c_p), ("offsets", c_p), ("status", c_p),
                ("total_points", u64)]


class CHatchingOptions(ctypes.Structure):
    _fields_ = [("tolerance", ctypes.c_float), ("angle", ctypes.c_float),
                ("uv_origin_x", ctypes.c_float), ("uv_origin_y", ctypes.c_float),
                ("interval", ctypes.c_float), ("column_interval", ctypes.c_float),
                ("compute_tangents", i32)]


class CHatchOutput(ctypes.Structure):
    _fields_ = [("segments", c_p), ("dots", c_p), ("offsets", c_p), ("status", c_p),
                ("total", u64)]


class CFillTuning(ctypes.Structure):
    _fields_ = [("blocks_per_sm", u32), ("lanes", u32)]


class CSvgOutput(ctypes.Structure):
    _fields_ = [("batch", CPathBatch), ("widths", c_p), ("status", c_p), ("error_line", c_p),
                ("error_column", c_p), ("total_verbs", u64), ("total_points", u64),
                ("num_failed", u32)]


class CSrvConfig(ctypes.Structure):
    _fields_ = [("device", ctypes.c_int), ("num_workers", u32), ("max_batch_paths", u32),
                ("device_budget_bytes", u64), ("num_stroke_workers", u32),
                ("fill_blocks_per_sm", u32), ("max_stroke_batch_paths", u32)]


class CSrvResult(ctypes.Structure):
    _fields_ = [("status", ctypes.c_int), ("num_paths", u32), ("num_failed_paths", u32),
                ("vertices", c_p), ("num_vertices", u64), ("indices", c_p), ("num_indices", u64),
                ("path_vertex_offsets", c_p), ("path_index_offsets", c_p), ("path_status", c_p),
                ("vertex_base", u64), ("index_base", u64), ("queue_ms", ctypes.c_double),
                ("latency_ms", ctypes.c_double)]


class CSrvLoadItem(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int), ("batch", CPathBatch), ("options", c_p),
                ("num_options", u32)]


class CSrvLoadStats(ctypes.Structure):
    _fields_ = [("submitted", u32), ("completed", u32), ("failed", u32),
                ("offered_rate", ctypes.c_double), ("elapsed_s", ctypes.c_double),
                ("achieved_rate", ctypes.c_double), ("paths", u64), ("vertices", u64),
                ("indices", u64), ("p50_ms", ctypes.c_double), ("p99_ms", ctypes.c_double),
                ("p999_ms", ctypes.c_double), ("max_ms", ctypes.c_double), ("batches", u64),
                ("mean_batch_paths", ctypes.c_double)]


class CSvgParseOptions(ctypes.Structure):
    _fields_ = [("num_attributes", u32), ("stop_at", ctypes.c_int32), ("num_threads", u32)]


class CStrokeTuning(ctypes.Structure):
    _fields_ = [("long_path_points", u32), ("blocks_per_sm", u32), ("short_path_points", u32)]


class NativeLibraryMissing(RuntimeError):
    pass


def lib_path() -> str:
    return _build.LIB_PATH


def load(build_if_missing: bool = True):
    """Loads the CUDA library, building it first when nvcc is available and it is stale."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = os.environ.get("LYON_GB300_LIB") or _build.LIB_PATH
        if path == _build.LIB_PATH and build_if_missing and not _build.up_to_date():
            try:
                _build.build()
            except Exception as e:  # noqa: BLE001
                if not os.path.exists(path):
                    raise NativeLibraryMissing(f"cannot build {path}: {e}") from e
        if not os.path.exists(path):
            raise NativeLibraryMissing(f"{path} is missing; run lyon_gb300.build.build()")
        L = ctypes.CDLL(path)
        L.lyon_gpu_version.restype = ctypes.c_char_p
        L.lyon_gpu_host_alloc.restype = c_p
        L.lyon_gpu_host_alloc.argtypes = [ctypes.c_size_t]
        L.lyon_gpu_host_free.restype = ctypes.c_int
        L.lyon_gpu_host_free.argtypes = [c_p]
        L.lyon_gpu_kernel_launches.restype = u64
        L.lyon_gpu_kernel_launches.argtypes = []
        L.lyon_gpu_create.restype = c_p
        L.lyon_gpu_create.argtypes = [ctypes.c_int]
        L.lyon_gpu_destroy.argtypes = [c_p]
        L.lyon_gpu_stream.restype = c_p
        L.lyon_gpu_stream.argtypes = [c_p]
        L.lyon_gpu_last_error.restype = ctypes.c_char_p
        L.lyon_gpu_last_error.argtypes = [c_p]
        L.lyon_gpu_synchronize.restype = ctypes.c_int
        L.lyon_gpu_synchronize.argtypes = [c_p]
        for name in ("lyon_gpu_stroke_path", "lyon_gpu_fill_path",
                     "lyon_gpu_stroke_path_attributes"):
            f = getattr(L, name)
            f.restype = ctypes.c_int
            f.argtypes = [c_p, c_p, u32, c_p, u32, c_p, ctypes.c_int, u32,
                          ctypes.POINTER(CResult)]
        for name in ("lyon_gpu_stroke_paths", "lyon_gpu_fill_paths",
                     "lyon_gpu_stroke_paths_attributes"):
            f = getattr(L, name)
            f.restype = ctypes.c_int
            f.argtypes = [c_p, ctypes.POINTER(CPathBatch), c_p, u32, ctypes.c_int, ctypes.c_int,
                          u32, ctypes.POINTER(CBatchOutput)]
        L.lyon_gpu_stroke_paths_each.restype = ctypes.c_int
        L.lyon_gpu_stroke_paths_each.argtypes = [c_p, ctypes.POINTER(CPathBatch), c_p, u32,
                                                 ctypes.c_int, u32, u32, ctypes.POINTER(u64)]
        for name in ("lyon_gpu_stroke_paths_host", "lyon_gpu_fill_paths_host"):
            f = getattr(L, name)
            f.restype = ctypes.c_int
            f.argtypes = [c_p, ctypes.POINTER(CPathBatch), c_p, u32, ctypes.c_int, ctypes.c_int,
                          u32, c_p, u64, c_p, u64, c_p, ctypes.POINTER(u64), ctypes.POINTER(u64)]
        L.lyon_gpu_set_timing.argtypes = [c_p, ctypes.c_int]
        L.lyon_gpu_last_timings.restype = ctypes.c_int
        L.lyon_gpu_last_timings.argtypes = [c_p, ctypes.POINTER(ctypes.c_float)]
        L.lyon_gpu_flatten_counts.restype = ctypes.c_int
        L.lyon_gpu_flatten_counts.argtypes = [c_p, ctypes.POINTER(CPathBatch), ctypes.c_float,
                                              c_p]
        L.lyon_gpu_flatten_paths.restype = ctypes.c_int
        L.lyon_gpu_flatten_paths.argtypes = [c_p, ctypes.POINTER(CPathBatch), ctypes.c_float,
                                             ctypes.POINTER(c_p), ctypes.POINTER(c_p),
                                             ctypes.POINTER(u64)]
        L.lyon_srv_create.restype = c_p
        L.lyon_srv_create.argtypes = [ctypes.POINTER(CSrvConfig)]
        L.lyon_srv_destroy.argtypes = [c_p]
        L.lyon_srv_get_config.restype = ctypes.c_int
        L.lyon_srv_get_config.argtypes = [c_p, ctypes.POINTER(CSrvConfig)]
        L.lyon_srv_submit.restype = u64
        L.lyon_srv_submit.argtypes = [c_p, ctypes.c_int, ctypes.POINTER(CPathBatch), c_p, u32]
        for name in ("lyon_srv_poll", "lyon_srv_wait"):
            f = getattr(L, name)
            f.restype = ctypes.c_int
            f.argtypes = [c_p, u64, ctypes.POINTER(CSrvResult)]
        L.lyon_srv_release.restype = ctypes.c_int
        L.lyon_srv_release.argtypes = [c_p, u64]
        L.lyon_srv_run_load.restype = ctypes.c_int
        L.lyon_srv_run_load.argtypes = [c_p, ctypes.POINTER(CSrvLoadItem), u32, ctypes.c_double,
                                        ctypes.c_double, u64, ctypes.POINTER(CSrvLoadStats),
                                        c_p, u32]
        for name in ("lyon_gpu_set_stroke_tuning", "lyon_gpu_get_stroke_tuning"):
            f = getattr(L, name)
            f.restype = ctypes.c_int
            f.argtypes = [c_p, ctypes.POINTER(CStrokeTuning)]
        for name in ("lyon_gpu_set_fill_tuning", "lyon_gpu_get_fill_tuning"):
            f = getattr(L, name)
            f.restype = ctypes.c_int
            f.argtypes = [c_p, ctypes.POINTER(CFillTuning)]
        L.lyon_gpu_autotune_fill.restype = ctypes.c_int
        L.lyon_gpu_autotune_fill.argtypes = [c_p, ctypes.POINTER(CPathBatch), c_p, u32, u32,
                                             ctypes.POINTER(CFillTuning), c_p,
                                             ctypes.POINTER(u32)]
        L.lyon_gpu_svg_parse_paths.restype = ctypes.c_int
        L.lyon_gpu_svg_parse_paths.argtypes = [c_p, c_p, c_p, u32, c_p, ctypes.POINTER(CSvgOutput)]
        L.lyon_svg_parse_paths.restype = ctypes.c_int
        L.lyon_svg_parse_paths.argtypes = [c_p, c_p, u32, c_p, c_p, u64, c_p, u64, c_p, c_p, c_p,
                                           c_p, c_p, c_p, c_p, c_p]
        L.lyon_gpu_fill_shapes.restype = ctypes.c_int
        L.lyon_gpu_fill_shapes.argtypes = [c_p, ctypes.c_int, c_p, u32, c_p, u32, ctypes.c_int,
                                           ctypes.c_int, u32, c_p]
        L.lyon_gpu_stroke_paths_variable_width.restype = ctypes.c_int
        L.lyon_gpu_stroke_paths_variable_width.argtypes = [c_p, c_p, c_p, c_p, u32,
                                                           ctypes.c_int, ctypes.c_int, u32,
                                                           ctypes.c_int, c_p]
        L.lyon_gpu_stroke_path_variable_width.restype = ctypes.c_int
        L.lyon_gpu_stroke_path_variable_width.argtypes = [c_p, c_p, u32, c_p, u32, c_p, c_p,
                                                          ctypes.c_int, u32, ctypes.c_int, c_p]
        L.lyon_gpu_stroke_paths_custom.restype = ctypes.c_int
        L.lyon_gpu_stroke_paths_custom.argtypes = [c_p, c_p, c_p, u32, i32, c_p, u32,
                                                   ctypes.c_int, ctypes.c_int, u32, ctypes.c_int,
                                                   c_p, c_p]
        L.lyon_gpu_interpolate_attributes.restype = ctypes.c_int
        L.lyon_gpu_interpolate_attributes.argtypes = [c_p, c_p, u64, c_p, u32, u64, c_p]
        L.lyon_gpu_stroke_path_custom.restype = ctypes.c_int
        L.lyon_gpu_stroke_path_custom.argtypes = [c_p, c_p, u32, c_p, u32, c_p, u32, i32, c_p,
                                                  ctypes.c_int, u32, ctypes.c_int, c_p,
                                                  ctypes.POINTER(c_p), ctypes.POINTER(c_p)]
        L.lyon_gpu_fill_paths_custom.restype = ctypes.c_int
        L.lyon_gpu_fill_paths_custom.argtypes = [c_p, c_p, c_p, u32, c_p, u32, ctypes.c_int,
                                                 ctypes.c_int, u32, c_p, c_p]
        L.lyon_gpu_interpolate_fill_attributes.restype = ctypes.c_int
        L.lyon_gpu_interpolate_fill_attributes.argtypes = [c_p, c_p, c_p, u64, c_p, u32, u64,
                                                           c_p]
        L.lyon_gpu_fill_path_custom.restype = ctypes.c_int
        L.lyon_gpu_fill_path_custom.argtypes = [c_p, c_p, u32, c_p, u32, c_p, u32, c_p,
                                                ctypes.c_int, u32, c_p, ctypes.POINTER(c_p),
                                                ctypes.POINTER(c_p), ctypes.POINTER(c_p)]
        L.lyon_gpu_flatten_arcs.restype = ctypes.c_int
        L.lyon_gpu_flatten_arcs.argtypes = [c_p, c_p, u32, ctypes.c_float, c_p]
        for _fn in ("lyon_gpu_hatch_paths", "lyon_gpu_dot_paths"):
            getattr(L, _fn).restype = ctypes.c_int
            getattr(L, _fn).argtypes = [c_p, c_p, c_p, c_p]
        L.lyon_gpu_query_sizes.restype = ctypes.c_int
        L.lyon_gpu_query_sizes.argtypes = [c_p, ctypes.c_int, c_p, c_p, u32, ctypes.c_int,
                                           ctypes.c_int, u32, ctypes.POINTER(u64),
                                           ctypes.POINTER(u64), ctypes.POINTER(u32)]
        L.lyon_gpu_emit_into.restype = ctypes.c_int
        L.lyon_gpu_emit_into.argtypes = [c_p, ctypes.c_int, c_p, c_p, u32, ctypes.c_int,
                                         ctypes.c_int, u32, c_p, c_p, c_p]
        L.lyon_gpu_autotune_stroke.restype = ctypes.c_int
        L.lyon_gpu_autotune_stroke.argtypes = [c_p, ctypes.POINTER(CPathBatch), c_p, u32, u32,
                                               ctypes.POINTER(CStrokeTuning),
                                               ctypes.POINTER(ctypes.c_float),
                                               ctypes.POINTER(u32)]
        f = L.lyon_gpu_stroke_paths_noalloc
        f.restype = ctypes.c_int
        f.argtypes = [ctypes.POINTER(CPathBatch), c_p, u32, ctypes.c_int, ctypes.c_int, u32,
                      c_p, u64, c_p, u64, c_p, c_p, c_p, ctypes.POINTER(u64),
                      ctypes.POINTER(u64), ctypes.POINTER(u32), c_p, ctypes.c_char_p,
                      ctypes.c_size_t]
        _lib = L
        return L


# Symbols that include/lyon_gpu.h declares (checked by the CPU test suite).
EXPORTED = [
    "lyon_gpu_create", "lyon_gpu_destroy", "lyon_gpu_stream", "lyon_gpu_last_error",
    "lyon_gpu_stroke_path", "lyon_gpu_fill_path", "lyon_gpu_stroke_paths", "lyon_gpu_fill_paths",
    "lyon_gpu_stroke_paths_each", "lyon_gpu_coverage_compare",
    "lyon_gpu_flatten_counts", "lyon_gpu_flatten_paths", "lyon_gpu_synchronize",
    "lyon_gpu_version", "lyon_gpu_stroke_paths_host", "lyon_gpu_fill_paths_host",
    "lyon_gpu_host_alloc", "lyon_gpu_host_free",
    "lyon_gpu_set_timing", "lyon_gpu_last_timings", "lyon_gpu_stroke_paths_noalloc",
    "lyon_srv_create", "lyon_srv_destroy", "lyon_srv_get_config", "lyon_srv_submit", "lyon_srv_poll", "lyon_srv_wait",
    "lyon_srv_release", "lyon_srv_run_load", "lyon_gpu_set_stroke_tuning",
    "lyon_gpu_get_stroke_tuning", "lyon_gpu_autotune_stroke", "lyon_gpu_kernel_launches",
    "lyon_gpu_stroke_path_attributes", "lyon_gpu_stroke_paths_attributes",
    "lyon_gpu_stroke_paths_variable_width", "lyon_gpu_stroke_path_variable_width",
    "lyon_gpu_fill_shapes", "lyon_svg_parse_paths", "lyon_gpu_svg_parse_paths",
    "lyon_gpu_set_fill_tuning", "lyon_gpu_get_fill_tuning", "lyon_gpu_autotune_fill", "lyon_gpu_stroke_paths_custom",
    "lyon_gpu_interpolate_attributes", "lyon_gpu_stroke_path_custom",
    "lyon_gpu_fill_paths_custom", "lyon_gpu_interpolate_fill_attributes",
    "lyon_gpu_fill_path_custom", "lyon_gpu_flatten_arcs", "lyon_gpu_hatch_paths",
    "lyon_gpu_dot_paths", "lyon_gpu_query_sizes", "lyon_gpu_emit_into",
]
