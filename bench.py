"""Benchmark: output vertices/s of batched stroke tessellation on one GB300 (per GPU replica).

Workload (default): 1,000,000 stroke paths, log-normal segment counts (median 12, sigma 1,
clamped to 1..4096), a third each of lines, quadratics and cubics, f32 points uniform in
[0, 1024]^2, half of the paths closed, round joins and caps, tolerance 0.05, per-path widths
uniform in [0.5, 8], u32 indices in one global index space; seeded synthetic data.

One step = one `lyon_gpu_stroke_paths` call (count kernel, index-range check, look-back scan,
emit kernel) over the whole batch. `value` times K steps with inputs resident in HBM; `e2e`
times the C ABI call with host buffers (`lyon_gpu_stroke_paths_host`: inputs copied in, every
output byte copied back to host memory). The roofline is taken for the emit kernel from CUDA
events the library records around it on its stream. The CPU baseline is the oracle (the C++
restatement of lyon's stroker) on a bounded sample with all host threads.

Usage: python bench.py [--gpus N --steps K --warmup W] [--impl reference] [--paths P]
"""

from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

METRIC = "output vertices/s"
UNIT = "vertices/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--paths", type=int, default=1_000_000)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-sample", type=int, default=1_000_000)
    ap.add_argument("--fill-paths", type=int, default=200_000)
    ap.add_argument("--no-fill", action="store_true")
    ap.add_argument("--no-serve", action="store_true")
    ap.add_argument("--no-polylines", action="store_true")
    ap.add_argument("--no-variable-width", action="store_true")
    ap.add_argument("--vw-paths", type=int, default=200_000)
    ap.add_argument("--no-custom-attributes", action="store_true")
    ap.add_argument("--no-producers", action="store_true",
                    help="skip the arc flattening and hatching lines")
    ap.add_argument("--polyline-paths", type=int, default=2_000_000)
    ap.add_argument("--serve-seconds", type=float, default=0.1)
    ap.add_argument("--profile-fill", action="store_true",
                    help="only run the fill warm-up and timed steps (for profilers)")
    ap.add_argument("--fill-lanes", type=int, default=0,
                    help="with --profile-fill: sweepers per warp (0: the library's choice)")
    ap.add_argument("--fill-blocks-per-sm", type=int, default=0,
                    help="with --profile-fill: sweep blocks per SM (0: the library's default)")
    ap.add_argument("--profile", action="store_true",
                    help="only run the warm-up and timed device steps (for profilers)")
    ap.add_argument("--profile-producers", action="store_true",
                    help="only run the stroke/fill custom-attribute, arc and hatching lines "
                         "(one timed step each, no CPU baselines; for profilers)")
    ap.add_argument("--profile-polylines", action="store_true",
                    help="only run the map-polyline stroke (tolerance 0.1, default launch "
                         "settings, --polyline-paths paths) for --warmup + --steps calls "
                         "(for profilers)")
    return ap.parse_args()


def workload_config(n_paths: int) -> dict:
    return {
        "workload": f"batched_stroke_{n_paths}_paths",
        "paths": n_paths,
        "segments": "lognormal(median 12, sigma 1.0), clamp 1..4096; 1/3 line, quad, cubic",
        "coordinates": "f32 uniform [0,1024]^2, 50% closed",
        "join": "round", "caps": "round", "tolerance": 0.05, "line_width": "U[0.5, 8] per path",
        "index_bits": 32, "index_mode": "global",
        "l2": "no flush: inputs (~0.5 GB) and outputs (~52 GB) exceed the 129 MB L2",
        "seed": 2,
    }


def dist_info():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class ClockSampler:
    """Samples nvidia-smi clocks and throttle reasons while the timed region runs."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:  # noqa: BLE001
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:  # noqa: BLE001
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx),
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peak_hbm():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:  # noqa: BLE001
        return 6800.0, "fallback"


def roofline_entry(alg_bytes, kernel_s, kernel, traffic=None):
    """The roofline object of a bench entry: algorithmic bytes over the kernel's event time,
    against the measured HBM copy bandwidth."""
    peak, kind = measured_peak_hbm()
    achieved = alg_bytes / max(kernel_s, 1e-12) / 1e9
    return {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": achieved / peak, "peak_source": kind, "traffic": traffic, "kernel": kernel,
            "algorithmic_bytes": alg_bytes, "kernel_ms": kernel_s * 1e3}


def profiled_figure(name, key):
    """A figure (`key: value` line) from a committed ncu summary under profiles/, if any."""
    p = os.path.join(ROOT, "profiles", name)
    try:
        for line in open(p):
            if line.startswith(key + ":"):
                return float(line.split(":", 1)[1].strip())
    except OSError:
        pass
    return None


def profiled_traffic_per_vertex():
    """DRAM bytes per output vertex of the emit kernel from the committed ncu summary, if any."""
    p = os.path.join(ROOT, "profiles", "stroke_emit_batched_stroke.md")
    try:
        for line in open(p):
            if line.startswith("dram_bytes_per_output_vertex:"):
                return float(line.split(":", 1)[1].strip())
    except OSError:
        pass
    return None


def _oracle_rate(kind, batch, opts, n, threads, ties=None):
    """The oracle over the first n paths: each path tessellated into one reused VertexBuffers per
    thread (lyon's tessellate_path into a cleared buffer), nothing copied into batch arrays.
    Returns (vertices/s, vertices, seconds); `ties` (a dict), when given, receives the oracle's
    near-tie counts (count decisions within 1e-6 of an integer)."""
    from oracle import lyon_oracle as orc
    sub = batch.head(n)
    sub_opts = opts[:n] if len(opts) > 1 else opts
    w = min(n, 2000)
    orc.batch(kind, sub.head(w), sub_opts[:w] if len(sub_opts) > 1 else sub_opts, 32, threads,
              want_output=False)
    t0 = time.perf_counter()
    r = orc.batch(kind, sub, sub_opts, 32, threads, want_output=False)
    dt = time.perf_counter() - t0
    verts = int(r["vtx_counts"].sum())
    if ties is not None:
        ties["near_ties"] = int(r["near_ties"].sum())
        ties["paths_with_near_ties"] = int((r["near_ties"] > 0).sum())
        ties["paths"] = n
    return verts / dt, verts, dt


def cpu_baseline(batch, opts, sample_paths: int, kind: str = "stroke",
                 single_paths: int = 10_000):
    """The oracle (lyon's algorithm restated) on the host cores: all threads on a bounded sample,
    and one thread on a smaller one (lyon itself is single-threaded per tessellator)."""
    threads = os.cpu_count() or 1
    n = min(sample_paths, batch.num_paths)
    ties = {}
    v, verts, dt = _oracle_rate(kind, batch, opts, n, threads, ties)
    n1 = min(single_paths, batch.num_paths)
    v1, verts1, dt1 = _oracle_rate(kind, batch, opts, n1, 1)
    return {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"first {n} paths of the workload, {verts} output vertices, {dt:.2f} s "
                      f"wall on {threads} threads; every path tessellated into a reused "
                      f"per-thread VertexBuffers, outputs not copied into batch arrays",
            "single_thread": {"value": v1, "unit": UNIT, "cores": 1, "kind": "port",
                              "sample": f"first {n1} paths, {verts1} output vertices, "
                                        f"{dt1:.2f} s wall on 1 thread"},
            "near_ties": ties}


def run_reference(args):
    """The reference arm: lyon's algorithm on the host cores (the oracle port: lyon itself is
    Rust and has no toolchain on this machine), every step the whole workload on all threads,
    each path tessellated into a reused per-thread VertexBuffers (outputs not copied into batch
    arrays); warm-up steps run on a tenth of it."""
    rank, world, _ = dist_info()
    if rank != 0:
        return 0
    from lyon_gb300 import workloads
    from oracle import lyon_oracle as orc
    batch, opts = workloads.batched_stroke(args.paths, seed=2)
    threads = os.cpu_count() or 1
    warm = max(1, batch.num_paths // 10)
    for _ in range(args.warmup):
        orc.batch("stroke", batch.head(warm), opts[:warm], 32, threads, want_output=False)
    verts = 0
    t0 = time.perf_counter()
    for _ in range(args.steps):
        r = orc.batch("stroke", batch, opts, 32, threads, want_output=False)
        verts += int(r["vtx_counts"].sum())
    dt = time.perf_counter() - t0
    value = verts / dt
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt / args.steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded)", "config": workload_config(args.paths),
        "impl": "reference",
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"all {batch.num_paths} paths of the workload per step, "
                                   f"each tessellated into a reused per-thread VertexBuffers "
                                   f"(outputs not copied into batch arrays)"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    import torch
    from lyon_gb300 import _native, workloads
    from lyon_gb300 import tessellation as T

    rank, world, local = dist_info()
    dev = local if world > 1 else 0
    torch.cuda.set_device(dev)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")

    if args.profile_polylines:
        ctx = T.Context(dev)
        pb, popts = workloads.map_polylines(args.polyline_paths, seed=4)
        popts["tolerance"] = 0.1
        pdb = T.DeviceBatch.upload(pb, dev)
        pod = T.upload_options(popts, dev)
        stream = torch.cuda.ExternalStream(ctx.stream, device=torch.device("cuda", dev))
        for _ in range(args.warmup):
            res = T.tessellate_paths("stroke", pdb, pod, len(popts), 32, T.INDEX_GLOBAL, 0, ctx)
        ctx.synchronize()
        start = torch.cuda.Event(enable_timing=True)
        end = torch.cuda.Event(enable_timing=True)
        start.record(stream)
        for _ in range(args.steps):
            res = T.tessellate_paths("stroke", pdb, pod, len(popts), 32, T.INDEX_GLOBAL, 0, ctx)
        end.record(stream)
        end.synchronize()
        print(json.dumps({"profile_polylines_ms_per_step": start.elapsed_time(end) / args.steps,
                          "paths": pb.num_paths, "vertices": res.total_vertices}))
        ctx.close()
        return 0
    if args.profile_producers:
        ctx = T.Context(dev)
        args.steps = 1
        out = {}
        for name, fn in (("custom_attributes", run_custom_attributes),
                         ("fill_custom_attributes", run_fill_custom), ("arcs", run_arcs),
                         ("hatching", run_hatching)):
            r = fn(ctx, args, T, baseline=False)
            out[name] = {"value": r["value"], "ms_per_step": r["ms_per_step"]}
        print(json.dumps(out))
        ctx.close()
        return 0
    if args.profile_fill:
        ctx = T.Context(dev)
        lib = ctx.lib
        lib.lyon_gpu_set_timing(ctx.h, 1)
        if args.fill_lanes or args.fill_blocks_per_sm:
            from lyon_gb300 import _native
            tuning = _native.CFillTuning()
            tuning.blocks_per_sm = args.fill_blocks_per_sm
            tuning.lanes = args.fill_lanes
            assert lib.lyon_gpu_set_fill_tuning(ctx.h, ctypes.byref(tuning)) == 0
        out = run_fill(ctx, args, T, world)
        print(json.dumps({k: v for k, v in out.items() if k != "config"}))
        ctx.close()
        return 0
    batch, opts = workloads.batched_stroke(args.paths, seed=2)
    ctx = T.Context(dev)
    lib = ctx.lib
    db = T.DeviceBatch.upload(batch, dev)
    od = T.upload_options(opts, dev)
    stream = torch.cuda.ExternalStream(ctx.stream, device=torch.device("cuda", dev))
    lib.lyon_gpu_set_timing(ctx.h, 1)

    def step():
        return T.tessellate_paths("stroke", db, od, len(opts), 32, T.INDEX_GLOBAL, 0, ctx)

    for _ in range(args.warmup):
        res = step()
    ctx.synchronize()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    emit_ms = []
    start = torch.cuda.Event(enable_timing=True)
    end = torch.cuda.Event(enable_timing=True)
    launches0 = lib.lyon_gpu_kernel_launches()
    with ClockSampler(dev) as clocks:
        start.record(stream)
        t0 = time.perf_counter()
        for _ in range(args.steps):
            res = step()
            ms4 = (ctypes.c_float * 4)()
            lib.lyon_gpu_last_timings(ctx.h, ms4)
            emit_ms.append(ms4[2])
        end.record(stream)
        end.synchronize()
        wall = time.perf_counter() - t0
    launches = lib.lyon_gpu_kernel_launches() - launches0
    torch.cuda.synchronize()
    elapsed_ms = start.elapsed_time(end)
    if world > 1:
        t = torch.tensor([elapsed_ms], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        elapsed_ms = float(t.item())
    verts_per_step = res.total_vertices
    idx_per_step = res.total_indices
    ms_per_step = elapsed_ms / args.steps
    value = verts_per_step * world / (ms_per_step / 1e3)
    if args.profile:
        if rank == 0:
            print(json.dumps({"profile_ms_per_step": ms_per_step, "vertices": verts_per_step}))
        return 0

    # Roofline of the emit kernel: algorithmic bytes / its event-timed duration.
    n = batch.num_paths
    in_bytes = batch.input_bytes(options_bytes_per_path=24)
    out_bytes = verts_per_step * 8 + idx_per_step * 4 + 16 * n
    emit_s = statistics.median(emit_ms) / 1e3
    achieved = (in_bytes + out_bytes) / emit_s / 1e9
    peak, peak_kind = measured_peak_hbm()
    tpv = profiled_traffic_per_vertex()
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "peak_source": peak_kind,
                "traffic": (tpv * verts_per_step) if tpv is not None else None,
                "kernel": "stroke_kernel<true> (emit)",
                "algorithmic_bytes": in_bytes + out_bytes,
                "emit_ms": emit_s * 1e3}

    # End to end through the C ABI with host buffers.
    e2e = None
    if not args.no_e2e:
        e2e = run_e2e(lib, ctx, batch, opts, verts_per_step, idx_per_step, args, T, _native)

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded)", "config": workload_config(args.paths),
        "roofline": roofline, "clocks": clocks.summary(),
        "gpu_launches": launches,
        "wall_ms_per_step": wall / args.steps * 1e3,
        "output_vertices_per_step": verts_per_step, "output_indices_per_step": idx_per_step,
    }
    if e2e is not None:
        line["e2e"] = e2e
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(batch, opts, args.cpu_sample)
        # Count decisions of the workload within 1e-6 of an integer (the oracle's count over
        # the baseline's paths): there lyon on another libm may round the other way.
        line["near_ties"] = line["cpu_baseline"]["near_ties"]
    if rank == 0:
        line["plain_per_path"] = plain_per_path(ctx, db, od, len(opts), value, T)
        if not args.no_fill:
            line["fill"] = run_fill(ctx, args, T, world)
        if not args.no_polylines:
            line["polylines_autotuned"] = run_polylines(ctx, args, T)
        if not args.no_variable_width:
            line["variable_width"] = run_variable_width(ctx, args, T)
        if not args.no_custom_attributes:
            line["custom_attributes"] = run_custom_attributes(ctx, args, T)
            line["fill_custom_attributes"] = run_fill_custom(ctx, args, T)
        if not args.no_producers:
            line["arcs"] = run_arcs(ctx, args, T)
            line["hatching"] = run_hatching(ctx, args, T)
        if not args.no_serve and world == 1:
            del db, od
            ctx.close()
            ctx = None
            torch.cuda.empty_cache()
            line["serving"] = run_serving(args)
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()
    if ctx is not None:
        ctx.close()
    return 0


def run_fill(ctx, args, T, world, batch=None):
    """Batched fill of the glyph workload (200,000 closed paths, tolerance 0.1, u32 global
    indices), non-zero and even-odd; inputs resident; CPU baseline: the oracle on a sample."""
    import torch
    from lyon_gb300 import workloads
    from lyon_gb300.options import FILL_OPTIONS_DTYPE, FillRule
    from oracle import lyon_oracle as orc
    if batch is None:
        batch, _ = workloads.glyph_fill(args.fill_paths, seed=3)
    db = T.DeviceBatch.upload(batch, 0)
    stream = torch.cuda.ExternalStream(ctx.stream, device=torch.device("cuda", 0))
    out = {"workload": f"glyph_fill_{batch.num_paths}_paths",
           "config": {"paths": batch.num_paths, "contours": "1-6 of 8-40 quadratics; 10% stars",
                      "tolerance": 0.1, "index_bits": 32, "index_mode": "global", "seed": 3}}
    threads = os.cpu_count() or 1
    from lyon_gb300 import _native
    saved = _native.CFillTuning()
    ctx.lib.lyon_gpu_get_fill_tuning(ctx.h, ctypes.byref(saved))
    for name, rule in (("non_zero", FillRule.NonZero), ("even_odd", FillRule.EvenOdd)):
        opts = np.zeros(1, dtype=FILL_OPTIONS_DTYPE)
        opts[0] = (0.1, rule, 0, 1)
        od = T.upload_options(opts, 0)
        # The fill autotuner picks blocks per SM and sweepers per warp on a sample of half the
        # batch: a sample with few paths per sweeper favours one sweeper per warp, which is 1.6x
        # slower on the whole batch (measured with a 20,000-path sample).
        tune = None
        if not args.profile_fill:
            best = _native.CFillTuning()
            times = (ctypes.c_float * 10)()
            nc = ctypes.c_uint32()
            cb = db.c()
            sample = min(batch.num_paths, 100_000)
            ctx.lib.lyon_gpu_autotune_fill(ctx.h, ctypes.byref(cb), od.data_ptr(), 1, sample,
                                           ctypes.byref(best), times, ctypes.byref(nc))
            tune = {"chosen": {"blocks_per_sm": best.blocks_per_sm, "lanes": best.lanes},
                    "candidate_ms": [round(float(t), 3) for t in times[:nc.value]],
                    "candidates": "blocks_per_sm {16, 8} x lanes {1, 4, 8, 12, 16}",
                    "sample_paths": sample}
        for _ in range(2):
            res = T.tessellate_paths("fill", db, od, 1, 32, T.INDEX_GLOBAL, 0, ctx)
        ctx.synchronize()
        steps = max(1, args.steps)
        sweep_ms, phases = [], []
        # Phase events on: the end-to-end leg switches them off, and without them the
        # context's last timings would still be another call's.
        ctx.lib.lyon_gpu_set_timing(ctx.h, 1)
        start = torch.cuda.Event(enable_timing=True)
        end = torch.cuda.Event(enable_timing=True)
        launches0 = ctx.lib.lyon_gpu_kernel_launches()
        start.record(stream)
        for _ in range(steps):
            res = T.tessellate_paths("fill", db, od, 1, 32, T.INDEX_GLOBAL, 0, ctx)
            ms4 = (ctypes.c_float * 4)()
            ctx.lib.lyon_gpu_last_timings(ctx.h, ms4)
            sweep_ms.append(ms4[0])
            phases.append([ms4[0], ms4[1], ms4[2], ms4[3]])
        end.record(stream)
        end.synchronize()
        ms = start.elapsed_time(end) / steps
        v = res.total_vertices
        entry = {"metric": "output vertices/s", "value": v / (ms / 1e3), "unit": "vertices/s",
                 "ms_per_step": ms, "vertices_per_step": v, "indices_per_step": res.total_indices,
                 "failed_paths": res.num_failed_paths,
                 "sweep_kernel_ms": statistics.median(sweep_ms),
                 "phases_ms": {"sweep": phases[-1][0], "scan": phases[-1][1],
                               "emit": phases[-1][2], "call": phases[-1][3]},
                 "gpu_launches": ctx.lib.lyon_gpu_kernel_launches() - launches0}
        if tune is not None:
            entry["autotune"] = tune
        if args.profile_fill:
            out[name] = entry
            continue
        # Roofline of the sweep kernel (the dominant one): the call's algorithmic bytes (inputs,
        # output vertices and indices, per-path descriptors) over the sweep's event time.
        alg = (batch.input_bytes(options_bytes_per_path=0) + 16 + v * 8 +
               res.total_indices * 4 + 16 * batch.num_paths)
        tpp = profiled_figure("fill_sweep_glyph_fill.md", "dram_bytes_per_path")
        entry["roofline"] = roofline_entry(
            alg, statistics.median(sweep_ms) / 1e3, "fill_sweep_kernel",
            tpp * batch.num_paths if tpp is not None else None)
        n = min(20_000, batch.num_paths)
        rate, cv, dt = _oracle_rate("fill", batch, opts, n, threads)
        n1 = min(2_000, batch.num_paths)
        rate1, cv1, dt1 = _oracle_rate("fill", batch, opts, n1, 1)
        entry["cpu_baseline"] = {"value": rate, "unit": "vertices/s", "cores": threads,
                                 "kind": "port",
                                 "sample": f"first {n} paths, {cv} output vertices, "
                                           f"{dt:.2f} s wall on {threads} threads",
                                 "single_thread": {"value": rate1, "unit": "vertices/s",
                                                   "cores": 1, "kind": "port",
                                                   "sample": f"first {n1} paths, {cv1} output "
                                                             f"vertices, {dt1:.2f} s wall on "
                                                             f"1 thread"}}
        out[name] = entry
    ctx.lib.lyon_gpu_set_fill_tuning(ctx.h, ctypes.byref(saved))
    return out


def run_variable_width(ctx, args, T):
    """Variable line width (StrokeOptions::variable_line_width): the batched-stroke generator's
    paths (seed 2, round joins and caps, tolerance 0.05) with a width factor per point drawn from
    U[0.5, 2]; one thread per path. CPU baseline: the oracle on a sample."""
    import torch
    from lyon_gb300 import workloads
    from oracle import lyon_oracle as orc
    batch, opts = workloads.batched_stroke(args.vw_paths, seed=2)
    widths = np.random.default_rng(21).uniform(0.5, 2.0, size=len(batch.points)).astype(
        np.float32)
    db = T.DeviceBatch.upload(batch, 0)
    od = T.upload_options(opts, 0)
    wd = torch.from_numpy(widths).cuda()
    stream = torch.cuda.ExternalStream(ctx.stream, device=torch.device("cuda", 0))
    res = T.tessellate_paths("stroke", db, od, len(opts), 32, T.INDEX_GLOBAL, 0, ctx, widths=wd)
    ctx.synchronize()
    steps = max(1, args.steps)
    launches0 = ctx.lib.lyon_gpu_kernel_launches()
    start = torch.cuda.Event(enable_timing=True)
    end = torch.cuda.Event(enable_timing=True)
    start.record(stream)
    for _ in range(steps):
        res = T.tessellate_paths("stroke", db, od, len(opts), 32, T.INDEX_GLOBAL, 0, ctx,
                                 widths=wd)
    end.record(stream)
    end.synchronize()
    ms = start.elapsed_time(end) / steps
    out = {"workload": f"variable_width_{batch.num_paths}_paths",
           "config": {"paths": batch.num_paths, "generator": "batched stroke, seed 2",
                      "width_factors": "U[0.5, 2] per point, seed 21", "index_bits": 32,
                      "index_mode": "global"},
           "metric": "output vertices/s", "value": res.total_vertices / (ms / 1e3),
           "unit": "vertices/s", "ms_per_step": ms, "vertices_per_step": res.total_vertices,
           "gpu_launches": ctx.lib.lyon_gpu_kernel_launches() - launches0}
    # Inputs (with a width factor per point), positions, indices and per-path offsets, over the
    # whole call (both passes of the sequential stepper, the scan).
    alg = (batch.input_bytes(options_bytes_per_path=24) + 4 * len(batch.points) +
           res.total_vertices * 8 + res.total_indices * 4 + 16 * batch.num_paths)
    out["roofline"] = roofline_entry(alg, ms / 1e3, "whole call (stroke_seq_kernel count and emit)")
    threads = os.cpu_count() or 1
    n = min(20_000, batch.num_paths)
    sub = batch.head(n)
    t0 = time.perf_counter()
    r = orc.batch("stroke", sub, opts[:n], 32, threads, want_output=False,
                  widths=widths[:int(batch.point_offsets[n])])
    dt = time.perf_counter() - t0
    cv = int(r["vtx_counts"].sum())
    out["cpu_baseline"] = {"value": cv / dt, "unit": "vertices/s", "cores": threads,
                           "kind": "port",
                           "sample": f"first {n} paths, {cv} output vertices, "
                                     f"{dt:.2f} s wall on {threads} threads"}
    return out


def run_custom_attributes(ctx, args, T, baseline=True):
    """Custom endpoint attributes (lyon_gpu_stroke_paths_custom): the variable-width workload's
    paths with a fixed width and two f32 attributes per point; every vertex's source and its
    interpolated attributes are written beside the positions. CPU baseline: the oracle strokes a
    sample recording sources, then interpolates with numpy."""
    import torch
    from lyon_gb300 import workloads
    from oracle import lyon_oracle as orc
    batch, opts = workloads.batched_stroke(args.vw_paths, seed=2)
    attrs = np.random.default_rng(22).uniform(0.0, 1.0, size=(len(batch.points), 2)).astype(
        np.float32)
    db = T.DeviceBatch.upload(batch, 0)
    od = T.upload_options(opts, 0)
    ad = torch.from_numpy(attrs).cuda()
    stream = torch.cuda.ExternalStream(ctx.stream, device=torch.device("cuda", 0))
    res = T.tessellate_paths("stroke", db, od, len(opts), 32, T.INDEX_GLOBAL, 0, ctx,
                             custom_attributes=ad)
    ctx.synchronize()
    steps = max(1, args.steps)
    launches0 = ctx.lib.lyon_gpu_kernel_launches()
    start = torch.cuda.Event(enable_timing=True)
    end = torch.cuda.Event(enable_timing=True)
    start.record(stream)
    for _ in range(steps):
        res = T.tessellate_paths("stroke", db, od, len(opts), 32, T.INDEX_GLOBAL, 0, ctx,
                                 custom_attributes=ad)
    end.record(stream)
    end.synchronize()
    ms = start.elapsed_time(end) / steps
    out = {"workload": f"custom_attributes_{batch.num_paths}_paths",
           "config": {"paths": batch.num_paths, "generator": "batched stroke, seed 2",
                      "attributes": "2 f32 per point, U[0, 1], seed 22", "width": "fixed",
                      "index_bits": 32, "index_mode": "global",
                      "outputs": "positions, indices, vertex sources, interpolated attributes"},
           "metric": "output vertices/s", "value": res.total_vertices / (ms / 1e3),
           "unit": "vertices/s", "ms_per_step": ms, "vertices_per_step": res.total_vertices,
           "gpu_launches": ctx.lib.lyon_gpu_kernel_launches() - launches0}
    # Inputs with 8 B of attributes per point; per vertex its position, 12 B source and 8 B of
    # interpolated attributes; indices; per-path offsets. Over the whole call.
    alg = (batch.input_bytes(options_bytes_per_path=24) + 8 * len(batch.points) +
           res.total_vertices * (8 + 12 + 8) + res.total_indices * 4 + 16 * batch.num_paths)
    out["roofline"] = roofline_entry(alg, ms / 1e3,
                                     "whole call (warp count, sequential emit, interpolation)")
    if not baseline:
        return out
    threads = os.cpu_count() or 1
    n = min(20_000, batch.num_paths)
    sub = batch.head(n)
    # The oracle's output pass (stroke with sources into per-path buffers, copied to the
    # offsets its count pass gave) and its C interpolation; the count pass is not timed.
    r = orc.batch_stroke_sources(sub, opts[:n], 32, threads)
    t0 = time.perf_counter()
    orc.interpolate_attributes_threads(r["sources"], attrs, threads)
    dt = r["output_pass_s"] + time.perf_counter() - t0
    cv = int(r["vtx_counts"].sum())
    out["cpu_baseline"] = {"value": cv / dt, "unit": "vertices/s", "cores": threads,
                           "kind": "port",
                           "sample": f"first {n} paths, {cv} output vertices, "
                                     f"{dt:.2f} s wall on {threads} threads (output pass "
                                     f"and interpolation)"}
    return out


def _time_calls(ctx, steps, fn):
    """Device time per call of `fn` on the library's stream (after one untimed call), and the
    library's kernel launches during the timed calls."""
    import torch
    stream = torch.cuda.ExternalStream(ctx.stream, device=torch.device("cuda", 0))
    res = fn()
    ctx.synchronize()
    launches0 = ctx.lib.lyon_gpu_kernel_launches()
    start = torch.cuda.Event(enable_timing=True)
    end = torch.cuda.Event(enable_timing=True)
    start.record(stream)
    for _ in range(steps):
        res = fn()
    end.record(stream)
    end.synchronize()
    return res, start.elapsed_time(end) / steps, ctx.lib.lyon_gpu_kernel_launches() - launches0


def run_fill_custom(ctx, args, T, baseline=True):
    """Fills with custom attributes (lyon_gpu_fill_paths_custom): 50,000 glyph paths (seed 3),
    non-zero, two attributes per point; sources and interpolated attributes written beside the
    fill. CPU baseline: the oracle's output pass with sources and its interpolation."""
    import torch
    from lyon_gb300 import workloads
    from lyon_gb300.options import FILL_OPTIONS_DTYPE, FillRule
    from oracle import lyon_oracle as orc
    batch, _ = workloads.glyph_fill(50_000, seed=3)
    opts = np.zeros(1, FILL_OPTIONS_DTYPE)
    opts[0] = (0.1, FillRule.NonZero, 0, 1)
    attrs = np.random.default_rng(23).uniform(size=(len(batch.points), 2)).astype(np.float32)
    db = T.DeviceBatch.upload(batch, 0)
    od = T.upload_options(opts, 0)
    ad = torch.from_numpy(attrs).cuda()
    res, ms, launches = _time_calls(ctx, max(1, args.steps), lambda: T.tessellate_paths(
        "fill", db, od, 1, 32, T.INDEX_GLOBAL, 0, ctx, custom_attributes=ad))
    out = {"workload": f"fill_custom_attributes_{batch.num_paths}_paths",
           "config": {"paths": batch.num_paths, "generator": "glyph fill, seed 3",
                      "fill_rule": "non-zero", "attributes": "2 f32 per point, seed 23",
                      "outputs": "positions, indices, vertex sources, interpolated attributes"},
           "metric": "output vertices/s", "value": res.total_vertices / (ms / 1e3),
           "unit": "vertices/s", "ms_per_step": ms, "vertices_per_step": res.total_vertices,
           "sources_per_step": res.total_sources, "gpu_launches": launches}
    # Inputs with 8 B of attributes per point; per vertex its position, first-source offset and
    # 8 B of interpolated attributes; 12 B per source; indices. Over the whole call.
    alg = (batch.input_bytes(options_bytes_per_path=0) + 16 + 8 * len(batch.points) +
           res.total_vertices * (8 + 8 + 8) + res.total_sources * 12 + res.total_indices * 4)
    out["roofline"] = roofline_entry(alg, ms / 1e3, "whole call (fill sweep with sources, "
                                                    "emit, interpolation)")
    if not baseline:
        return out
    threads = os.cpu_count() or 1
    sub = batch.head(5_000)
    r = orc.batch_fill_sources(sub, opts, 32, threads)
    t0 = time.perf_counter()
    orc.interpolate_fill_attributes_c(r["sources"], r["source_counts"], attrs)
    dt = r["output_pass_s"] + time.perf_counter() - t0
    cv = int(r["vtx_counts"].sum())
    out["cpu_baseline"] = {"value": cv / dt, "unit": "vertices/s", "cores": threads,
                           "kind": "port", "sample": f"first 5000 paths, {cv} output vertices, "
                                                     f"{dt:.2f} s wall on {threads} threads"}
    return out


def run_arcs(ctx, args, T, baseline=True):
    """Arc flattening (lyon_gpu_flatten_arcs): 1,000,000 elliptic arcs (centres in
    [-1000, 1000]^2, radii e^U[-3, 7], sweeps U[-20, 20] rad, seed 24), tolerance 0.1. CPU
    baseline: the oracle, one thread, on 20,000 arcs."""
    import torch
    from oracle import lyon_oracle as orc
    n = 1_000_000
    rng = np.random.default_rng(24)
    a = np.zeros(n, T.ARC_DTYPE)
    a["center_x"] = rng.uniform(-1000, 1000, n)
    a["center_y"] = rng.uniform(-1000, 1000, n)
    a["radius_x"] = np.exp(rng.uniform(-3, 7, n))
    a["radius_y"] = np.exp(rng.uniform(-3, 7, n))
    a["start_angle"] = rng.uniform(-10, 10, n)
    a["sweep_angle"] = rng.uniform(-20, 20, n)
    a["x_rotation"] = rng.uniform(-4, 4, n)
    d = torch.from_numpy(a.view(np.uint8).copy()).cuda()
    res, ms, launches = _time_calls(ctx, max(1, args.steps),
                                    lambda: T.flatten_arcs(d, n, 0.1, ctx))
    out = {"workload": f"arcs_{n}", "config": {"arcs": n, "tolerance": 0.1, "seed": 24},
           "metric": "flattened points/s", "value": res.total_points / (ms / 1e3),
           "unit": "points/s", "ms_per_step": ms, "points_per_step": res.total_points,
           "gpu_launches": launches}
    # 28 B per arc read; 8 B position and 4 B parameter per point, 8 B offset per arc written.
    # The kernels are FP64-bound (f64 trigonometry), so this fraction is low by design.
    alg = n * (28 + 8) + res.total_points * 12
    out["roofline"] = roofline_entry(alg, ms / 1e3, "whole call (arc count and emit kernels)")
    if not baseline:
        return out
    k = 20_000
    t0 = time.perf_counter()
    pts, _, _, _ = orc.flatten_arcs(a[:k].view(orc.ARC_DTYPE), 0.1)
    dt = time.perf_counter() - t0
    out["cpu_baseline"] = {"value": len(pts) / dt, "unit": "points/s", "cores": 1,
                           "kind": "port", "sample": f"first {k} arcs, {len(pts)} points, "
                                                     f"{dt:.2f} s wall, one thread, counting and output passes"}
    return out


def run_hatching(ctx, args, T, baseline=True):
    """Hatching (lyon_gpu_hatch_paths): the fill workload's 200,000 glyph paths hatched every
    2.0 at 0.7 rad with tangents. CPU baseline: the oracle, one thread, on 10,000 paths."""
    import ctypes
    import ctypes.util
    from lyon_gb300 import hatching as H, workloads
    from oracle import lyon_oracle as orc
    batch, _ = workloads.glyph_fill(args.fill_paths, seed=3)
    db = T.DeviceBatch.upload(batch, 0)
    opts = H.HatchingOptions(0.1, 0.7, True)
    res, ms, launches = _time_calls(ctx, max(1, args.steps),
                                    lambda: H.hatch_paths(db, opts, 2.0, ctx))
    out = {"workload": f"hatching_glyph_{batch.num_paths}_paths",
           "config": {"paths": batch.num_paths, "interval": 2.0, "angle": 0.7,
                      "tolerance": 0.1, "tangents": True},
           "metric": "hatch segments/s", "value": res.total / (ms / 1e3), "unit": "segments/s",
           "ms_per_step": ms, "segments_per_step": res.total, "gpu_launches": launches}
    # Path bytes read; 48 B per segment written. Over the whole call.
    alg = batch.input_bytes(options_bytes_per_path=0) + res.total * 48
    out["roofline"] = roofline_entry(alg, ms / 1e3, "whole call (hatch bound, count and emit)")
    if not baseline:
        return out
    libm = ctypes.CDLL(ctypes.util.find_library("m") or "libm.so.6")
    for f in ("cosf", "sinf"):
        getattr(libm, f).restype = ctypes.c_float
        getattr(libm, f).argtypes = [ctypes.c_float]
    prm = [0.1, libm.cosf(0.7), libm.sinf(0.7), libm.cosf(-0.7), libm.sinf(-0.7), 0.0, 0.0,
           2.0, 1.0, 0.0, 0.0]
    k = 10_000
    t0 = time.perf_counter()
    segs, _, _ = orc.hatch(batch.head(k), prm)
    dt = time.perf_counter() - t0
    out["cpu_baseline"] = {"value": len(segs) / dt, "unit": "segments/s", "cores": 1,
                           "kind": "port", "sample": f"first {k} paths, {len(segs)} segments, "
                                                     f"{dt:.2f} s wall, one thread, counting and output passes"}
    return out


def run_polylines(ctx, args, T):
    """Map-like strokes (2,000,000 open polylines, Pareto lengths up to 20,000 points, mixed
    joins, widths 1-8) at tolerances 0.01, 0.1 and 1.0; for each, the autotuner picks the stroke
    launch settings on a 200,000-path sample, then the whole batch is timed with them."""
    import torch
    from lyon_gb300 import _native, workloads
    from oracle import lyon_oracle as orc
    batch, opts = workloads.map_polylines(args.polyline_paths, seed=4)
    db = T.DeviceBatch.upload(batch, 0)
    cb = db.c()
    stream = torch.cuda.ExternalStream(ctx.stream, device=torch.device("cuda", 0))
    saved = _native.CStrokeTuning()
    ctx.lib.lyon_gpu_get_stroke_tuning(ctx.h, ctypes.byref(saved))
    out = {"workload": f"map_polylines_{batch.num_paths}_paths",
           "config": {"lengths": "Pareto alpha 1.2, 2..20000 points", "joins": "miter/bevel/round",
                      "widths": "U[1, 8]", "index_bits": 32, "index_mode": "global", "seed": 4,
                      "autotune_sample_paths": 200_000}}
    threads = os.cpu_count() or 1
    for tol in (0.01, 0.1, 1.0):
        o = opts.copy()
        o["tolerance"] = tol
        od = T.upload_options(o, 0)
        best = _native.CStrokeTuning()
        times = (ctypes.c_float * 16)()
        nc = ctypes.c_uint32()
        ctx.lib.lyon_gpu_autotune_stroke(ctx.h, ctypes.byref(cb), od.data_ptr(), len(o), 200_000,
                                         ctypes.byref(best), times, ctypes.byref(nc))
        res = T.tessellate_paths("stroke", db, od, len(o), 32, T.INDEX_GLOBAL, 0, ctx)
        ctx.synchronize()
        ctx.lib.lyon_gpu_set_timing(ctx.h, 1)
        steps = max(1, args.steps)
        start = torch.cuda.Event(enable_timing=True)
        end = torch.cuda.Event(enable_timing=True)
        launches0 = ctx.lib.lyon_gpu_kernel_launches()
        emit_ms = []
        start.record(stream)
        for _ in range(steps):
            res = T.tessellate_paths("stroke", db, od, len(o), 32, T.INDEX_GLOBAL, 0, ctx)
            ms4 = (ctypes.c_float * 4)()
            ctx.lib.lyon_gpu_last_timings(ctx.h, ms4)
            emit_ms.append(ms4[2])
        end.record(stream)
        end.synchronize()
        ms = start.elapsed_time(end) / steps
        entry = {"metric": "output vertices/s", "value": res.total_vertices / (ms / 1e3),
                 "unit": "vertices/s", "ms_per_step": ms, "vertices_per_step": res.total_vertices,
                 "chosen": {"long_path_points": best.long_path_points,
                            "blocks_per_sm": best.blocks_per_sm,
                            "short_path_points": best.short_path_points},
                 "candidate_ms": [round(float(t), 3) for t in times[:nc.value]],
                 "gpu_launches": ctx.lib.lyon_gpu_kernel_launches() - launches0}
        alg = (batch.input_bytes(options_bytes_per_path=24) + res.total_vertices * 8 +
               res.total_indices * 4 + 16 * batch.num_paths)
        tpv = profiled_figure("stroke_emit_map_polylines_300k.md", "dram_bytes_per_output_vertex")
        entry["roofline"] = roofline_entry(
            alg, statistics.median(emit_ms) / 1e3, "stroke_kernel<true> (emit: warp walk and one-thread short paths)",
            tpv * res.total_vertices if tpv is not None else None)
        if tol == 0.1:
            n = batch.num_paths  # the whole batch: well under a second on the host cores
            sub = batch.head(n)
            t0 = time.perf_counter()
            r = orc.batch("stroke", sub, o[:n], 32, threads, want_output=False)
            dt = time.perf_counter() - t0
            cv = int(r["vtx_counts"].sum())
            entry["cpu_baseline"] = {"value": cv / dt, "unit": "vertices/s", "cores": threads,
                                     "kind": "port",
                                     "sample": f"first {n} paths, {cv} output vertices, "
                                               f"{dt:.2f} s wall on {threads} threads"}
        out[f"tolerance_{tol}"] = entry
    ctx.lib.lyon_gpu_set_stroke_tuning(ctx.h, ctypes.byref(saved))
    return out


def _latency_groups(stats, reqs):
    """p50/p99/p99.9 of a load's request latencies per kind and size class (the latencies come
    in arrival order; arrival k submitted request k % len(reqs))."""
    lat = np.asarray(stats.get("latencies_ms", []), np.float64)
    out = {}
    if len(lat) == 0:
        return out
    kinds = np.array([reqs[k % len(reqs)].kind for k in range(len(lat))])
    sizes = np.array([reqs[k % len(reqs)].count for k in range(len(lat))])
    for kname, kv in (("stroke", 0), ("fill", 1)):
        for sname, sel in (("le_1000_paths", sizes <= 1000), ("gt_1000_paths", sizes > 1000),
                           ("all", sizes > 0)):
            m = (kinds == kv) & sel
            if m.sum() == 0:
                continue
            x = lat[m]
            out[f"{kname}_{sname}"] = {"requests": int(m.sum()),
                                       "p50_ms": float(np.percentile(x, 50)),
                                       "p99_ms": float(np.percentile(x, 99)),
                                       "p999_ms": float(np.percentile(x, 99.9)),
                                       "max_ms": float(x.max())}
    return out


def _guarded(fn, *a):
    """An auxiliary figure: its failure is reported in the line instead of ending the run."""
    try:
        return fn(*a)
    except Exception as e:  # noqa: BLE001
        return {"unavailable": f"{type(e).__name__}: {e}"}


def _serving_cpu_baseline(reqs, count: int = 400):
    """The oracle (lyon restated) serving the same requests on the host cores: the first `count`
    requests of the pool one after another, each tessellated on all threads (outputs not
    written), as a CPU server would take them."""
    from lyon_gb300.path import PathBatch
    from oracle import lyon_oracle as orc
    threads = os.cpu_count() or 1
    sample = reqs[:count]
    t_total, verts = 0.0, 0
    for r in sample:
        b = r.batch
        sub = PathBatch(b.verbs, b.points, b.verb_offsets[r.start:r.start + r.count + 1],
                        b.point_offsets[r.start:r.start + r.count + 1])
        t0 = time.perf_counter()
        res = orc.batch("stroke" if r.kind == 0 else "fill", sub, r.options, 32, threads,
                        want_output=False)
        t_total += time.perf_counter() - t0
        verts += int(res["vtx_counts"].sum())
    return {"value": verts / t_total, "unit": "vertices/s", "cores": threads, "kind": "port",
            "requests_per_s": len(sample) / t_total,
            "sample": f"first {len(sample)} requests of the pool one after another, each on "
                      f"{threads} threads (outputs not written): {verts} output vertices in "
                      f"{t_total:.2f} s"}


def run_serving(args):
    """Serving loop: Poisson arrivals of scenes of 1-5,000 paths (log-uniform), 70 % strokes from
    the plain-stroke generator, 30 % fills from the glyph generator; outputs stay resident; each
    request released on completion. Two stroke workers on high-priority streams, two fill
    workers. Reported: the offered 50,000 requests/s (saturated), the saturation throughput of
    each kind alone, and loads below saturation with p50/p99/p99.9 latency (from the scheduled
    arrival to the output on the device) per kind and size class."""
    from lyon_gb300 import serving, workloads
    sp, so = workloads.plain_stroke(20_000, seed=1)
    fp, fo = workloads.glyph_fill(5_000, seed=3)
    reqs = serving.mixed_requests(sp, so, fp, fo, 4096, seed=5, max_paths=5000)
    small = [r for r in reqs if r.count <= 1000]
    strokes = [r for r in reqs if r.kind == serving.KIND_STROKE]
    fills = [r for r in reqs if r.kind == serving.KIND_FILL]
    srv = serving.Server(0, num_workers=2, num_stroke_workers=2, max_stroke_batch_paths=16384)
    cfg = srv.config()
    try:
        # Warm-up: the largest request of each kind first (buffers grow to their final sizes),
        # then a short mixed load.
        for group in (strokes, fills):
            big = max(group, key=lambda r: r.count)
            t = srv.submit(big)
            srv.wait(t)
            srv.release(t)
        srv.run_load(reqs[:64], rate_per_s=2000.0, duration_s=0.2, seed=1)
        offered = srv.run_load(reqs, rate_per_s=50_000.0, duration_s=args.serve_seconds, seed=2,
                               want_latencies=True)
        sat_stroke = srv.run_load(strokes, rate_per_s=50_000.0, duration_s=0.2, seed=6)
        sat_fill = srv.run_load(fills, rate_per_s=50_000.0, duration_s=0.02, seed=7)
        cap_paths = offered["paths"] / max(offered["elapsed_s"], 1e-9)
        mean_paths = float(np.mean([r.count for r in reqs]))
        moderate_rate = max(50.0, 0.3 * cap_paths / mean_paths)
        moderate = srv.run_load(reqs, rate_per_s=moderate_rate, duration_s=2.0, seed=3,
                                want_latencies=True)
        small_load = srv.run_load(small, rate_per_s=moderate_rate, duration_s=2.0, seed=4,
                                  want_latencies=True)
    finally:
        srv.close()

    in_per_path = ((sp.input_bytes(options_bytes_per_path=24) / sp.num_paths) * 0.7 +
                   (fp.input_bytes(options_bytes_per_path=16) / fp.num_paths) * 0.3)

    def brief(st, pool=None):
        out = {k: st[k] for k in ("offered_rate", "submitted", "completed", "failed",
                                  "achieved_rate", "elapsed_s", "p50_ms", "p99_ms", "p999_ms",
                                  "max_ms", "batches", "mean_batch_paths")} | {
            "vertices_per_s": st["vertices"] / max(st["elapsed_s"], 1e-9),
            "paths_per_s": st["paths"] / max(st["elapsed_s"], 1e-9)}
        # The whole loop against HBM: the requests' algorithmic bytes (inputs estimated from
        # the pools' mean bytes per path, outputs exact) over the load's wall time.
        alg = st["paths"] * in_per_path + st["vertices"] * 8 + st["indices"] * 4
        out["roofline"] = roofline_entry(alg, st["elapsed_s"], "serving loop (wall clock)")
        if pool is not None:
            out["by_kind_and_size"] = _latency_groups(st, pool)
        return out

    return {"workload": "Poisson scenes of 1-5000 paths, 70% plain-stroke / 30% glyph-fill, "
                        "u32, device-resident outputs",
            "workers": {"stroke": cfg["num_stroke_workers"], "fill": cfg["num_workers"],
                        "fill_blocks_per_sm": cfg["fill_blocks_per_sm"],
                        "max_stroke_batch_paths": cfg["max_stroke_batch_paths"]},
            "requests_in_pool": len(reqs), "mean_paths_per_request": mean_paths,
            "cpu_baseline": _guarded(_serving_cpu_baseline, reqs),
            "offered_50k_per_s": brief(offered, reqs),
            "saturation_stroke_only": brief(sat_stroke),
            "saturation_fill_only": brief(sat_fill),
            "below_saturation": brief(moderate, reqs),
            "below_saturation_requests_le_1000_paths": brief(small_load, small)}


def plain_per_path(ctx, db, opts_dev, num_options, batched_vps, T, count: int = 2000):
    """The plain per-path GPU method: the count -> scan -> emit pipeline
    launched once per path from C (lyon_gpu_stroke_paths_each) on the device-resident batch,
    one host wait per path; no Python loop and no host staging. Its rate beside the batched
    call's gives the batched / plain ratio."""
    import torch
    lib = ctx.lib
    cb = db.c()
    tv = ctypes.c_uint64(0)
    r = lib.lyon_gpu_stroke_paths_each(ctx.h, ctypes.byref(cb), opts_dev.data_ptr(),
                                       num_options, 32, 0, 64, ctypes.byref(tv))  # warm-up
    assert r == 0, r
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    r = lib.lyon_gpu_stroke_paths_each(ctx.h, ctypes.byref(cb), opts_dev.data_ptr(),
                                       num_options, 32, 0, count, ctypes.byref(tv))
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    assert r == 0, r
    value = tv.value / dt
    return {"value": value, "unit": UNIT, "paths": count, "vertices": tv.value,
            "us_per_path": dt / count * 1e6,
            "method": "lyon_gpu_stroke_paths_each: one count/scan/emit pipeline per path, "
                      "device-resident inputs, first paths of the workload",
            "batched_over_plain": batched_vps / value}


def run_e2e(lib, ctx, batch, opts, tv, ti, args, T, _native):
    """Times lyon_gpu_stroke_paths_host: host inputs, host outputs (every byte). Inputs and
    outputs live in pinned host memory (cudaHostAlloc through torch), the inputs filled before
    the timed region, as an application keeps its scene there."""
    import torch

    def host_copy(a):
        t = torch.from_numpy(np.ascontiguousarray(a).view(np.uint8).reshape(-1)).pin_memory()
        return t, t.numpy().view(a.dtype)

    hv = torch.empty(int(tv) * 2, dtype=torch.float32, pin_memory=True)
    hi = torch.empty(int(ti), dtype=torch.int32, pin_memory=True)
    vptr, iptr = hv.data_ptr(), hi.data_ptr()
    host_kind = "pinned (cudaHostAlloc), inputs and outputs"
    keep = [host_copy(batch.verbs), host_copy(batch.points), host_copy(batch.verb_offsets),
            host_copy(batch.point_offsets), host_copy(opts)]
    (_, verbs), (_, pts), (_, vo), (_, po), (_, oh) = keep
    hb = _native.CPathBatch(verbs.ctypes.data, pts.ctypes.data, vo.ctypes.data, po.ctypes.data,
                            batch.num_paths)
    status = np.zeros(batch.num_paths, np.int32)
    tvo = ctypes.c_uint64()
    tio = ctypes.c_uint64()

    def call():
        r = lib.lyon_gpu_stroke_paths_host(ctx.h, ctypes.byref(hb), oh.ctypes.data, len(oh), 32,
                                           T.INDEX_GLOBAL, 0, vptr, tv, iptr, ti,
                                           status.ctypes.data, ctypes.byref(tvo),
                                           ctypes.byref(tio))
        if r != 0:
            raise RuntimeError(f"lyon_gpu_stroke_paths_host: {r} {ctx.last_error()}")

    lib.lyon_gpu_set_timing(ctx.h, 0)
    call()
    steps = max(1, args.steps)
    launches0 = lib.lyon_gpu_kernel_launches()
    t0 = time.perf_counter()
    for _ in range(steps):
        call()
    dt = (time.perf_counter() - t0) / steps
    launches = lib.lyon_gpu_kernel_launches() - launches0
    h2d = batch.input_bytes(options_bytes_per_path=24)
    d2h = int(tv) * 8 + int(ti) * 4 + batch.num_paths * 4
    out = {"value": int(tvo.value) / dt, "unit": UNIT, "h2d_bytes_per_step": h2d,
           "d2h_bytes_per_step": d2h, "ms_per_step": dt * 1e3, "steps": steps,
           "host_buffers": host_kind, "gpu_launches": launches}
    # The box's device-to-host link on its own: plain 4 GB copies into the same host buffer, the
    # best of five (the link is shared with the machine's other GPUs and its rate moves from one
    # moment to the next). The call moves d2h bytes, so d2h / this rate approximates the floor
    # under its time.
    if hv.numel() > 0:
        n = min(hv.numel(), (4 << 30) // 4)
        src = torch.empty(n, dtype=torch.float32, device="cuda")
        src.fill_(1.0)
        hv[:n].copy_(src, non_blocking=True)
        torch.cuda.synchronize()
        rates = []
        for _ in range(5):
            t0 = time.perf_counter()
            hv[:n].copy_(src, non_blocking=True)
            torch.cuda.synchronize()
            rates.append(n * 4 / (time.perf_counter() - t0) / 1e9)
        del src
        gbs = max(rates)
        out["link_d2h_gbs"] = gbs
        out["link_d2h_gbs_samples"] = [round(r, 1) for r in rates]
        out["d2h_floor_ms"] = d2h / (gbs * 1e9) * 1e3
    return out


if __name__ == "__main__":
    sys.exit(main())
