#!/usr/bin/env python3
"""Benchmark of the LBVH rebuild + trace hot path on GB300.

Default workload (the per-frame rebuild configuration): a geodesic icosphere
of 2,099,520 fp32 triangles displaced by seeded value-noise fBm, 16 frames
each perturbing every vertex by N(0, 1e-3); every step is one frame: full
LBVH rebuild (depth 20) + 1920x1080 primary rays + shadow ray + one mirror
ray per pixel.  Metric: frame Mtri/s = triangles rebuilt and traced per
second (N / frame time); build Mtri/s and trace Mrays/s are reported beside.

  python bench.py [--steps K] [--warmup W] [--impl ours|reference]
                  [--workload frame|torus|pt] [--gpus N]

Multi-GPU: the path does not shard (one global sort per frame), so N > 1
runs N independent replicas (one per rank, torchrun) and value is the sum
of the replicas' frames over the slowest rank's time.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT / "raytracer-gpupro4_gb300"))

METRIC = "LBVH build Mtri/s; trace Mrays/s; batched/adjoint vs plain, same GB300"
BUILD_BYTES_PER_TRI = 256  # bounds 36 + Morton 44 + sort 68 + emit/refit 108
L2_FLUSH_BYTES = 256 << 20


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=16)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=["frame", "torus", "pt", "adjoint", "batch"], default="frame")
    ap.add_argument("--scenes", type=int, default=256, help="batch workload: number of scenes")
    ap.add_argument("--batch-res", type=int, default=256, help="batch workload: square image size per scene")
    ap.add_argument("--freq", type=int, default=324, help="icosphere frequency (324 -> 2,099,520 triangles)")
    ap.add_argument("--depth", type=int, default=20)
    ap.add_argument("--frames", type=int, default=16)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-components", action="store_true",
                    help="frame workload: skip the batched / path-traced / adjoint component runs")
    return ap.parse_args()


# ---------------------------------------------------------------------------
class Dist:
    def __init__(self):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        self.pg = None

    def init(self, backend):
        if self.world > 1:
            import torch.distributed as dist
            dist.init_process_group(backend=backend)
            self.pg = dist

    def barrier(self):
        if self.pg:
            self.pg.barrier()

    def max(self, x: float) -> float:
        if not self.pg:
            return x
        import torch
        t = torch.tensor([x], dtype=torch.float64, device="cuda" if torch.cuda.is_available() else "cpu")
        self.pg.all_reduce(t, op=self.pg.ReduceOp.MAX)
        return float(t.item())

    def sum(self, x: float) -> float:
        if not self.pg:
            return x
        import torch
        t = torch.tensor([x], dtype=torch.float64, device="cuda" if torch.cuda.is_available() else "cpu")
        self.pg.all_reduce(t)
        return float(t.item())


def replica_rate(dist: "Dist", local_units: float, local_seconds: float) -> float:
    """Whole-job throughput of independent replicas: the units every rank
    processed over the slowest rank's time (units per second)."""
    return dist.sum(float(local_units)) / dist.max(float(local_seconds))


class Clocks:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        rows = []
        try:
            for line in open(self.path):
                f = [x.strip() for x in line.split(",")]
                if len(f) >= 9 and f[1].replace(".", "").isdigit():
                    rows.append(f)
        except OSError:
            pass
        finally:
            try:
                os.unlink(self.path)
            except OSError:
                pass
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm = [float(r[1]) for r in rows]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k].lower().startswith("active")})
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": float(rows[0][2]), "reasons": reasons,
                "samples": len(rows), "power_w_max": max(float(r[3]) for r in rows if r[3].replace(".", "").isdigit())}


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return d.get("hbm_gbs", 6800.0), "measured"
    return 6800.0, "fallback"


def _ncu_summary() -> dict:
    p = ROOT / "profiles" / "ncu_traffic.json"
    try:
        return json.loads(p.read_text())
    except (ValueError, OSError):
        return {}


def ncu_traffic(*kernels: str):
    """Per-launch DRAM traffic (read + write bytes) of a stage's kernels, summed,
    from the committed ncu summary; None when one of them was not captured."""
    d = _ncu_summary().get("dram_bytes", {})
    vals = [d.get(k) for k in kernels]
    return None if any(v is None for v in vals) else int(sum(vals))


def ncu_cache_fractions(kernel: str):
    """L1 / L2 throughput of a kernel (percent of peak) from the committed ncu
    summary: the trace kernels are L1/L2-latency-bound, so these are their
    real utilisation figures beside the HBM-roofline fraction."""
    d = _ncu_summary()
    l1, l2 = d.get("l1_pct", {}).get(kernel), d.get("l2_pct", {}).get(kernel)
    if l1 is None and l2 is None:
        return None
    return {"kernel": kernel, "l1_throughput_pct": l1, "l2_throughput_pct": l2,
            "active_lanes_of_32": d.get("active_lanes", {}).get(kernel)}


# ---------------------------------------------------------------------------
def frame_workload(args):
    from rtgpu import scenes
    if args.workload == "torus":
        tris = scenes.torus()
        frames = [tris]
        cam = scenes.torus_camera()
        name = "torus 65,536 tris, 512x512 primary+shadow+mirror, depth %d" % args.depth
        light = scenes.TORUS_LIGHT
    else:
        s = scenes.icosphere(args.freq)
        frames = [s.frame(k) for k in range(args.frames)]
        cam = scenes.sphere_camera()
        name = ("icosphere %d tris (fBm 0.15, 6 oct), %d frames perturbed N(0,1e-3), full rebuild depth %d, "
                "1920x1080 primary+shadow+mirror" % (s.n_tris, args.frames, args.depth))
        light = scenes.TORUS_LIGHT
    return frames, cam, light, name


def run_ours(args, dist: Dist):
    import torch
    from rtgpu import _lib as L
    from rtgpu import build as B
    from rtgpu.api import LBVH, Context, Frame, Pipe, RayTracer

    B.build_cuda()
    torch.cuda.set_device(dist.local)
    dist.init("nccl")
    dev = torch.device("cuda", dist.local)
    if args.workload in ("pt", "adjoint"):
        return run_pt(args, dist, adjoint=args.workload == "adjoint")
    if args.workload == "batch":
        return run_batch(args, dist)
    frames, cam, light, name = frame_workload(args)
    n = len(frames[0])
    npx = cam.width * cam.height
    host = torch.from_numpy(np.stack(frames)).pin_memory()
    dfr = host.to(dev)
    ctx = Context(dist.local)
    lb = LBVH(ctx, n, args.depth)
    rt = RayTracer(ctx)
    hits = torch.empty((npx, 4), dtype=torch.int32, device=dev)
    leaves = torch.empty(npx, dtype=torch.int32, device=dev)
    mirror = torch.empty((npx, 4), dtype=torch.int32, device=dev)
    mleaves = torch.empty(npx, dtype=torch.int32, device=dev)
    vis = torch.empty(npx, dtype=torch.uint8, device=dev)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.int32, device=dev)

    # algorithmic trace bytes of frame 0: per-ray node visits and triangle
    # tests of the reference's own walk (LBVH_IntersectP in the shader's order,
    # shadow and mirror rays restarted at the primary leaf, closest hit for
    # both), the counts the trace bytes are defined on
    lb.Build(dfr[0])
    _, svis, _, pst, sst, mst = rt.frame_shader_order(lb, cam, light, stats=True)
    ctx.check()
    pst, sst, mst = (x.to(torch.int64).sum(0).tolist() for x in (pst, sst, mst))
    visn = svis.cpu().numpy()
    n_prim = npx
    n_shadow = int((visn >= 2).sum())
    n_mirror = int((visn >= 1).sum())
    bytes_primary = 32 * pst[0] + 40 * pst[1] + 32 * n_prim
    bytes_secondary = 32 * (sst[0] + mst[0]) + 40 * (sst[1] + mst[1]) + 32 * (n_shadow + n_mirror)
    rays_per_frame = n_prim + n_shadow + n_mirror
    # the same figure on this project's own walk (split-axis child order, any-hit
    # shadow rays, shading rays restarted at the primary leaf): its counting
    # variants' box and triangle tests per ray
    ohits, oleaves, opst = rt.primary_leaves(lb, cam, stats=True)
    _, _, _, osst, omst = rt.shadow_mirror_from(lb, cam, light, ohits, oleaves, stats=True)
    ctx.check()
    opst, osst, omst = (x.to(torch.int64).sum(0).tolist() for x in (opst, osst, omst))
    own_primary = 32 * opst[0] + 40 * opst[1] + 32 * n_prim
    own_secondary = 32 * (osst[0] + omst[0]) + 40 * (osst[1] + omst[1]) + 32 * (n_shadow + n_mirror)

    stream = torch.cuda.current_stream(dev)

    def step(k, evs=None):
        f = dfr[k % len(frames)]
        if evs:
            evs[0].record(stream)
        lb.Build(f)
        if evs:
            evs[1].record(stream)
        rt.primary_leaves(lb, cam, out=hits, leaves=leaves)
        if evs:
            evs[2].record(stream)
        rt.shadow_mirror_from(lb, cam, light, hits, leaves, vis=vis, mirror=mirror, mirror_leaves=mleaves)
        if evs:
            evs[3].record(stream)

    # (1) per-stage split: the frame issued call by call with events between stages
    for k in range(args.warmup):
        flush.zero_()
        step(k)
    ctx.check()
    evs = [[torch.cuda.Event(enable_timing=True) for _ in range(4)] for _ in range(args.steps)]
    torch.cuda.synchronize()
    for k in range(args.steps):
        flush.zero_()  # > L2 (129 MB) written between steps, outside the per-step events
        step(args.warmup + k, evs[k])
    torch.cuda.synchronize()
    ctx.check()
    per = np.array([[a.elapsed_time(b) for a, b in zip(e[:-1], e[1:])] for e in evs])  # ms: build, primary, secondary
    build_ms, prim_ms, sec_ms = per.mean(0)
    stream_frame_ms = float(per.sum(1).mean())

    # (2) the timed steps: each frame is one CUDA-graph launch (rt_frame_capture
    # of rebuild + primary + shadow + mirror), one graph per frame buffer
    graphs = [Frame(ctx, lb, dfr[k], cam, light, hits, vis, mirror) for k in range(len(frames))]
    for k in range(args.warmup):
        flush.zero_()
        graphs[k % len(graphs)].launch()
    ctx.check()
    gevs = [[torch.cuda.Event(enable_timing=True) for _ in range(2)] for _ in range(args.steps)]
    dist.barrier()
    torch.cuda.synchronize()
    with Clocks(dist.local) as clk:
        t0 = time.perf_counter()
        for k in range(args.steps):
            flush.zero_()
            gevs[k][0].record(stream)
            graphs[(args.warmup + k) % len(graphs)].launch()
            gevs[k][1].record(stream)
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
    dist.barrier()
    ctx.check()
    step_ms = np.array([e[0].elapsed_time(e[1]) for e in gevs])
    frames_done = dist.sum(float(args.steps))
    value = replica_rate(dist, args.steps * n, float(step_ms.sum()) / 1e3) / 1e6
    for g in graphs:
        g.close()

    # e2e: the public C ABI with host buffers, copies inside the timed region.
    # rt_pipe_* keeps two frames in flight: frame k's pinned soup upload and
    # frame k-1's read-back (hits / visibility / mirror hits into pinned host
    # buffers) run on two copy streams while the frames' captured rebuild +
    # trace graphs run one after another on the context stream; every
    # frame's upload and read-back is inside the timed region.  The warm-up
    # passes every frame's host soup through the pipe once: the first upload
    # from a pinned buffer that has not been read by a copy for a while ran
    # 0.6-2.6 ms instead of 0.37 ms on these hosts (a steady loop reuses its
    # staging buffers, which stay warm).
    e2e = None
    if not args.no_e2e:
        pipe = Pipe(ctx, lb, n, cam, light)
        outs = [(torch.empty((npx, 4), dtype=torch.int32).pin_memory(), torch.empty(npx, dtype=torch.uint8).pin_memory(),
                 torch.empty((npx, 4), dtype=torch.int32).pin_memory()) for _ in range(2)]

        def e2e_frame(k):  # tickets are issued in submission order, from 0
            if k >= 2:
                pipe.wait(k - 2)  # frame k-2 is done with the host buffers frame k reuses
            pipe.submit(host[k % len(frames)], *outs[k % 2])

        e2e_warm = max(args.warmup, len(frames))
        for k in range(e2e_warm):
            e2e_frame(k)
        pipe.wait(e2e_warm - 1)
        dist.barrier()
        torch.cuda.synchronize()
        # at least 64 frames: the pipeline's fill and drain (one upload before
        # the first frame's kernels, one read-back after the last's, ~0.75 ms
        # in all) are spread over the timed frames
        e2e_steps = max(args.steps, 64)
        t0 = time.perf_counter()
        for k in range(e2e_steps):
            e2e_frame(e2e_warm + k)
        last_k = e2e_warm + e2e_steps - 1
        pipe.wait(last_k - 1)
        pipe.wait(last_k)
        te = dist.max(time.perf_counter() - t0)
        ctx.check()
        # the last frame read back equals the device path's result for its soup
        lb.Build(dfr[last_k % len(frames)])
        rt.primary_leaves(lb, cam, out=hits, leaves=leaves)
        e2e_ok = bool(np.array_equal(outs[last_k % 2][0].numpy(), hits.cpu().numpy()))
        e2e_done = dist.sum(float(e2e_steps))
        e2e = {"value": round(e2e_done * n / te / 1e6, 3), "unit": "Mtri/s",
               "h2d_bytes_per_step": int(n * 36), "d2h_bytes_per_step": int(npx * (16 + 1 + 16)),
               "ms_per_step": round(te / e2e_steps * 1e3, 3), "frames": e2e_steps,
               "call": "rt_pipe_submit / rt_pipe_wait: two frames in flight, copies on two copy streams, "
                       "frame graphs in order on the context stream (pinned host soup in, hits / visibility / "
                       "mirror hits out); warm-up: every host soup through the pipe once",
               "matches_device_path": e2e_ok}
        pipe.close()

    peak, peak_kind = measured_peaks()
    # stage: (ms, algorithmic bytes, kernels of the stage's ncu traffic)
    nb = build_launches(n)
    build_label = f"build ({nb} kernels)"
    groups = {"k_trace_primary (+ k_trace_heavy)": (prim_ms, bytes_primary, ("k_trace_primary", "k_trace_heavy")),
              "k_trace_shade (+ k_trace_heavy_team)": (sec_ms, bytes_secondary,
                                                      ("k_trace_shade", "k_trace_heavy_team")),
              build_label: (build_ms, BUILD_BYTES_PER_TRI * n,
                            ("k_bounds", "k_morton_hist") + ("k_onesweep",) * 4 +
                            ("k_emit_tiles", "k_emit_prefix", "k_emit_units", "k_emit_chunks", "k_emit_merge"))}
    dom = max(groups, key=lambda g: groups[g][0])
    ms, byts, kern = groups[dom]
    achieved = byts / (ms / 1e3) / 1e9
    frame_bytes = BUILD_BYTES_PER_TRI * n + bytes_primary + bytes_secondary
    own_frame_bytes = BUILD_BYTES_PER_TRI * n + own_primary + own_secondary
    frame_ms = float(step_ms.mean())

    def frac(b, t_ms):
        return round(b / (t_ms / 1e3) / 1e9 / peak, 4)

    roofline = {"bound": "hbm", "kernel": dom, "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                "frac": round(achieved / peak, 4), "peak_kind": peak_kind,
                "traffic": ncu_traffic(*kern), "algorithmic_bytes_per_launch": int(byts),
                "avg_launch_ms": round(float(ms), 4),
                "bytes_defined_on": "node visits and triangle tests of the reference's own walk (LBVH_IntersectP order)",
                "cache": ncu_cache_fractions(kern[0]),
                "frame": {"algorithmic_bytes": int(frame_bytes), "ms": round(frame_ms, 4),
                          "achieved": round(frame_bytes / (frame_ms / 1e3) / 1e9, 1),
                          "frac": frac(frame_bytes, frame_ms)},
                # the same fractions with the trace bytes of this project's own walk
                "own_walk": {"frame_algorithmic_bytes": int(own_frame_bytes), "frame_frac": frac(own_frame_bytes, frame_ms),
                             "primary_frac": frac(own_primary, prim_ms), "shading_frac": frac(own_secondary, sec_ms)},
                "stages": {"build": {"ms": round(float(build_ms), 4), "frac": frac(BUILD_BYTES_PER_TRI * n, build_ms),
                                     "traffic": ncu_traffic(*groups[build_label][2])},
                           "primary": {"ms": round(float(prim_ms), 4), "frac": frac(bytes_primary, prim_ms),
                                       "cache": ncu_cache_fractions("k_trace_primary")},
                           "shading": {"ms": round(float(sec_ms), 4), "frac": frac(bytes_secondary, sec_ms),
                                       "cache": ncu_cache_fractions("k_trace_shade")}}}
    out = {
        "metric": METRIC, "value": round(value, 3), "unit": "Mtri/s", "n_gpus": dist.world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(float(step_ms.mean()), 4), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded procedural scene)",
        "config": frame_config(name, n, npx, args.depth),
        "timing": {"l2": "flushed between steps (256 MiB write outside the per-step events)",
                   "parallelism": "replicas" if dist.world > 1 else "single GPU"},
        "components": {"graph_frame_ms": round(float(step_ms.mean()), 4), "stream_frame_ms": round(stream_frame_ms, 4),
                       "build_ms": round(float(build_ms), 4), "build_mtri_s": round(n / build_ms / 1e3, 2),
                       "primary_ms": round(float(prim_ms), 4), "secondary_ms": round(float(sec_ms), 4),
                       "trace_mrays_s": round(rays_per_frame / ((prim_ms + sec_ms) / 1e3) / 1e6, 1),
                       "rays_per_frame": {"primary": n_prim, "shadow": n_shadow, "mirror": n_mirror},
                       "wall_s": round(wall, 3)},
        "roofline": roofline,
        "e2e": e2e,
        # per graph: the build's kernels; k_order_begin (which also zeroes the
        # frame's counters), k_trace_primary (which also lists the shading
        # rays), k_trace_heavy; k_trace_shade, k_trace_heavy_team
        "gpu_launches": (nb + 5) * args.steps,
    }
    out["clocks"] = clk.summary()
    if dist.rank == 0 and dist.world == 1 and not args.no_cpu_baseline:
        out["cpu_baseline"] = cpu_frame_baseline(frames[0], cam, light, args.depth, n)
    lb.close()
    ctx.close()
    del dfr, host, graphs
    if args.workload == "frame" and not args.no_components and dist.world == 1:
        # the other forms, each on its own workload, timed the same way
        # (CUDA events on the launching stream, L2 flushed between steps)
        comps = out["components"]
        for key, fn in (("batched", lambda: run_batch(args, dist)), ("pt", lambda: run_pt(args, dist)),
                        ("adjoint", lambda: run_pt(args, dist, adjoint=True))):
            torch.cuda.empty_cache()
            comps[key] = component_summary(fn())
            out["gpu_launches"] += comps[key].get("gpu_launches", 0)
    return out


def build_launches(n: int) -> int:
    """Kernels of one rt_lbvh_build: k_bounds, k_morton_hist, four radix
    passes, k_emit_tiles, k_emit_prefix, k_emit_units, k_emit_chunks (the
    tile level of the merge), k_emit_merge (every level above it)."""
    return 11


def frame_config(name, n, npx, depth):
    return {"workload": name, "triangles": n, "pixels": npx, "depth": depth}


def component_summary(r: dict) -> dict:
    """One form's bench line, nested under the headline's components."""
    keep = ("value", "unit", "ms_per_step", "steps", "warmup", "config", "components", "roofline", "e2e",
            "cpu_baseline", "clocks", "gpu_launches")
    return {k: r[k] for k in keep if k in r}


# ---------------------------------------------------------------------------
def batch_workload(args):
    from rtgpu import scenes
    sizes = scenes.batch_sizes(args.scenes)
    soup = scenes.batch_scene(sizes)
    cams, lights = scenes.batch_views(len(sizes), args.batch_res, args.batch_res)
    name = ("batch of %d random-soup scenes, N_i = round(exp U[ln 1e3, ln 2e5]) (sum %d tris), depth %d, "
            "%dx%d primary+shadow per scene" % (len(sizes), int(sizes.sum()), args.depth, args.batch_res,
                                               args.batch_res))
    return sizes, soup, cams, lights, name


def run_batch(args, dist: Dist):
    """Batched form: every step rebuilds all scenes of the batch and traces a
    primary and a shadow ray per pixel of each, as one CUDA-graph launch of
    the batched build + the persistent (scene, tile) trace kernel, after the
    autotuner has picked the trace's launch shape.  The same work issued as a
    plain per-scene loop (rt_lbvh_build + rt_trace_primary +
    rt_trace_shadow_mirror per scene) is timed beside it."""
    import torch
    from rtgpu import autotune
    from rtgpu.api import LBVH, Batch, BatchFrame, Context, RayTracer

    dev = torch.device("cuda", dist.local)
    sizes, soup, cams, lights, name = batch_workload(args)
    S = len(sizes)
    total = int(sizes.sum())
    off = np.concatenate([[0], np.cumsum(sizes)])
    W = H = args.batch_res
    npx = W * H
    host = torch.from_numpy(soup).pin_memory()
    dsoup = host.to(dev)
    ctx = Context(dist.local)
    stream = torch.cuda.current_stream(dev)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.int32, device=dev)

    b = Batch(ctx, sizes, args.depth)
    b.set_views(cams, lights)
    hits, vis = b.alloc_outputs()
    b.build(dsoup)
    ctx.check()
    tune_cache = autotune.TuneCache(Path(tempfile.gettempdir()) / "rtgpu_batch_tuning.json")
    best = autotune.autotune_batch(b, hits, vis, cache=tune_cache)

    # plain per-scene loop with the per-ray test counters: algorithmic bytes
    lb = LBVH(ctx, int(sizes.max()), args.depth)
    rt = RayTracer(ctx)
    phits = torch.empty((S, npx, 4), dtype=torch.int32, device=dev)
    pleaves = torch.empty(npx, dtype=torch.int32, device=dev)
    pvis = torch.empty((S, npx), dtype=torch.uint8, device=dev)
    nb = nt = 0
    n_shadow = 0
    for s in range(S):  # counts of the reference's own walk (LBVH_IntersectP order), per scene
        lb.Build(dsoup[off[s]:off[s + 1]])
        _, svis, _, pst, sst, _ = rt.frame_shader_order(lb, cams[s], lights[s], stats=True, with_mirror=False)
        nb += int(pst[:, 0].sum() + sst[:, 0].sum())
        nt += int(pst[:, 1].sum() + sst[:, 1].sum())
        n_shadow += int((svis >= 2).sum())
    ctx.check()
    rays = S * npx + n_shadow
    trace_bytes = 32 * nb + 40 * nt + 32 * rays

    def plain_step():
        for s in range(S):
            lb.Build(dsoup[off[s]:off[s + 1]])
            rt.primary_leaves(lb, cams[s], out=phits[s], leaves=pleaves)
            rt.shadow_mirror_from(lb, cams[s], lights[s], phits[s], pleaves, vis=pvis[s], with_mirror=False)

    def timed(fn, steps):
        evs = [[torch.cuda.Event(enable_timing=True) for _ in range(2)] for _ in range(steps)]
        torch.cuda.synchronize()
        for k in range(steps):
            flush.zero_()
            evs[k][0].record(stream)
            fn()
            evs[k][1].record(stream)
        torch.cuda.synchronize()
        ctx.check()
        return np.array([a.elapsed_time(c) for a, c in evs])

    for _ in range(args.warmup):
        flush.zero_()
        plain_step()
    plain_ms = timed(plain_step, max(1, min(args.steps, 4)))

    # batched, stream-issued, with the build / trace split
    def split_step(evs):
        evs[0].record(stream)
        b.build(dsoup)
        evs[1].record(stream)
        b.trace(hits, vis)
        evs[2].record(stream)

    for _ in range(args.warmup):
        flush.zero_()
        b.build(dsoup)
        b.trace(hits, vis)
    sevs = [[torch.cuda.Event(enable_timing=True) for _ in range(3)] for _ in range(args.steps)]
    torch.cuda.synchronize()
    for k in range(args.steps):
        flush.zero_()
        split_step(sevs[k])
    torch.cuda.synchronize()
    ctx.check()
    per = np.array([[e[0].elapsed_time(e[1]), e[1].elapsed_time(e[2])] for e in sevs])
    build_ms, trace_ms = per.mean(0)
    # parity of the batched frame with the plain loop (same trees, same rays)
    assert torch.equal(hits.view(S, npx, 4), phits) and torch.equal(vis.view(S, npx), pvis), \
        "batched and per-scene results differ"

    # timed steps: one CUDA-graph launch per batched frame
    frame = BatchFrame(ctx, b, dsoup, hits, vis)
    for _ in range(args.warmup):
        flush.zero_()
        frame.launch()
    ctx.check()
    dist.barrier()
    with Clocks(dist.local) as clk:
        step_ms = timed(frame.launch, args.steps)
    dist.barrier()
    value = replica_rate(dist, args.steps * total, float(step_ms.sum()) / 1e3) / 1e6

    # e2e: pinned host soup in, hits + visibility out, inside the timed region.
    # Two batches on two streams take alternate frames (upload, graph launch,
    # read-back queued on the lane's stream), so one frame's copies overlap the
    # other frame's kernels.
    e2e = None
    if not args.no_e2e:
        frame.close()
        lanes = [(b, torch.cuda.current_stream(dev), dsoup, hits, vis)]
        st2 = torch.cuda.Stream(dev)
        ctx2 = Context(dist.local, stream=st2)
        b2 = Batch(ctx2, sizes, args.depth)
        b2.set_views(cams, lights)
        b2.tuning = best
        h2, v2 = b2.alloc_outputs()
        lanes.append((b2, st2, torch.empty_like(dsoup), h2, v2))
        graphs, outs = [], []
        for bq, sq, dq, hq, vq in lanes:
            with torch.cuda.stream(sq):
                dq.copy_(host, non_blocking=True)
            sq.synchronize()
            graphs.append(BatchFrame(bq.ctx, bq, dq, hq, vq))
            outs.append((torch.empty(hq.shape, dtype=hq.dtype).pin_memory(),
                         torch.empty(vq.shape, dtype=vq.dtype).pin_memory()))

        def e2e_step(k):
            q = k % 2
            bq, sq, dq, hq, vq = lanes[q]
            sq.synchronize()  # this lane's previous frame is done with its buffers
            with torch.cuda.stream(sq):
                dq.copy_(host, non_blocking=True)
                graphs[q].launch()
                outs[q][0].copy_(hq, non_blocking=True)
                outs[q][1].copy_(vq, non_blocking=True)

        for k in range(args.warmup):
            e2e_step(k)
        torch.cuda.synchronize()
        dist.barrier()
        t0 = time.perf_counter()
        for k in range(args.steps):
            e2e_step(args.warmup + k)
        torch.cuda.synchronize()
        te = dist.max(time.perf_counter() - t0)
        e2e_ok = all(torch.equal(outs[q][0], phits.view(-1, 4).cpu()) and torch.equal(outs[q][1], pvis.view(-1).cpu())
                     for q in range(2))
        e2e = {"value": round(dist.sum(float(args.steps)) * total / te / 1e6, 3), "unit": "Mtri/s",
               "h2d_bytes_per_step": int(host.numel() * 4), "d2h_bytes_per_step": int(hits.numel() * 4 + vis.numel()),
               "ms_per_step": round(te / args.steps * 1e3, 3),
               "call": "two batches on two streams, alternate frames: pinned soup -> rt_batch_frame_capture graph "
                       "(build + trace) -> pinned hits/vis",
               "matches_device_path": bool(e2e_ok)}
        for g in graphs:
            g.close()
        b2.close()
        ctx2.close()
    else:
        frame.close()

    peak, peak_kind = measured_peaks()
    groups = {"k_batch_trace": (trace_ms, trace_bytes), "batched build (12 kernels)": (build_ms, BUILD_BYTES_PER_TRI * total)}
    dom = max(groups, key=lambda g: groups[g][0])
    ms, byts = groups[dom]
    achieved = byts / (ms / 1e3) / 1e9
    out = {
        "metric": METRIC, "value": round(value, 3), "unit": "Mtri/s", "n_gpus": dist.world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(float(step_ms.mean()), 4), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded random soups)",
        "config": batch_config(name, S, total, npx, args.depth),
        "timing": {"l2": "flushed between steps (256 MiB write outside the per-step events); inputs 416 MB > L2",
                   "parallelism": "replicas" if dist.world > 1 else "single GPU"},
        "components": {"graph_frame_ms": round(float(step_ms.mean()), 4), "build_ms": round(float(build_ms), 4),
                       "trace_ms": round(float(trace_ms), 4), "build_mtri_s": round(total / build_ms / 1e3, 1),
                       "trace_mrays_s": round(rays / (trace_ms / 1e3) / 1e6, 1),
                       "rays": {"primary": S * npx, "shadow": n_shadow},
                       "plain_loop_ms": round(float(plain_ms.mean()), 4),
                       "batched_vs_plain": round(float(plain_ms.mean()) / float(step_ms.mean()), 3),
                       "tuning": best},
        "roofline": {"bound": "hbm", "kernel": dom, "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 4), "peak_kind": peak_kind, "traffic": ncu_traffic(dom),
                     "algorithmic_bytes_per_launch": int(byts), "avg_launch_ms": round(float(ms), 4)},
        "e2e": e2e,
        # per graph: 12 build kernels, k_reset_words, k_batch_trace (primary rays, listing the
        # shadow rays), k_trace_shade (the shadow rays)
        "gpu_launches": 15 * args.steps,
    }
    out["clocks"] = clk.summary()
    if dist.rank == 0 and dist.world == 1 and not args.no_cpu_baseline:
        out["cpu_baseline"] = cpu_batch_baseline(soup, off, cams, lights, args.depth,
                                                 budget_s=8.0 if args.workload == "frame" else 15.0)
    b.close()
    lb.close()
    ctx.close()
    return out


def batch_config(name, scenes_n, total, npx, depth):
    return {"workload": name, "scenes": scenes_n, "triangles": total, "pixels_per_scene": npx, "depth": depth}


def cpu_batch_baseline(soup, off, cams, lights, depth, budget_s: float = 15.0):
    """Scenes of the batch on the host (oracle port: build on 1 thread, primary
    + shadow on all cores) until about budget_s seconds have passed."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle as O
    O.build_oracle()
    nth = O.nthreads_default()
    done_tris = 0
    t0 = time.perf_counter()
    s = 0
    while s < len(off) - 1 and time.perf_counter() - t0 < budget_s:
        tris = soup[off[s]:off[s + 1]]
        nodes, ids, _, _ = O.lbvh_build(tris, depth)
        prim = O.trace(nodes, depth, ids, tris, O.primary_rays(cams[s]), nthreads=nth)
        O.shadow_mirror(nodes, depth, ids, tris, cams[s], lights[s], prim, nthreads=nth)
        done_tris += len(tris)
        s += 1
    dt = time.perf_counter() - t0
    return {"value": round(done_tris / dt / 1e6, 4), "unit": "Mtri/s", "cores": nth, "kind": "port",
            "sample": f"first {s} scenes ({done_tris} tris) in {dt:.1f}s: build on 1 thread, primary+shadow on {nth}",
            "cpu": _cpu_name()}


def cpu_frame_baseline(tris, cam, light, depth, n, nthreads=None):
    """One frame on the host: the oracle port (restated LBVH::Build, 1 thread as
    the reference runs it) + primary/shadow/mirror traversal on all cores."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle as O
    O.build_oracle()
    nth = nthreads or O.nthreads_default()
    t0 = time.perf_counter()
    nodes, ids, keys, _ = O.lbvh_build(tris, depth)
    t1 = time.perf_counter()
    hits = O.trace(nodes, depth, ids, tris, O.primary_rays(cam), nthreads=nth)
    O.shadow_mirror(nodes, depth, ids, tris, cam, light, hits, nthreads=nth)
    t2 = time.perf_counter()
    return {"value": round(n / (t2 - t0) / 1e6, 4), "unit": "Mtri/s", "cores": nth, "kind": "port",
            "sample": f"1 frame: build {t1 - t0:.2f}s on 1 thread, primary+shadow+mirror {t2 - t1:.2f}s on {nth} threads",
            "cpu": _cpu_name()}


def _cpu_name():
    try:
        for line in open("/proc/cpuinfo"):
            if line.lower().startswith(("model name", "hardware", "cpu part")):
                return line.split(":", 1)[1].strip()
    except OSError:
        pass
    import platform
    return platform.processor() or platform.machine()


def run_reference(args, dist: Dist):
    """Reference arm: the reference's CPU algorithm on the host cores (its LBVH
    build single-threaded as written, traversal over all cores), one frame per
    step, on the same workload and metric."""
    if dist.rank != 0:
        return None
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle as O
    O.build_oracle()
    if args.workload in ("pt", "adjoint"):
        return {"impl": "reference", "unavailable": "the reference has no CPU path tracer or adjoint; its GI is "
                "an HLSL shader (unavailable on this box)"}
    if args.workload == "batch":
        return run_reference_batch(args, dist, O)
    frames, cam, light, name = frame_workload(args)
    n = len(frames[0])
    nth = O.nthreads_default()
    use_ref = O.ref_available()
    kind = "reference" if use_ref else "port"

    def frame(k):
        tris = frames[k % len(frames)]
        if use_ref:  # reference LBVH::Build and LBVH::IntersectP compiled from its sources
            ref = O.RefStructure(tris, "lbvh", args.depth)
            nodes, ids = ref.nodes(), ref.ids()
            prim = np.zeros(cam.width * cam.height, O.HIT_DTYPE)
            hid, t, u, v = ref.intersect(O.primary_rays(cam), nthreads=nth)
            prim["id"], prim["t"], prim["u"], prim["v"] = hid, t, u, v
            O.shadow_mirror(nodes, args.depth, ids, tris, cam, light, prim, nthreads=nth)
            ref.close()
        else:
            nodes, ids, _, _ = O.lbvh_build(tris, args.depth)
            prim = O.trace(nodes, args.depth, ids, tris, O.primary_rays(cam), nthreads=nth)
            O.shadow_mirror(nodes, args.depth, ids, tris, cam, light, prim, nthreads=nth)

    for k in range(args.warmup):
        frame(k)
    t0 = time.perf_counter()
    for k in range(args.steps):
        frame(args.warmup + k)
    dt = time.perf_counter() - t0
    value = args.steps * n / dt / 1e6
    return {"metric": METRIC, "value": round(value, 4), "unit": "Mtri/s", "n_gpus": dist.world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(dt / args.steps * 1e3, 3), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded procedural scene)",
            "config": frame_config(name, n, cam.width * cam.height, args.depth),
            "impl": "reference",
            "cpu_baseline": {"value": round(value, 4), "unit": "Mtri/s", "cores": nth, "kind": kind,
                             "sample": "every step one full frame: LBVH build on 1 thread, primary/shadow/mirror "
                                       f"on {nth} threads", "cpu": _cpu_name()},
            "e2e": {"value": round(value, 4), "unit": "Mtri/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def run_reference_batch(args, dist: Dist, O):
    """Reference arm of the batched workload: the reference has no batched
    form, so each step is the per-scene loop on the host (LBVH::Build on one
    thread, primary + shadow on all cores) over a rotating sample of 16 scenes."""
    sizes, soup, cams, lights, name = batch_workload(args)
    off = np.concatenate([[0], np.cumsum(sizes)])
    nth = O.nthreads_default()
    use_ref = O.ref_available()
    per_step = 16

    def one(s):
        tris = soup[off[s]:off[s + 1]]
        if use_ref:
            ref = O.RefStructure(tris, "lbvh", args.depth)
            nodes, ids = ref.nodes(), ref.ids()
            prim = np.zeros(cams[s].width * cams[s].height, O.HIT_DTYPE)
            hid, t, u, v = ref.intersect(O.primary_rays(cams[s]), nthreads=nth)
            prim["id"], prim["t"], prim["u"], prim["v"] = hid, t, u, v
            ref.close()
        else:
            nodes, ids, _, _ = O.lbvh_build(tris, args.depth)
            prim = O.trace(nodes, args.depth, ids, tris, O.primary_rays(cams[s]), nthreads=nth)
        O.shadow_mirror(nodes, args.depth, ids, tris, cams[s], lights[s], prim, nthreads=nth)
        return len(tris)

    k = 0
    for _ in range(args.warmup):
        for _ in range(per_step):
            one(k % len(sizes))
            k += 1
    t0 = time.perf_counter()
    tris_done = 0
    for _ in range(args.steps):
        for _ in range(per_step):
            tris_done += one(k % len(sizes))
            k += 1
    dt = time.perf_counter() - t0
    value = tris_done / dt / 1e6
    kind = "reference" if use_ref else "port"
    return {"metric": METRIC, "value": round(value, 4), "unit": "Mtri/s", "n_gpus": dist.world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(dt / args.steps * 1e3, 3), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded random soups)",
            "config": batch_config(name, len(sizes), int(sizes.sum()), args.batch_res * args.batch_res, args.depth),
            "impl": "reference",
            "cpu_baseline": {"value": round(value, 4), "unit": "Mtri/s", "cores": nth, "kind": kind,
                             "sample": f"every step {per_step} scenes of the batch (rotating): LBVH build on 1 thread, "
                                       f"primary+shadow on {nth} threads", "cpu": _cpu_name()},
            "e2e": {"value": round(value, 4), "unit": "Mtri/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def run_pt(args, dist: Dist, adjoint: bool = False):
    """Path-traced GI (closed box + 262,144 random triangles, 1024x1024, 4 spp,
    4 bounces), or with adjoint=True the differentiable workload (same scene at
    512x512, 8 spp, 3 bounces: forward render + L2 image loss + adjoint
    gradients w.r.t. every albedo and the emitter radiance).  A step = LBVH
    rebuild + render (+ loss and backward)."""
    import torch
    from rtgpu import scenes
    from rtgpu.api import LBVH, Context, RayTracer
    from rtgpu.autograd import render
    dev = torch.device("cuda", dist.local)
    sc = scenes.gi_box(262144, seed=3)
    if adjoint:
        W = H = 512
        spp, bounces = 8, 3
    else:
        W = H = 1024
        spp, bounces = 4, 4
    cam = scenes.gi_camera(W, H)
    n = len(sc.tris)
    ctx = Context(dist.local)
    lb = LBVH(ctx, n, args.depth)
    rt = RayTracer(ctx)
    tris = torch.from_numpy(sc.tris).to(dev)
    alb = torch.from_numpy(sc.albedo).to(dev)
    em = torch.from_numpy(sc.emission).to(dev)
    mask = torch.from_numpy((sc.emission[:, 0] > 0).astype(np.float32)).to(dev)
    le = torch.tensor([10.0, 10.0, 10.0], device=dev)
    img = torch.empty((W * H, 4), dtype=torch.float32, device=dev)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.int32, device=dev)
    lb.Build(tris)
    # walk counts of one render (this project's walk): the algorithmic bytes
    _, cnt = rt.pathtrace_counted(lb, alb, em, cam, spp, bounces, 999)
    target = None
    if adjoint:
        rng = np.random.Generator(np.random.PCG64(7))
        talb = np.clip(sc.albedo + rng.uniform(-0.1, 0.1, sc.albedo.shape), 0, 1).astype(np.float32)
        with torch.no_grad():
            target = render(torch.from_numpy(talb).to(dev), le, mask, rt, lb, cam, spp, bounces, 12345)
    stream = torch.cuda.current_stream(dev)

    def step(k, evs=None):
        seed = 1000 + k
        if evs:
            evs[0].record(stream)
        lb.Build(tris)
        if evs:
            evs[1].record(stream)
        if adjoint:
            a = alb.clone().requires_grad_(True)
            lp = le.clone().requires_grad_(True)
            out = render(a, lp, mask, rt, lb, cam, spp, bounces, seed)
            if evs:
                evs[2].record(stream)
            loss = ((out[:, :3] - target[:, :3]) ** 2).mean()
            loss.backward()
        else:
            rt.pathtrace(lb, alb, em, cam, spp, bounces, seed, out=img)
            if evs:
                evs[2].record(stream)
        if evs:
            evs[3].record(stream)

    for k in range(args.warmup):
        flush.zero_()
        step(k)
    ctx.check()
    evs = [[torch.cuda.Event(enable_timing=True) for _ in range(4)] for _ in range(args.steps)]
    dist.barrier()
    torch.cuda.synchronize()
    with Clocks(dist.local) as clk:
        for k in range(args.steps):
            flush.zero_()
            step(args.warmup + k, evs[k])
        torch.cuda.synchronize()
    dist.barrier()
    ctx.check()
    per = np.array([[e[0].elapsed_time(e[1]), e[1].elapsed_time(e[2]), e[2].elapsed_time(e[3])] for e in evs])
    build_ms, fwd_ms, bwd_ms = (float(x) for x in per.mean(0))
    step_ms = per.sum(1)
    value = replica_rate(dist, W * H * spp * args.steps, float(step_ms.sum()) / 1e3) / 1e6
    name = (f"GI box {n} tris, {W}x{H}, {spp} spp, {bounces} bounces" +
            (", forward + L2 loss + adjoint (albedo x3, emitter radiance)" if adjoint else ""))
    # algorithmic bytes: per traced segment 32 per box test + 40 per triangle
    # test + 32 (ray in, hit out); 12 B albedo per hit; 16 B accumulator per
    # pixel-sample.  The adjoint kernel replays the same walk and adds a 12 B
    # gradient atomic per hit and the 16 B dL/dI read per pixel.
    trace_bytes = 32 * cnt["box_tests"] + 40 * cnt["tri_tests"] + 32 * cnt["segments"]
    fwd_bytes = trace_bytes + 12 * cnt["hits"] + 16 * W * H * spp
    bwd_bytes = trace_bytes + 24 * cnt["hits"] + 16 * W * H
    peak, peak_kind = measured_peaks()
    kern, k_ms, k_bytes = (("k_pathtrace_adjoint", bwd_ms, bwd_bytes) if adjoint else ("k_pathtrace", fwd_ms, fwd_bytes))
    achieved = k_bytes / (k_ms / 1e3) / 1e9
    roofline = {"bound": "hbm", "kernel": kern, "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                "frac": round(achieved / peak, 4), "peak_kind": peak_kind, "traffic": ncu_traffic(kern),
                "algorithmic_bytes_per_launch": int(k_bytes), "avg_launch_ms": round(k_ms, 4),
                "bytes_defined_on": "box / triangle tests of this project's walk (rt_pathtrace_counted)",
                "cache": ncu_cache_fractions(kern),
                "walk": {k: int(v) for k, v in cnt.items()}}
    if adjoint:
        step_bytes = BUILD_BYTES_PER_TRI * n + fwd_bytes + bwd_bytes
        roofline["step"] = {"algorithmic_bytes": int(step_bytes), "ms": round(float(step_ms.mean()), 4),
                            "frac": round(step_bytes / (float(step_ms.mean()) / 1e3) / 1e9 / peak, 4)}
    segs_per_s = cnt["segments"] / (fwd_ms / 1e3) / 1e6
    out = {"metric": METRIC, "value": round(value, 3), "unit": "Msamples/s", "n_gpus": dist.world,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(float(step_ms.mean()), 4),
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
           "data": "synthetic (seeded procedural scene)",
           "config": {"workload": name, "triangles": n, "pixels": W * H, "spp": spp, "bounces": bounces,
                      "depth": args.depth},
           "timing": {"l2": "flushed between steps (256 MiB write outside the events)"},
           "components": {"build_ms": round(build_ms, 4), "forward_ms": round(fwd_ms, 4),
                          "forward_msegments_s": round(segs_per_s, 1)},
           "roofline": roofline,
           "clocks": clk.summary(),
           # per step: 10 build kernels + the render (+ the adjoint kernel)
           "gpu_launches": (build_launches(n) + 1 + (1 if adjoint else 0)) * args.steps}
    if adjoint:
        out["components"]["backward_ms"] = round(bwd_ms, 4)
        out["components"]["backward_over_forward"] = round(bwd_ms / fwd_ms, 3)
        out["components"]["adjoint_vs_plain"] = {
            "forward_only_msamples_s": round(W * H * spp / ((build_ms + fwd_ms) / 1e3) / 1e6, 3),
            "forward_plus_adjoint_msamples_s": round(value, 3)}
    if dist.rank == 0 and dist.world == 1 and not args.no_cpu_baseline:
        out["cpu_baseline"] = cpu_pt_baseline(sc, cam, spp, bounces, args.depth, adjoint=adjoint)
    lb.close()
    ctx.close()
    return out


def cpu_pt_baseline(sc, cam, spp, bounces, depth, adjoint=False):
    """The oracle's path tracer (and with adjoint=True its FP64 adjoint) on a
    128x128 crop of the same image (same pixels and sample streams), all host
    cores, after the oracle's LBVH build of the scene."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle as O
    O.build_oracle()
    nth = O.nthreads_default()
    nodes, ids, _, _ = O.lbvh_build(sc.tris, depth)
    win = ((cam.width - 128) // 2, (cam.height - 128) // 2, 128, 128)
    t0 = time.perf_counter()
    img = O.pathtrace(nodes, depth, ids, sc.tris, sc.albedo, sc.emission, cam, spp, bounces, 1000, nthreads=nth,
                      window=win)
    if adjoint:
        g = np.zeros_like(img)
        g[:, :3] = 1.0 / (cam.width * cam.height * 3)
        O.pathtrace_adjoint(nodes, depth, ids, sc.tris, sc.albedo, sc.emission, cam, spp, bounces, 1000, g,
                            nthreads=nth, window=win)
    dt = time.perf_counter() - t0
    what = "forward + FP64 adjoint" if adjoint else "forward"
    return {"value": round(128 * 128 * spp / dt / 1e6, 4), "unit": "Msamples/s", "cores": nth, "kind": "port",
            "sample": f"128x128 crop, {spp} spp, {bounces} bounces, {what}, {dt:.2f}s on {nth} threads",
            "cpu": _cpu_name()}


def main():
    args = parse()
    dist = Dist()
    if args.impl == "reference":
        out = run_reference(args, dist)
    else:
        out = run_ours(args, dist)
    if out is not None and dist.rank == 0:
        print(json.dumps(out), flush=True)


if __name__ == "__main__":
    main()
