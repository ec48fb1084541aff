#!/usr/bin/env python3
"""Benchmark of the GB300 wavefront path-tracing pass.

Workload (the plain pass at scale): the procedural terrain scene of 1,482,242
triangles (512 x 512-vertex fBm heightfield + 2000 UV spheres, gradient sky
baked to a 1024 x 512 RGBA16F equirect map with an importance-sampling alias table, one
sun), rendered at 1920 x 1080, 64 spp, 8 extend segments (primary + 7
bounces), fp32 accumulation.  A step is one full frame.  Inputs are synthetic
and seeded (no dataset exists for this pass).

Metric: Mrays/s = rays entering the closest-hit (extend) kernel per second of
device time; frames/s reported beside it.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

`--impl reference` times the CPU implementation of the pass (the
multithreaded C++ oracle: the reference's own pass runs only through a
graphics API's ray-tracing pipeline, which this machine does not have) on the
host cores, on the same workload, as a bounded sample per step.
Prints ONE JSON line (rank 0).
"""
from __future__ import annotations

import argparse
import importlib
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Mrays/s (extend rays entering closest-hit) at 1 GB300, plain wavefront PT"
DEV_VIEW_BYTES = 128  # bytes of the per-view record the render call uploads (DevView)
EXTEND_BYTES_PER_RAY = 48  # 32 B ray read + 16 B hit written (compulsory HBM)
NODE_BYTES, TRI_BYTES = 80, 48


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=5)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--width", type=int, default=1920)
    p.add_argument("--height", type=int, default=1080)
    p.add_argument("--spp", type=int, default=64)
    p.add_argument("--segments", type=int, default=8)
    p.add_argument("--grid", type=int, default=512)
    p.add_argument("--spheres", type=int, default=2000)
    p.add_argument("--seed", type=int, default=1)
    p.add_argument("--block", type=int, default=0, help="threads per block of the traversal kernels (0 = tuned)")
    p.add_argument("--capacity", type=int, default=0, help="wavefront paths per chunk (0 = automatic)")
    p.add_argument("--regcap", type=int, default=-1, help="1/0: force the 64-register traversal kernels (-1: tuned)")
    p.add_argument("--postpone", type=int, default=-1, help="traversal stack budget for postponed triangle groups")
    p.add_argument("--refill", type=int, default=-1, help="idle lanes that make a warp fetch new rays")
    p.add_argument("--collapse", type=int, default=0, help="BVH collapse: 0 SAH-optimal, 1 greedy")
    p.add_argument("--tri-cost", type=float, default=0.0, help="SAH-optimal collapse: triangle / node test cost")
    p.add_argument("--bins", type=int, default=0, help="binned SAH bins (0 = 32)")
    p.add_argument("--max-leaf", type=int, default=0, help="largest leaf (triangles, 1..2; 0 = 2)")
    p.add_argument("--workload", default="plain", choices=["plain", "batch", "serve", "cache", "instanced"],
                   help="plain: the single-frame pass (the bench line); batch: 256 uneven views in one wavefront "
                        "against a loop of plain renders")
    p.add_argument("--views", type=int, default=256)
    p.add_argument("--rates", default="10,50,100,200,500,1000,2000", help="serve: Poisson arrival rates (req/s)")
    p.add_argument("--serve-seconds", type=float, default=6.0, help="serve: arrival window per rate")
    p.add_argument("--max-requests", type=int, default=600, help="serve: cap on requests per rate")
    p.add_argument("--serve-chunk", type=int, default=1 << 21, help="serve: paths per chunk")
    p.add_argument("--serve-lanes", type=int, default=4, help="serve: lanes (streams)")
    p.add_argument("--ref-spp", type=int, default=4096, help="cache: spp of the plain reference render")
    p.add_argument("--train-frames", type=int, default=120, help="cache: online training frames before timing")
    p.add_argument("--cache-spps", default="1,2,4,8,16,32,64", help="cache: samples per pixel of the compared frames")
    p.add_argument("--cache-seeds", type=int, default=8, help="cache: frames (seeds) averaged per spp point")
    p.add_argument("--no-extras", action="store_true",
                   help="plain workload: leave out the BVH builder comparison and the batch / serve / cache "
                        "summaries of the bench line")
    p.add_argument("--ema", type=float, default=-1.0, help="cache: weight moving-average decay (-1: library default)")
    p.add_argument("--cache-lr", type=float, default=-1.0, help="cache: Adam learning rate (-1: library default)")
    p.add_argument("--train-paths", type=int, default=0, help="cache: training paths per frame (0: library default)")
    p.add_argument("--train-segments", type=int, default=0, help="cache: segments of a training path (0: default)")
    p.add_argument("--tune-cache", default=None, help="autotuner cache file (batch workload)")
    p.add_argument("--cpu-seconds", type=float, default=12.0, help="CPU baseline sample budget")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--jitter", action="store_true", help="jitter the camera ray inside the pixel per sample")
    p.add_argument("--deterministic", action="store_true",
                   help="plain pass: bit-reproducible fixed-point accumulation (BSM_PT_DETERMINISTIC)")
    return p.parse_args()


def workload_config(a, tris=None):
    return {"workload": f"terrain fBm {a.grid}x{a.grid} + {a.spheres} UV spheres, {a.width}x{a.height}, "
                        f"{a.spp} spp, {a.segments} segments",
            "scene_triangles": tris, "width": a.width, "height": a.height, "spp": a.spp,
            "max_segments": a.segments, "sky": "1024x512 RGBA16F equirect + alias table", "seed": a.seed,
            "camera": "jittered inside the pixel per sample" if a.jitter else "pixel-centre rays (as the reference)",
            **({"accumulation": "32.32 fixed point (BSM_PT_DETERMINISTIC)"} if a.deterministic else {}),
            "parallelism": "replicas" if a.gpus > 1 else "single GPU",
            "l2": "inputs larger than L2 (the wavefront queues hold up to 2^27 paths, 312 B each: 41 GB for "
                  "the 1920x1080x64 frame) and a 512 MB device copy between timed steps flushes L2"}


# ----------------------------------------------------------- distributed ----
class Dist:
    def __init__(self):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        self.pg = None
        if self.world > 1:
            import torch.distributed as dist
            os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
            dist.init_process_group("gloo")
            self.pg = dist

    def barrier(self):
        if self.pg:
            self.pg.barrier()

    def max(self, x: float) -> float:
        if not self.pg:
            return x
        import torch
        t = torch.tensor([x], dtype=torch.float64)
        self.pg.all_reduce(t, op=self.pg.ReduceOp.MAX)
        return float(t.item())

    def sum(self, x: float) -> float:
        if not self.pg:
            return x
        import torch
        t = torch.tensor([x], dtype=torch.float64)
        self.pg.all_reduce(t, op=self.pg.ReduceOp.SUM)
        return float(t.item())

    def close(self):
        if self.pg:
            self.pg.destroy_process_group()


# ---------------------------------------------------------------- clocks ----
class Clocks:
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(index), f"--query-gpu={self.Q}",
                                       "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                                      stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None

    def stop(self):
        if self.p:
            self.p.terminate()
            try:
                self.p.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.p.kill()
        self.f.flush()
        self.f.seek(0)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.f.read().splitlines():
            c = [x.strip() for x in line.split(",")]
            if len(c) < 9:
                continue
            try:
                sm.append(float(c[1]))
                mx.append(float(c[2]))
            except ValueError:
                continue
            for n, v in zip(names, c[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        os.unlink(self.f.name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            j = json.load(f)
        return float(j["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def profile_traffic():
    """The extend kernel's DRAM bytes per ray (primary and bounce launches), issue-slot use and L2 traffic from
    the last ncu capture committed under profiles/ (a file, not a measurement of this run), or None."""
    path = os.path.join(ROOT, "profiles", "k_extend_traffic.json")
    try:
        with open(path) as f:
            return json.load(f)
    except (OSError, ValueError):
        return None


# -------------------------------------------------------------- CPU legs ----
def cpu_sample(scene, cam_arr, a, budget_s: float, threads: int = 0):
    """Times the oracle on whole rows of the frame, sized to about budget_s seconds: a band of rows at 1 spp,
    or the whole frame at as many samples per pixel (up to the workload's) as the budget holds."""
    import oracle
    osc = oracle.OracleScene(scene)
    h = a.height
    mid = h // 2
    probe = (mid - 4, mid + 4)
    _, st, sec = osc.render(cam_arr, spp=1, max_segments=a.segments, seed=a.seed, rows=probe, threads=threads)
    per_row = max(sec / 8.0, 1e-4)
    rows = int(min(h, max(8, budget_s / per_row)))
    spp = int(max(1, min(a.spp, budget_s / (per_row * h)))) if rows == h else 1
    r0 = max(0, mid - rows // 2)
    r1 = min(h, r0 + rows)
    _, st, sec = osc.render(cam_arr, spp=spp, max_segments=a.segments, seed=a.seed, rows=(r0, r1), threads=threads)
    rays = int(st[:16].sum())
    return {"rays": rays, "seconds": sec, "rows": (r0, r1), "spp": spp, "shadow_rays": int(st[16:].sum())}


def nthreads():
    return os.cpu_count() or 1


# ------------------------------------------------------------ reference ----
def run_reference(a, dist: Dist):
    if dist.rank != 0:
        return 0
    bsm = importlib.import_module("bisemutum-engine_gb300")
    scene = bsm.generate_scene(bsm.BSM_SCENE_TERRAIN, seed=a.seed, grid=a.grid, spheres=a.spheres, width=a.width,
                               height=a.height)
    cam = scene.camera.as_array()
    budget = max(1.0, min(a.cpu_seconds, 20.0))
    for _ in range(a.warmup):
        cpu_sample(scene, cam, a, budget / 4)
    rays, secs, rows = 0, 0.0, None
    for _ in range(a.steps):
        r = cpu_sample(scene, cam, a, budget)
        rays += r["rays"]
        secs += r["seconds"]
        rows, spp = r["rows"], r["spp"]
    value = rays / secs / 1e6
    cores = nthreads()
    sample = f"rows {rows[0]}-{rows[1]} of the {a.width}x{a.height} frame at {spp} spp per step, {a.segments} segments"
    line = {"impl": "reference", "metric": METRIC, "value": round(value, 3), "unit": "Mrays/s", "n_gpus": a.gpus,
            "steps": a.steps, "warmup": a.warmup, "ms_per_step": round(secs / a.steps * 1e3, 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": workload_config(a, scene.num_triangles),
            "cpu_baseline": {"value": round(value, 3), "unit": "Mrays/s", "cores": cores, "kind": "port",
                             "sample": sample},
            "e2e": {"value": round(value, 3), "unit": "Mrays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "note": "CPU implementation of the pass (multithreaded C++ oracle, -O3, no -march=native, no fast-math); the reference's "
                    "own pass needs a graphics ray-tracing pipeline, unavailable on this box"}
    print(json.dumps(line), flush=True)
    return 0


# ------------------------------------------------------------------ ours ----
def run_ours(a, dist: Dist):
    bsm = importlib.import_module("bisemutum-engine_gb300")
    scene = bsm.generate_scene(bsm.BSM_SCENE_TERRAIN, seed=a.seed, grid=a.grid, spheres=a.spheres, width=a.width,
                               height=a.height)
    ctx = bsm.Context(dist.local)
    t0 = time.perf_counter()
    sid = ctx.upload(scene)
    bvh = ctx.build_bvh(sid, sah_bins=a.bins, max_leaf=a.max_leaf, collapse=a.collapse, tri_cost=a.tri_cost)
    setup_s = time.perf_counter() - t0
    if a.regcap >= 0 or a.postpone >= 0 or a.refill >= 0:
        ctx.set_tuning(sid, bsm.TuneParams(a.block or 128, a.capacity, a.postpone if a.postpone >= 0 else 16,
                                           a.refill if a.refill >= 0 else 8, a.regcap if a.regcap >= 0 else 1))
    cam = scene.camera
    seed = a.seed + 1000 * dist.rank
    jitter = bsm.BSM_PT_JITTER if a.jitter else 0
    if a.deterministic:
        jitter |= bsm.BSM_PT_DETERMINISTIC
    flags_timed = bsm.BSM_PT_STAGE_TIMING | jitter
    s_timed = bsm.settings(spp=a.spp, max_segments=a.segments, seed=seed, flags=flags_timed, block_size=a.block,
                           wavefront_capacity=a.capacity)

    # traversal working set of this workload (counting variant, untimed)
    _, cst = ctx.render(sid, [cam], bsm.settings(spp=max(1, a.spp // 16), max_segments=a.segments, seed=seed,
                                                 flags=bsm.BSM_PT_COUNT_TRAVERSAL | jitter), outputs=False)
    nodes_per_ray = cst.traversal_nodes / max(1, cst.extend_rays)
    tris_per_ray = cst.traversal_tris / max(1, cst.extend_rays)

    # L2 flush buffer (512 MB device copy between timed steps)
    L = bsm.lib()
    import ctypes as C
    flush = C.c_void_p()
    ctx.check(L.bsm_device_alloc(ctx.h, 2 << 28, C.byref(flush)))

    def flush_l2():
        ctx.check(L.bsm_memcpy(ctx.h, C.c_void_p(flush.value + (1 << 28)), flush, 1 << 28, 2))

    for _ in range(a.warmup):
        ctx.render(sid, [cam], s_timed, outputs=False)
    ctx.sync()

    clocks = Clocks(dist.local) if dist.rank == 0 else None
    dist.barrier()
    ctx.sync()
    wall0 = time.perf_counter()
    ms_dev, ms_ext, ms_shade, ms_shadow, ms_cam, rays, shadow_rays, launches = [], 0.0, 0.0, 0.0, 0.0, 0, 0, 0
    for _ in range(a.steps):
        flush_l2()
        _, st = ctx.render(sid, [cam], s_timed, outputs=False)
        ms_dev.append(st.ms_total)
        ms_ext += st.ms_extend
        ms_shade += st.ms_shade
        ms_shadow += st.ms_shadow
        ms_cam += st.ms_camera
        rays += st.extend_rays
        shadow_rays += st.shadow_rays
        launches += st.chunks * (1 + 3 * a.segments)
        ext_launches = st.extend_launches
        seg_rays = [int(st.rays_per_segment[k]) for k in range(a.segments)]
    ctx.sync()
    dist.barrier()
    wall = time.perf_counter() - wall0
    clk = clocks.stop() if clocks else None

    dev_s = sum(ms_dev) / 1e3
    dev_s_max = dist.max(dev_s)
    rays_all = dist.sum(float(rays))
    value = rays_all / dev_s_max / 1e6
    ms_per_step = dev_s_max / a.steps * 1e3

    # e2e: public API with host buffers (pinned output, camera uploaded each step)
    out_px = a.width * a.height
    host = C.c_void_p()
    ctx.check(L.bsm_host_alloc(ctx.h, out_px * 16, C.byref(host)))
    outs = (bsm.ViewOutput * 1)()
    outs[0].rgba = host.value
    outs[0].row_pitch_px = 0
    outs[0].location = bsm.BSM_HOST
    cams = (bsm.Camera * 1)(cam)
    s_e2e = bsm.settings(spp=a.spp, max_segments=a.segments, seed=seed, block_size=a.block,
                         wavefront_capacity=a.capacity, flags=jitter)
    ctx.check(L.bsm_render(ctx.h, sid, cams, 1, C.byref(s_e2e), outs, None))
    dist.barrier()
    e0 = time.perf_counter()
    e2e_steps = max(1, min(a.steps, 3))
    for _ in range(e2e_steps):
        ctx.check(L.bsm_render(ctx.h, sid, cams, 1, C.byref(s_e2e), outs, None))  # returns after the D2H copy
    e2e_s = dist.max(time.perf_counter() - e0)
    e2e_val = rays_all / a.steps * e2e_steps / e2e_s / 1e6
    L.bsm_host_free(ctx.h, host)
    # the same frame with bit-reproducible fixed-point accumulation (BSM_PT_DETERMINISTIC), device time
    det = None
    if not a.no_extras and not a.deterministic:
        s_det = bsm.settings(spp=a.spp, max_segments=a.segments, seed=seed,
                             flags=flags_timed | bsm.BSM_PT_DETERMINISTIC, block_size=a.block,
                             wavefront_capacity=a.capacity)
        ctx.render(sid, [cam], s_det, outputs=False)
        det_ms, det_rays, det_steps = 0.0, 0, 3
        for _ in range(det_steps):
            flush_l2()
            _, dst = ctx.render(sid, [cam], s_det, outputs=False)
            det_ms += dst.ms_total
            det_rays += dst.extend_rays
        det = {"mrays_per_s": round(det_rays / (det_ms / 1e3) / 1e6, 2), "ms_per_step": round(det_ms / det_steps, 3),
               "steps": det_steps,
               "what": "BSM_PT_DETERMINISTIC: exact 32.32 fixed-point per-pixel sums; images bit-identical from run "
                       "to run and to the CPU oracle's fixed-point mode"}
    L.bsm_device_free(ctx.h, flush)
    bvh_cmp = None
    if dist.rank == 0 and not a.no_extras:
        bvh_cmp = bvh_comparison(bsm, ctx, scene, a, bvh, st_dev_frame=(rays, sum(ms_dev)))

    line = None
    if dist.rank == 0:
        peak, peak_kind = peaks()
        per_launch_rays = rays / max(1, a.steps * ext_launches)
        per_launch_ms = ms_ext / max(1, a.steps * ext_launches)
        achieved = EXTEND_BYTES_PER_RAY * rays / (ms_ext / 1e3) / 1e9 if ms_ext > 0 else None
        prof = profile_traffic()
        traffic = None
        if prof:
            # per launch: segment 0's rays at the primary launch's bytes per ray, the others at the bounce figure
            b0, b1 = prof["dram_bytes_per_ray_primary"], prof["dram_bytes_per_ray_bounce"]
            traffic = round((b0 * seg_rays[0] + b1 * sum(seg_rays[1:])) / max(1, ext_launches))
        roofline = {"bound": "hbm", "kernel": "k_extend", "achieved": round(achieved, 2) if achieved else None,
                    "peak": peak, "unit": "GB/s", "frac": round(achieved / peak, 5) if achieved else None,
                    "peak_kind": peak_kind + " (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured" else peak_kind,
                    "traffic": traffic,
                    "traffic_source": (f"last ncu capture (commit {prof['captured_at_commit']}, {prof['capture']}): "
                                       f"{prof['dram_bytes_per_ray_primary']} B/ray on primary and "
                                       f"{prof['dram_bytes_per_ray_bounce']} B/ray on bounce launches, weighted by "
                                       f"this frame's rays per segment") if prof else None,
                    "algorithmic_bytes_per_launch": round(EXTEND_BYTES_PER_RAY * per_launch_rays),
                    "avg_launch_ms": round(per_launch_ms, 4),
                    "l2_traversal_gbs": round((NODE_BYTES * nodes_per_ray + TRI_BYTES * tris_per_ray) * rays /
                                              (ms_ext / 1e3) / 1e9, 1) if ms_ext > 0 else None,
                    "nodes_per_ray": round(nodes_per_ray, 2), "tris_per_ray": round(tris_per_ray, 2),
                    "extend_mrays_per_s_kernel_only": round(rays / (ms_ext / 1e3) / 1e6, 1) if ms_ext > 0 else None,
                    "from_last_ncu_capture": ({"commit": prof["captured_at_commit"], "l2": prof["l2"],
                                               "issue": prof["issue"]} if prof else None)}
        cpu = None
        if not a.no_cpu_baseline:
            r = cpu_sample(scene, cam.as_array(), a, a.cpu_seconds)
            cpu = {"value": round(r["rays"] / r["seconds"] / 1e6, 3), "unit": "Mrays/s", "cores": nthreads(),
                   "kind": "port",
                   "sample": f"rows {r['rows'][0]}-{r['rows'][1]} of the frame at {r['spp']} spp ({r['rays']} extend rays, "
                             f"{r['seconds']:.1f} s)"}
        line = {"metric": METRIC, "value": round(value, 2), "unit": "Mrays/s", "n_gpus": a.gpus, "steps": a.steps,
                "warmup": a.warmup, "ms_per_step": round(ms_per_step, 3), "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded procedural scene)",
                "config": workload_config(a, scene.num_triangles),
                "frames_per_s": round(1e3 / ms_per_step * a.gpus, 4),
                "e2e": {"value": round(e2e_val, 2), "unit": "Mrays/s",
                        "h2d_bytes_per_step": DEV_VIEW_BYTES, "d2h_bytes_per_step": out_px * 16,
                        "api": "bsm_render with a host camera and a pinned host RGBA32F output"},
                "gpu_launches": launches,
                "roofline": roofline, "cpu_baseline": cpu, "clocks": clk,
                "stages_ms_per_step": {"camera": round(ms_cam / a.steps, 3), "extend": round(ms_ext / a.steps, 3),
                                       "shade": round(ms_shade / a.steps, 3),
                                       "shadow": round(ms_shadow / a.steps, 3)},
                "rays_per_step": {"extend": rays // a.steps, "shadow": shadow_rays // a.steps,
                                  "extend_per_segment": seg_rays},
                "shadow_mrays_per_s": round(shadow_rays / (ms_shadow / 1e3) / 1e6, 1) if ms_shadow > 0 else None,
                "bvh": {"collapse": "sah-optimal" if a.collapse == 0 else "greedy",
                        "builder": "device" if bvh.builder == bsm.BSM_BUILD_DEVICE else "host",
                        "build_ms": round(bvh.build_ms, 2), "nodes": bvh.num_nodes,
                        "depth": bvh.max_depth, "bytes": bvh.node_bytes + bvh.tri_bytes,
                        "upload_and_build_s": round(setup_s, 3), **(bvh_cmp or {})},
                "wall_s_timed": round(wall, 3),
                **({"deterministic": det} if det else {})}
    ctx.close()
    if line is not None and not a.no_extras:
        # the benchmark spec's other forms, each on its own context after the timed region: 64 uneven views batched
        # against one render per view, a Poisson request stream at 50 req/s for 10 s, and the radiance cache
        # against the plain pass at equal relMSE
        t_ex = time.perf_counter()
        line["batch"] = batch_summary(a, bsm, dist.local, 64, 2, compare=8)
        line["serve"] = serve_summary(a, bsm, dist.local, [50.0], 10.0, 600, 120)
        line["cache"] = cache_summary(a, bsm, dist.local, [2, 4, 8, 16, 32], 4, 1024, 120)
        line["extras_s"] = round(time.perf_counter() - t_ex, 1)
    if line is not None:
        print(json.dumps(line), flush=True)
    return 0


def bvh_comparison(bsm, ctx, scene, a, bvh, st_dev_frame):
    """Device against host BVH build (untimed region): build times for this scene and for the 4,973,058-triangle
    serving scene, and the plain frame's Mrays/s traversing the host-built tree against the device-built one the
    timed steps used (same frame, same paths)."""
    out = {}
    t0 = time.perf_counter()
    sid_h = ctx.upload(scene)
    hst = ctx.build_bvh(sid_h, sah_bins=a.bins, max_leaf=a.max_leaf, collapse=a.collapse, tri_cost=a.tri_cost,
                        builder=bsm.BSM_BUILD_HOST)
    out["host_build_ms"] = round(hst.build_ms, 1)
    out["host_tree"] = {"nodes": hst.num_nodes, "depth": hst.max_depth, "sah_cost": round(hst.sah_cost, 3)}
    out["device_tree"] = {"nodes": bvh.num_nodes, "depth": bvh.max_depth, "sah_cost": round(bvh.sah_cost, 3)}
    jitter = bsm.BSM_PT_JITTER if a.jitter else 0
    s = bsm.settings(spp=a.spp, max_segments=a.segments, seed=a.seed, flags=jitter, block_size=a.block,
                     wavefront_capacity=a.capacity)
    ctx.render(sid_h, [scene.camera], s, outputs=False)
    _, st = ctx.render(sid_h, [scene.camera], s, outputs=False)
    rays, ms = st_dev_frame
    out["mrays_per_s_device_tree"] = round(rays / (ms / 1e3) / 1e6, 1)
    out["mrays_per_s_host_tree"] = round(st.extend_rays / (st.ms_total / 1e3) / 1e6, 1)
    ctx.release(sid_h)
    big = bsm.generate_scene(bsm.BSM_SCENE_TERRAIN, seed=a.seed, grid=1024, spheres=6000)
    sid_b = ctx.upload(big)
    dst = ctx.build_bvh(sid_b)
    out["device_build_ms_4.97M"] = round(dst.build_ms, 1)
    hb = ctx.build_bvh(sid_b, builder=bsm.BSM_BUILD_HOST)
    out["host_build_ms_4.97M"] = round(hb.build_ms, 1)
    out["triangles_4.97M"] = big.num_triangles
    ctx.release(sid_b)
    out["comparison_s"] = round(time.perf_counter() - t0, 1)
    return out


# ----------------------------------------------------------------- batch ----
def batch_views(bsm, a, n=None):
    """Uneven views of the terrain: side log-uniform in [64, 1024], spp in {4, 8, 16, 32, 64}."""
    rng = np.random.default_rng(a.seed + 77)
    views = []
    for i in range(a.views if n is None else n):
        side = int(round(float(np.exp(rng.uniform(np.log(64), np.log(1024))))))
        spp = int(rng.choice([4, 8, 16, 32, 64]))
        pos = (rng.uniform(0.15, 0.85), rng.uniform(0.35, 0.6), rng.uniform(-0.15, 0.35))
        tgt = (rng.uniform(0.25, 0.75), 0.0, rng.uniform(0.45, 0.85))
        cam = bsm.make_camera(pos, tuple(np.subtract(tgt, pos)), yfov_deg=60.0, width=side, height=side)
        views.append((cam, spp, a.segments, a.seed + i))
    return views


def batch_summary(a, bsm, device, n_views, steps, compare=16):
    """Uneven views rendered by one bsm_render_batch call (one wavefront, one graph; launch parameters from the
    autotuner) against one bsm_render call per view (same paths, so equal relMSE: checked pixel by pixel on
    `compare` views).  Device time (events) for both forms."""
    scene = bsm.generate_scene(bsm.BSM_SCENE_TERRAIN, seed=a.seed, grid=a.grid, spheres=a.spheres)
    ctx = bsm.Context(device)
    try:
        sid = ctx.load_scene(scene)
        views = batch_views(bsm, a, n_views)
        s = bsm.settings(max_segments=a.segments, spp=1)
        t0 = time.perf_counter()
        tune = ctx.autotune(sid, views, s, a.tune_cache)
        tune_s = time.perf_counter() - t0
        ctx.render_batch(sid, views, s, outputs=False)
        b_ms, b_rays = [], 0
        for _ in range(steps):
            _, st = ctx.render_batch(sid, views, s, outputs=False)
            b_ms.append(st.ms_total)
            b_rays += st.extend_rays
        for cam, spp, segs, seed in views[:4]:
            ctx.render(sid, [cam], bsm.settings(spp=spp, max_segments=segs, seed=seed), outputs=False)
        p_steps = max(1, steps // 2)
        p_ms, p_wall, p_rays = 0.0, 0.0, 0
        for _ in range(p_steps):
            ctx.sync()
            w0 = time.perf_counter()
            for cam, spp, segs, seed in views:
                _, st = ctx.render(sid, [cam], bsm.settings(spp=spp, max_segments=segs, seed=seed), outputs=False)
                p_ms += st.ms_total
                p_rays += st.extend_rays
            ctx.sync()
            p_wall += time.perf_counter() - w0
        sample = views[:compare]
        imgs, _ = ctx.render_batch(sid, sample, s)
        worst = 0.0
        for (cam, spp, segs, seed), img in zip(sample, imgs):
            alone, _ = ctx.render(sid, [cam], bsm.settings(spp=spp, max_segments=segs, seed=seed))
            g, c = img[..., :3].astype(np.float64), alone[0][..., :3].astype(np.float64)
            worst = max(worst, float((np.abs(g - c) / np.maximum(np.abs(c), 1e-3)).max()))
    finally:
        ctx.close()
    b_s = min(b_ms) / 1e3
    p_s = p_ms / p_steps / 1e3
    px = sum(v[0].width * v[0].height for v in views)
    paths = sum(v[0].width * v[0].height * v[1] for v in views)
    return {"metric": "views/s at equal relMSE, batched vs one render per view",
            "workload": f"{len(views)} views of the terrain, side log-uniform 64..1024, spp in {{4,8,16,32,64}}, "
                        f"{a.segments} segments",
            "views": len(views), "pixels": px, "paths": paths,
            "batched_views_per_s": round(len(views) / b_s, 2), "plain_views_per_s": round(len(views) / p_s, 2),
            "plain_views_per_s_wall": round(len(views) * p_steps / p_wall, 2),
            "speedup": round(p_s / b_s, 3),
            "batched_mrays_per_s": round(b_rays / steps / b_s / 1e6, 1),
            "plain_mrays_per_s": round(p_rays / p_steps / p_s / 1e6, 1),
            "batch_ms": round(b_s * 1e3, 2), "plain_ms_device": round(p_s * 1e3, 2),
            "equal_relmse_check": {"views_compared": len(sample), "max_rel_diff": worst},
            "tune": {"block_size": tune.best.block_size, "wavefront_capacity": tune.best.wavefront_capacity,
                     "postpone_depth": tune.best.postpone_depth, "refill_lanes": tune.best.refill_lanes,
                     "register_cap": tune.best.register_cap,
                     "best_ms": round(tune.best_ms, 3), "default_ms": round(tune.default_ms, 3),
                     "worst_ms": round(tune.worst_ms, 3),
                     "tried": tune.tried, "from_cache": tune.from_cache, "seconds": round(tune_s, 2)}}


def run_batch(a, dist):
    if dist.rank == 0:
        bsm = importlib.import_module("bisemutum-engine_gb300")
        line = {"workload": "batch", **batch_summary(a, bsm, dist.local, a.views, a.steps),
                "config": workload_config(a)}
        print(json.dumps(line), flush=True)
    return 0


# ----------------------------------------------------------------- serve ----
SERVE_MIX = "scene uniform, resolution log-uniform 128x128..1920x1080, spp {1,4,16,32}, bounces {2,4,8}"


def serve_summary(a, bsm, device, rates, seconds, max_requests, saturation_n):
    """Poisson request stream over four resident scenes (20,504 / 250,050 / 1,482,242 / 4,973,058 triangles);
    per request: scene uniform, resolution log-uniform 128x128..1920x1080, spp in {1,4,16,32}, bounces in
    {2,4,8}.  p50/p99 latency (submit -> result in host memory) and rays/s per arrival rate, then the
    efficiency at saturation against batched renders of the same views."""
    ctx = bsm.Context(device)
    try:
        specs = [(bsm.BSM_SCENE_ROOM, 0, 64), (bsm.BSM_SCENE_TERRAIN, 256, 250), (bsm.BSM_SCENE_TERRAIN, 512, 2000),
                 (bsm.BSM_SCENE_TERRAIN, 1024, 6000)]
        scenes, ids, tris = [], [], []
        t0 = time.perf_counter()
        for kind, grid, sph in specs:
            sc = bsm.generate_scene(kind, seed=a.seed, grid=grid, spheres=sph)
            scenes.append(sc)
            ids.append(ctx.load_scene(sc))
            tris.append(sc.num_triangles)
        setup_s = time.perf_counter() - t0
        rng = np.random.default_rng(a.seed + 5)
        results = []
        for lam in rates:
            n = int(min(max_requests, max(20, lam * seconds)))
            ctx.server_start(pool_bytes=16 << 30, chunk_paths=a.serve_chunk, lanes=a.serve_lanes)
            arrivals = np.cumsum(rng.exponential(1.0 / lam, n))
            reqs = []
            for i in range(n):
                k = int(rng.integers(0, 4))
                u = float(rng.uniform())
                w = int(round(128 * (1920 / 128) ** u))
                h = int(round(128 * (1080 / 128) ** u))
                base = scenes[k].camera
                cam = bsm.make_camera(tuple(base.position), tuple(base.front), width=w, height=h)
                reqs.append((ids[k], cam, int(rng.choice([1, 4, 16, 32])), int(rng.choice([2, 4, 8])), int(i + 1)))
            start = time.perf_counter()
            rids = []
            for (sid, cam, spp, segs, seed), t_arr in zip(reqs, arrivals):
                delay = start + t_arr - time.perf_counter()
                if delay > 0:
                    time.sleep(delay)
                rids.append(ctx.submit(sid, cam, spp, segs, seed)[0])
            lat = []
            for rid in rids:
                st = ctx.wait(rid, timeout_ms=600000)
                lat.append(st.done_ms - st.submit_ms)
            wall = time.perf_counter() - start
            ss = ctx.server_stats()
            ctx.server_stop()
            lat = np.array(lat)
            results.append({"rate_req_s": lam, "requests": n, "p50_ms": round(float(np.percentile(lat, 50)), 2),
                            "p90_ms": round(float(np.percentile(lat, 90)), 2),
                            "p99_ms": round(float(np.percentile(lat, 99)), 2),
                            "mean_ms": round(float(lat.mean()), 2), "completed_req_s": round(n / wall, 2),
                            "mrays_per_s": round(ss.extend_rays / wall / 1e6, 1), "wall_s": round(wall, 2)})
        saturated = serve_saturated(a, bsm, ctx, ids, scenes, rng, n=saturation_n) if saturation_n else None
    finally:
        ctx.close()
    return {"metric": "p50/p99 request latency and rays/s per Poisson arrival rate",
            "scenes_triangles": tris, "setup_s": round(setup_s, 1), "results": results, "saturated": saturated,
            "request_mix": SERVE_MIX,
            "server": {"pool_bytes": 16 << 30, "chunk_paths": a.serve_chunk, "lanes": a.serve_lanes}}


def run_serve(a, dist):
    if dist.rank == 0:
        bsm = importlib.import_module("bisemutum-engine_gb300")
        rates = [float(x) for x in a.rates.split(",")]
        line = {"workload": "serve", **serve_summary(a, bsm, dist.local, rates, a.serve_seconds, a.max_requests, 240)}
        print(json.dumps(line), flush=True)
    return 0


def serve_saturated(a, bsm, ctx, ids, scenes, rng, n=240):
    """Serving efficiency at saturation: n requests of the same mix submitted at once, against the same
    views rendered by one bsm_render_batch call per scene (same spp, bounces and seeds, so the same paths);
    both include the copy of every result to host memory."""
    reqs = []
    for i in range(n):
        k = int(rng.integers(0, 4))
        u = float(rng.uniform())
        w = int(round(128 * (1920 / 128) ** u))
        h = int(round(128 * (1080 / 128) ** u))
        base = scenes[k].camera
        cam = bsm.make_camera(tuple(base.position), tuple(base.front), width=w, height=h)
        reqs.append((k, cam, int(rng.choice([1, 4, 16, 32])), int(rng.choice([2, 4, 8])), int(i + 1)))
    ctx.server_start(pool_bytes=16 << 30, chunk_paths=a.serve_chunk, lanes=a.serve_lanes)
    ctx.sync()
    t0 = time.perf_counter()
    rids = [ctx.submit(ids[k], cam, spp, segs, seed)[0] for k, cam, spp, segs, seed in reqs]
    for rid in rids:
        ctx.wait(rid, timeout_ms=600000)
    serve_s = time.perf_counter() - t0
    rays = ctx.server_stats().extend_rays
    ctx.server_stop()
    s = bsm.settings(spp=1, max_segments=8)
    groups = [[(cam, spp, segs, seed) for k2, cam, spp, segs, seed in reqs if k2 == k] for k in range(4)]
    for k in range(4):  # warm-up: graphs and buffers of each scene
        if groups[k]:
            ctx.render_batch(ids[k], groups[k][:2], s, outputs=False)
    ctx.sync()
    t0 = time.perf_counter()
    brays = 0
    for k in range(4):
        if groups[k]:
            _, st = ctx.render_batch(ids[k], groups[k], s)
            brays += st.extend_rays
    batch_s = time.perf_counter() - t0
    return {"requests": n, "serve_s": round(serve_s, 3), "serve_mrays_per_s": round(rays / serve_s / 1e6, 1),
            "batch_s": round(batch_s, 3), "batch_mrays_per_s": round(brays / batch_s / 1e6, 1),
            "same_rays": bool(rays == brays), "efficiency": round(batch_s / serve_s, 3)}


# ------------------------------------------------------------- instanced ----
def run_instanced(a, dist):
    """Two-level scene (the reference's TLAS of drawables): a 512x512 ground grid and 4,000 instances of a UV
    sphere, a box and a tetrahedron, rendered through the TLAS + BLAS traversal and, for comparison, as the same
    triangles flattened into one world-space BVH; 1920x1080, 16 spp, 8 segments."""
    bsm = importlib.import_module("bisemutum-engine_gb300")
    ctx = bsm.Context(dist.local)
    inst = bsm.generate_instanced_scene(seed=a.seed, instances=4000, ground=512, width=a.width, height=a.height)
    flat = inst.flattened()
    spp = 16
    out = {}
    for name, sid in (("two_level", ctx.load_instanced(inst)), ("flat", ctx.load_scene(flat))):
        s = bsm.settings(spp=spp, max_segments=a.segments, seed=a.seed, flags=bsm.BSM_PT_STAGE_TIMING)
        for _ in range(a.warmup):
            ctx.render(sid, [inst.camera], s, outputs=False)
        ms, rays, stages = 0.0, 0, None
        for _ in range(a.steps):
            _, st = ctx.render(sid, [inst.camera], s, outputs=False)
            ms += st.ms_total
            rays += st.extend_rays
            stages = {"extend": round(st.ms_extend, 3), "shadow": round(st.ms_shadow, 3),
                      "shade": round(st.ms_shade, 3)}
        out[name] = {"mrays_per_s": round(rays / ms / 1e3, 1), "ms_per_frame": round(ms / a.steps, 2),
                     "stages_ms": stages}
        ctx.release(sid)
    ctx.close()
    line = {"workload": "instanced", "metric": "Mrays/s, two-level scene vs the same triangles flattened",
            "triangles": int(flat.num_triangles), "instances": int(len(inst.inst_geometry)),
            "two_level": out["two_level"], "flat": out["flat"],
            "ratio": round(out["two_level"]["mrays_per_s"] / out["flat"]["mrays_per_s"], 3),
            "config": {"workload": f"instanced ground + 4000 objects, {a.width}x{a.height}, {spp} spp, "
                                   f"{a.segments} segments", "seed": a.seed}}
    if dist.rank == 0:
        print(json.dumps(line), flush=True)
    return 0


# ----------------------------------------------------------------- cache ----
def equal_error_time(curve, key, target):
    """Frame time a method needs for `target` error, from its measured points (dicts with "ms" and `key`):
    log-log interpolation along the error envelope (points in order of frame time, each kept only if its error
    is below every cheaper point's), so that a noisy point whose error is above a cheaper one's cannot make an
    error look reachable sooner than measured.  None when the target lies outside the envelope's range."""
    env = []
    for c in sorted(curve, key=lambda c: c["ms"]):
        if not env or c[key] < env[-1][0]:
            env.append((c[key], c["ms"]))
    for (e0, t0_), (e1, t1) in zip(env[:-1], env[1:]):
        if e1 <= target <= e0:
            u = (np.log(target) - np.log(e0)) / (np.log(e1) - np.log(e0))
            return float(np.exp(np.log(t0_) + u * (np.log(t1) - np.log(t0_))))
    return None


def cache_summary(a, bsm, device, spps, seeds, ref_spp, train_frames):
    """Radiance cache on the terrain scene: relMSE against a high-spp plain render and DEVICE time per frame
    (CUDA events; the cached frame's training step included), for the plain pass (8 segments) and the cached
    pass (paths end in the cache at their third vertex; 32,768 training paths and 4 Adam steps of 16,384
    vertices per frame), then frames/s of each at equal relMSE, untrimmed and with the largest 0.1 % of per-value
    errors dropped.  Both passes use the same seeds (common random numbers): their paths agree up to the cache
    vertex, so rare fireflies of the shared prefix (sun glints on near-mirror spheres) fall on both sides."""
    scene = bsm.generate_scene(bsm.BSM_SCENE_TERRAIN, seed=a.seed, grid=a.grid, spheres=a.spheres, width=a.width,
                               height=a.height)
    ctx = bsm.Context(device)
    try:
        sid = ctx.load_scene(scene)
        cam = scene.camera
        per = min(256, ref_spp)
        ctx.render(sid, [cam], bsm.settings(spp=per, max_segments=a.segments, seed=90000, accumulate=0),
                   outputs=ref_spp <= per)
        imgs = None
        for k in range(1, ref_spp // per):
            last = k == ref_spp // per - 1
            imgs, _ = ctx.render(sid, [cam], bsm.settings(spp=per, max_segments=a.segments, seed=90000,
                                                          accumulate=1), outputs=last)
        ref = imgs[0] if imgs is not None else ctx.render(sid, [cam], bsm.settings(
            spp=per, max_segments=a.segments, seed=90000))[0][0]
        seed_of = [7 + 1000 * k for k in range(seeds)]

        def measure(render):
            rows = []
            for spp in spps:
                render(spp, seed_of[0])   # warm-up: graph capture for this size
                errs, terrs, ms = [], [], []
                for sd in seed_of:
                    img, st = render(spp, sd + spp)
                    errs.append(bsm.rel_mse(img, ref))
                    terrs.append(bsm.rel_mse(img, ref, trim=0.001))
                    ms.append(st.ms_total)
                rows.append({"spp": spp, "relmse": float(np.mean(errs)), "relmse_trimmed": float(np.mean(terrs)),
                             "relmse_median": float(np.median(errs)), "ms": float(np.mean(ms))})
            return rows

        def plain_render(spp, sd):
            img, st = ctx.render(sid, [cam], bsm.settings(spp=spp, max_segments=a.segments, seed=sd))
            return img[0], st

        plain = measure(plain_render)
        cache = bsm.RadianceCache(ctx, seed=a.seed)
        cs = bsm.cache_settings()
        if a.ema >= 0.0:
            cs.ema_decay = a.ema
        if a.cache_lr > 0.0:
            cs.lr = a.cache_lr
        if a.train_paths > 0:
            cs.train_paths = a.train_paths
        if a.train_segments > 0:
            cs.train_segments = a.train_segments
        t0 = time.perf_counter()
        losses = []
        for f in range(train_frames):
            _, _, loss = cache.render(sid, cam, bsm.settings(spp=1, seed=100000 + f), cs, outputs=False)
            losses.append(loss)
        train_s = time.perf_counter() - t0

        def cached_render(spp, sd):
            img, st, _ = cache.render(sid, cam, bsm.settings(spp=spp, seed=sd), cs)   # trains, then renders
            return img, st

        cached = measure(cached_render)
        cache.close()
    finally:
        ctx.close()

    equal = {}
    for key in ("relmse", "relmse_trimmed"):
        rows = []
        for c, k in zip(plain, cached):
            tc = equal_error_time(cached, key, c[key])
            # where the cached frame at the same spp is both at least as accurate and faster, it reaches the plain
            # frame's error in at most its own time: plain ms / cached ms bounds the equal-error speedup from below
            # (robust where single fireflies make the untrimmed error curve non-monotone in spp)
            lower = round(c["ms"] / k["ms"], 3) if k[key] <= c[key] else None
            rows.append({"plain_spp": c["spp"], "target": round(c[key], 6), "plain_fps": round(1e3 / c["ms"], 2),
                         "cached_fps": round(1e3 / tc, 2) if tc else None,
                         "speedup": round(c["ms"] / tc, 3) if tc else None,
                         "speedup_lower_bound_same_spp": lower})
        equal[key] = rows
    return {"metric": "frames/s at equal relMSE, cached vs plain pass (device time, training included)",
            "workload": f"radiance cache on the terrain scene, {a.width}x{a.height}, paths end in the cache after "
                        f"2 bounces",
            "reference_spp": ref_spp, "seeds_per_point": seeds, "seeds": "common random numbers (same per point)",
            "plain": plain, "cached": cached, "equal_relmse": equal,
            "train": {"frames": train_frames, "seconds": round(train_s, 2),
                      "loss_first10": round(float(np.mean(losses[:10])), 4),
                      "loss_last10": round(float(np.mean(losses[-10:])), 4),
                      "per_frame": f"{cs.train_paths} training paths, {cs.train_steps} Adam steps of {cs.train_batch} "
                                   f"vertices, lr {cs.lr:g}", "ema_decay": round(float(cs.ema_decay), 4)}}


def run_cache(a, dist):
    if dist.rank == 0:
        bsm = importlib.import_module("bisemutum-engine_gb300")
        spps = [int(x) for x in a.cache_spps.split(",")]
        line = {"workload": "cache", **cache_summary(a, bsm, dist.local, spps, a.cache_seeds, a.ref_spp,
                                                     a.train_frames), "config": workload_config(a)}
        print(json.dumps(line), flush=True)
    return 0


def main():
    a = parse()
    dist = Dist()
    if dist.world > 1:
        a.gpus = dist.world
    try:
        if a.impl == "reference":
            return run_reference(a, dist)
        if a.workload == "batch":
            return run_batch(a, dist)
        if a.workload == "serve":
            return run_serve(a, dist)
        if a.workload == "cache":
            return run_cache(a, dist)
        if a.workload == "instanced":
            return run_instanced(a, dist)
        return run_ours(a, dist)
    finally:
        dist.close()


if __name__ == "__main__":
    sys.exit(main())
