#!/usr/bin/env python
"""Throughput benchmark of the wavefront path tracer (one JSON line).

Workload (default): the procedural interior — an 8x4x6 room with a 1.5x1
window, 400 boxes and UV-spheres tessellated to 201,792 triangles (40 %
Lambert, 40 % GGX conductor, 20 % glass), a 2048x1024 HDR sky with a sun
lobe, 1280x720 pixels, maximum depth 10.  One step renders one sample per
pixel (921,600 paths) with NEE + MIS (`RayTracer::pathTrace`,
Renderer.h:531-613).  The metric is Mrays/s: extension plus shadow rays
traced per second of device time.

  python bench.py [--steps K] [--warmup W] [--impl pgx|reference]
                  [--mode plain|guided_quadtree] [--workload interior|cornell]

`--impl reference` times the reference's own CPU renderer
(`RayTracer::render`, Renderer.h:648-747, plain build) on all host cores
over the same scene, one frame per step.
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
sys.path.insert(0, str(ROOT))

L2_FLUSH_BYTES = 256 << 20  # > 129 MB L2


def make_workload(name: str):
    from pathguidingdissertation_gb300 import scenes
    if name == "cornell":
        return scenes.cornell_box(seed=1, width=256, height=256), 8, "cornell box, 36 tris, 256x256, depth 8"
    desc = scenes.interior(seed=2)
    return desc, 10, (f"procedural interior, {desc.ntris} tris, env 2048x1024, "
                      f"{desc.camera['width']}x{desc.camera['height']}, depth 10")


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during a region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self):
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.QUERY}", "--format=csv,noheader,nounits",
                                          "-lms", "200"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            self.proc.wait(timeout=5)

    def summary(self) -> dict:
        rows = []
        try:
            for line in open(self.path):
                parts = [p.strip() for p in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        except OSError:
            pass
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        smax = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": reasons, "samples": len(rows)}


class Ranks:
    """One process per GPU under torchrun.  The path does not shard (pixels
    and samples are independent), so N ranks are N replicas rendering their
    own samples; the only communication is the timing: barriers around the
    timed steps, sums of the units and the maximum of the times."""

    def __init__(self):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        self.pg = False
        self.device = "cpu"

    def init(self, backend: str) -> None:
        if self.world > 1:
            import torch
            import torch.distributed as dist
            os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
            if backend == "nccl":
                torch.cuda.set_device(self.local)
            dist.init_process_group(backend=backend)
            self.pg = True
            self.device = f"cuda:{self.local}" if backend == "nccl" else "cpu"

    def barrier(self) -> None:
        if self.pg:
            import torch.distributed as dist
            dist.barrier()

    def reduce(self, x: float, op: str = "sum") -> float:
        """Sum or maximum of x over the ranks (x itself with one rank)."""
        if not self.pg:
            return float(x)
        import torch
        import torch.distributed as dist
        t = torch.tensor([float(x)], dtype=torch.float64, device=self.device)
        dist.all_reduce(t, op=dist.ReduceOp.SUM if op == "sum" else dist.ReduceOp.MAX)
        return float(t.item())

    def close(self) -> None:
        if self.pg:
            import torch.distributed as dist
            dist.destroy_process_group()
            self.pg = False


def measured_peaks() -> dict:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return {"hbm_gbs": d.get("hbm_gbs", 6800.0), "source": "measured"}
    return {"hbm_gbs": 6800.0, "source": "fallback"}


def profile_traffic(kernel: str, units_per_launch: float) -> tuple[float | None, str | None, dict | None]:
    """Per-launch DRAM bytes of `kernel`, scaled from a committed ncu
    capture: its bytes per unit (extension ray) times the units of an average
    launch of this run; plus the capture's issue and cache figures."""
    p = ROOT / "profiles" / "traffic.json"
    if not p.exists():
        return None, None, None
    d = json.loads(p.read_text())
    e = d.get(kernel)
    if not e or "bytes_per_unit" not in e:
        return None, None, None
    return float(e["bytes_per_unit"]) * units_per_launch, e.get("note"), e.get("issue")


def cpu_baseline_reference(desc, frames_budget_s: float = 12.0) -> dict | None:
    """The reference's own plain renderer on all host cores, bounded sample."""
    try:
        from oracle.ffi import Reference, reference_available
        if not reference_available():
            return None
        ref = Reference(variant="plain_fast")
    except Exception as e:  # noqa: BLE001
        return {"unavailable": f"reference harness: {e}"}
    cores = os.cpu_count() or 1
    rs = ref.scene(desc, threads=cores)
    _, _, rays1, s1 = rs.render_native(1)
    frames = max(1, min(20, int(frames_budget_s / max(s1, 1e-3))))
    _, _, rays, secs = rs.render_native(frames)
    rs.close()
    return {"value": rays / secs / 1e6, "unit": "Mrays/s", "cores": cores, "kind": "reference",
            "sample": f"{frames} frame(s) of RayTracer::render (plain build, -O3) on the same scene, "
                      f"{rays} rays in {secs:.2f} s"}


# Training recipes of the guides on the 1280x720 interior (measured with
# --study relmse): the QuadTree guide from an unguided pass of 8 frames and a
# guided pass of 16 (each rebuilding the cache), 16,384-record regions,
# guide fraction 0.7, flux clamped at 20x the region's median, GGX conductors
# (alpha <= 1.62 for roughness <= 1) left to their BSDF; the learned guide
# trained online on 64 frames.
QT_RECIPE = dict(train_first=8, train_iters=2, qt_region=16384, qt_refine=0.01, qt_clamp=20.0, qt_uniform=0.2,
                 qt_compensate=0.0, qt_glossy_alpha=2.0, guide_fraction=0.7)
MLP_RECIPE = dict(guide_fraction=0.75, train_frames=64)


def prepare_mode(ctx, mode: int, depth: int) -> float:
    """Untimed set-up of a guided estimator (the QuadTree cache or the
    learned guide, trained by the recipes above); returns the guide
    fraction its renders use."""
    from pathguidingdissertation_gb300 import abi
    ctx.clear()
    if mode == abi.MODE_GUIDED_QUADTREE:
        r = QT_RECIPE
        ctx.guide_configure(region_records=r["qt_region"], refine_fraction=r["qt_refine"],
                            clamp_median=r["qt_clamp"], uniform_share=r["qt_uniform"],
                            compensate=r["qt_compensate"], glossy_alpha=r["qt_glossy_alpha"])
        for it in range(r["train_iters"]):
            n = r["train_first"] << it
            ctx.render(n, mode=abi.MODE_PLAIN if it == 0 else mode, seed=99 + it, max_depth=depth,
                       record_paths=n, guide_fraction=r["guide_fraction"])
        return r["guide_fraction"]
    if mode == abi.MODE_GUIDED_MLP:
        ctx.mlp_init(3)
        ctx.mlp_configure(lr=5e-3, decay=0.998, batch=1 << 18, steps=4)
        ctx.render(16, mode=mode, seed=99, max_depth=depth, train_guide=True,
                   guide_fraction=MLP_RECIPE["guide_fraction"])
        return MLP_RECIPE["guide_fraction"]
    return 0.5


def guarded(name: str, fn, *a) -> dict:
    """Runs one of the default line's side measurements; a failure there is
    recorded in the line ({"error": ...}) instead of ending the run, so the
    headline measured before it is still printed."""
    try:
        return fn(*a)
    except Exception as e:  # noqa: BLE001
        print(f"[bench] {name} failed: {type(e).__name__}: {e}", file=sys.stderr, flush=True)
        return {"error": f"{type(e).__name__}: {e}"}


def pick(r: dict, keys) -> dict:
    """The listed keys of a study's result (or its error)."""
    return r if "error" in r else {k: r[k] for k in keys}


def box_rate(flush, spp: int = 16, steps: int = 10, warmup: int = 3) -> dict:
    """Plain path tracing of the closed box (36 triangles, 256x256, depth 8,
    16 spp per step: the reference's CPU-runnable configuration), device
    time per step with the L2 flushed before each."""
    import torch

    from pathguidingdissertation_gb300 import abi
    from pathguidingdissertation_gb300.api import Context
    desc, depth, wl = make_workload("cornell")
    ctx = Context(0)
    ctx.upload(desc)
    ctx.bvh_build()
    ctx.clear()
    for _ in range(warmup):
        ctx.render(spp, mode=abi.MODE_PLAIN, seed=3, max_depth=depth, timing=True)
    rays = paths = 0
    ms = 0.0
    for _ in range(steps):
        flush.zero_()
        torch.cuda.synchronize()
        ctx.render(spp, mode=abi.MODE_PLAIN, seed=3, max_depth=depth, timing=True)
        st = ctx.render_stats()
        rays += st.extension_rays + st.shadow_rays
        paths += st.paths
        ms += st.ms_total
    ctx.close()
    return {"workload": wl, "spp_per_step": spp, "steps": steps, "ms_per_step": ms / steps,
            "mrays_per_s": rays / (ms * 1e-3) / 1e6, "mpaths_per_s": paths / (ms * 1e-3) / 1e6}


def side_mode_rate(ctx, mode: int, depth: int, spp: int, steps: int, seed: int, flush, ranks) -> dict:
    """Mrays/s and Mpaths/s of one more estimator on the bench's workload."""
    import torch
    frac = prepare_mode(ctx, mode, depth)
    ctx.clear()
    ctx.render(spp, mode=mode, seed=seed, max_depth=depth, timing=True, guide_fraction=frac)  # warm-up
    torch.cuda.synchronize()
    ranks.barrier()
    rays = paths = 0
    ms = 0.0
    for _ in range(steps):
        flush.zero_()
        torch.cuda.synchronize()
        ctx.render(spp, mode=mode, seed=seed, max_depth=depth, timing=True, guide_fraction=frac)
        st = ctx.render_stats()
        rays += st.extension_rays + st.shadow_rays
        paths += st.paths
        ms += st.ms_total
    torch.cuda.synchronize()
    ranks.barrier()
    ms_max = ranks.reduce(ms, "max")
    return {"mrays_per_s": ranks.reduce(rays, "sum") / (ms_max * 1e-3) / 1e6,
            "mpaths_per_s": ranks.reduce(paths, "sum") / (ms_max * 1e-3) / 1e6,
            "ms_per_step": ms_max / steps, "steps": steps, "max_depth": depth,
            "rays_per_path": rays / max(paths, 1)}


def run_pgx(args) -> dict:
    import torch

    from pathguidingdissertation_gb300 import abi
    from pathguidingdissertation_gb300 import build as pkg_build
    from pathguidingdissertation_gb300.api import Context

    ranks = Ranks()
    if ranks.rank == 0:
        pkg_build.build()
    ranks.init("nccl")
    if ranks.rank != 0:
        ranks.barrier()
        pkg_build.build()  # rank 0 compiled it; this only loads
    else:
        ranks.barrier()
    desc, depth, wl = make_workload(args.workload)
    if args.res:
        # a reduced image of the same scene (for profiler captures)
        w, h = (int(x) for x in args.res.split("x"))
        desc.camera = dict(desc.camera, width=w, height=h)
        wl = f"{wl}, image reduced to {args.res}"
    mode = {"plain": abi.MODE_PLAIN, "guided_quadtree": abi.MODE_GUIDED_QUADTREE,
            "guided_mlp": abi.MODE_GUIDED_MLP}[args.mode]
    seed = 1 + 1000003 * ranks.rank  # each replica renders its own samples
    ctx = Context(ranks.local)
    ctx.upload(desc)
    ctx.bvh_build()
    frac = prepare_mode(ctx, mode, depth)
    ctx.clear()
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device="cuda")
    spp = args.spp_per_step
    for i in range(args.warmup):
        ctx.render(spp, mode=mode, seed=seed, max_depth=depth, timing=True, guide_fraction=frac)
    # Node/triangle fetch counts of one step of the same workload (the counting
    # traversal kernels; untimed).  The timed steps run the uncounted kernels.
    ctx.render(spp, mode=mode, seed=seed, max_depth=depth, profile=True, guide_fraction=frac)
    cst = ctx.render_stats()
    visits_per_ray = cst.extend_interior_visits / max(cst.extension_rays, 1)
    tris_per_ray = cst.extend_tri_tests / max(cst.extension_rays, 1)
    sh_visits_per_ray = cst.shadow_interior_visits / max(cst.shadow_rays, 1)
    sh_tris_per_ray = cst.shadow_tri_tests / max(cst.shadow_rays, 1)
    torch.cuda.synchronize()
    ranks.barrier()
    rays = paths = ext_rays = sh_rays = 0
    ms = ms_ext = ms_shade = ms_shadow = 0.0
    ext_launches = launches = 0
    with ClockSampler() as clk:
        for k in range(args.steps):
            flush.zero_()
            torch.cuda.synchronize()
            ctx.render(spp, mode=mode, seed=seed, max_depth=depth, timing=True, guide_fraction=frac)
            st = ctx.render_stats()
            rays += st.extension_rays + st.shadow_rays
            paths += st.paths
            ms += st.ms_total
            ms_ext += st.ms_extend
            ms_shade += st.ms_shade
            ms_shadow += st.ms_shadow
            ext_rays += st.extension_rays
            sh_rays += st.shadow_rays
            ext_launches += st.extend_launches
            launches += st.kernel_launches
        torch.cuda.synchronize()
        ranks.barrier()
    clocks = clk.summary()
    ext_visits = visits_per_ray * ext_rays
    ext_tris = tris_per_ray * ext_rays
    # whole job: every replica's rays over the slowest replica's device time
    ms_max = ranks.reduce(ms, "max")
    rays_all = ranks.reduce(rays, "sum")
    paths_all = ranks.reduce(paths, "sum")
    value = rays_all / (ms_max * 1e-3) / 1e6

    # The other half of the metric: throughput of the guided estimators on the
    # same workload (each after its own untimed set-up, prepare_mode: the
    # QuadTree recipe's 8 + 16 training frames, or 16 frames of online
    # training), and plain path tracing at the reference arm's fixed depth 8
    # for an equal-depth anchor.
    # Same L2 flush and device timing as the steps above, fewer steps.
    side = {}
    if not args.no_side_modes:
        for name, m, d in (("guided_quadtree", abi.MODE_GUIDED_QUADTREE, depth),
                           ("guided_mlp", abi.MODE_GUIDED_MLP, depth), ("plain_depth8", abi.MODE_PLAIN, 8)):
            if m == mode and d == depth:
                continue
            side[name] = (side_mode_rate(ctx, m, d, spp, max(1, min(args.steps, 4)), seed, flush, ranks)
                          if ranks.world > 1 else
                          guarded(name, side_mode_rate, ctx, m, d, spp, max(1, min(args.steps, 4)), seed, flush,
                                  ranks))
        ctx.clear()

    # End to end through the C ABI: camera from host, render, film to pinned host memory.
    H, W = desc.camera["height"], desc.camera["width"]
    host_film = torch.empty((H, W, 3), dtype=torch.float32, pin_memory=True)
    import ctypes as C
    from pathguidingdissertation_gb300.api import camera_struct
    cam = camera_struct(desc.camera)
    cfg = abi.RenderConfig(mode, depth, seed, frac, 0, 0)
    spp_read = C.c_int32()
    e2e_rays = 0
    ranks.barrier()
    t0 = time.perf_counter()
    for k in range(args.steps):
        ctx.check(ctx.lib.pgx_set_camera(ctx.h, C.byref(cam)))
        ctx.check(ctx.lib.pgx_render(ctx.h, C.byref(cfg), spp))
        ctx.check(ctx.lib.pgx_film_read(ctx.h, host_film.data_ptr(), None, C.byref(spp_read)))
        st = ctx.render_stats()
        e2e_rays += st.extension_rays + st.shadow_rays
    e2e_s = time.perf_counter() - t0
    ranks.barrier()
    e2e_value = ranks.reduce(e2e_rays, "sum") / ranks.reduce(e2e_s, "max") / 1e6
    ctx.close()

    peaks = measured_peaks()
    alg_bytes = ext_visits * 64 + ext_tris * 48
    achieved = alg_bytes / (ms_ext * 1e-3) / 1e9 if ms_ext > 0 else None
    traffic, traffic_note, issue = profile_traffic("k_extend", ext_rays / max(ext_launches, 1))
    avg_launch_s = (ms_ext / max(ext_launches, 1)) * 1e-3
    dram_gbs = traffic / avg_launch_s / 1e9 if (traffic and avg_launch_s > 0) else None
    roofline = {
        "kernel": "k_extend (closest-hit traversal)",
        # The 20 MB tree stays in L2: DRAM carries only the path state, and
        # the kernel is limited by instruction issue of divergent warps.
        # achieved/frac are the algorithmic node and triangle bytes (counted
        # on the device) per second against the measured HBM copy rate, for
        # comparison across builds; dram_gbs/dram_frac are the DRAM bytes the
        # capture measured, scaled to this run's launches.
        "bound": "issue",
        "achieved": achieved,
        "peak": peaks["hbm_gbs"],
        "peak_source": peaks["source"],
        "unit": "GB/s",
        "frac": (achieved / peaks["hbm_gbs"]) if achieved else None,
        "traffic": traffic,
        "traffic_note": traffic_note,
        "dram_gbs": dram_gbs,
        "dram_frac": (dram_gbs / peaks["hbm_gbs"]) if dram_gbs else None,
        "issue_profile": issue,
        "alg_bytes_per_launch": alg_bytes / max(ext_launches, 1),
        "nodes_per_ray": visits_per_ray,
        "tris_per_ray": tris_per_ray,
        "counts_note": "per extension ray, from one untimed step run with the counting traversal kernels",
        "avg_launch_ms": ms_ext / max(ext_launches, 1),
        "extend_share_of_step": ms_ext / ms if ms else None,
    }
    # k_shade: one launch per depth, one path vertex per extension ray; per
    # vertex it reads the path state (80 B) and the hit triangle's shading
    # record (80 B), writes the continuation (64 B) and a shadow-ray record
    # (52 B) and updates the radiance (32 B): 308 B.
    shade_bytes = 308.0 * ext_rays
    shade_achieved = shade_bytes / (ms_shade * 1e-3) / 1e9 if ms_shade > 0 else None
    roofline_shade = {
        "kernel": "k_shade (path vertex: integrator step, BSDF, NEE)",
        "bound": "hbm",
        "achieved": shade_achieved,
        "peak": peaks["hbm_gbs"],
        "unit": "GB/s",
        "frac": (shade_achieved / peaks["hbm_gbs"]) if shade_achieved else None,
        "alg_bytes_per_vertex": 308,
        "shade_share_of_step": ms_shade / ms if ms else None,
        "note": "latency-bound (dependent gathers of shading data, 64 registers); traffic not captured",
    }
    # The other half of the metric: equal-time relMSE of the learned guide
    # against plain path tracing (a reduced form of --study relmse: the
    # converged image at 8,192 spp instead of 65,536; not part of the timed
    # steps).  Rank 0 of a single-GPU run only.
    equal_time = None
    if not args.no_equal_time and ranks.world == 1 and args.workload == "interior" and not args.res:
        import copy
        import tempfile
        equal_time = {
            "study": "QuadTree and learned guides vs plain GPU path tracing, time to plain's 1024-spp relMSE",
            "reference_spp": 8192,
            "metric": "relMSE (x-r)^2/(r^2+0.01) without the 0.1 % largest pixel errors; the plain relMSE beside",
            "guides": {},
        }
        with tempfile.TemporaryDirectory() as td:
            for guide, recipe in (("quadtree", QT_RECIPE), ("mlp", MLP_RECIPE)):
                sa = copy.copy(args)
                sa.study_res, sa.ref_spp, sa.plain_spp, sa.guide, sa.metric = "1280x720", 8192, 1024, guide, "robust"
                sa.ref_cache, sa.save_images = str(Path(td) / "reference.npy"), None  # one converged image for both
                for k, v in recipe.items():
                    setattr(sa, k, v)
                print(f"[bench] equal-time relMSE study ({guide})", file=sys.stderr, flush=True)
                r = guarded(f"equal-time study ({guide})", run_relmse_study, sa)
                if "error" in r:
                    equal_time["guides"][guide] = r
                    continue
                equal_time["workload"] = r["workload"]
                equal_time["plain_ms"] = r["plain"]["ms"]
                equal_time["plain_relmse"] = r["plain"]["relmse"]
                equal_time["plain_relmse_plain_metric"] = r["plain"]["relmse_other_metric"]
                equal_time["guides"][guide] = {
                    "recipe": recipe,
                    "train_ms": r["guided"]["train_ms"], "ms_to_plain_error": r["guided"]["ms_to_plain_error"],
                    "relmse_at_plain_time": r["guided"]["relmse_at_plain_time"],
                    "time_ratio_guided_over_plain": r["time_ratio_guided_over_plain"],
                    "time_ratio_plain_metric": r["time_ratio_other_metric"],
                }
    # k_shadow (any hit): node and triangle fetches of the shadow rays over
    # its CUDA-event time; like k_extend it reads a tree that stays in L2.
    sh_bytes = (sh_visits_per_ray * 64 + sh_tris_per_ray * 48) * sh_rays
    sh_achieved = sh_bytes / (ms_shadow * 1e-3) / 1e9 if ms_shadow > 0 else None
    roofline_shadow = {
        "kernel": "k_shadow (any-hit traversal of the NEE shadow rays)",
        "bound": "issue",
        "achieved": sh_achieved,
        "peak": peaks["hbm_gbs"],
        "unit": "GB/s",
        "frac": (sh_achieved / peaks["hbm_gbs"]) if sh_achieved else None,
        "nodes_per_ray": sh_visits_per_ray,
        "tris_per_ray": sh_tris_per_ray,
        "mrays_per_s": sh_rays / (ms_shadow * 1e-3) / 1e6 if ms_shadow > 0 else None,
        "shadow_share_of_step": ms_shadow / ms if ms else None,
        "note": "algorithmic node (64 B) and triangle (48 B) bytes per second against the HBM copy rate; the tree "
                "is L2-resident as for k_extend",
    }
    # The other configurations, each a bounded run outside the timed steps so
    # that the line records them too: the plain box (16 spp, 256x256, depth
    # 8), incoherent secondary rays on the 2M-triangle interior (10^7 rays),
    # the adjoint on the 2M-triangle terrain (with a few finite differences)
    # and the 64-scene batch.  Rank 0 of a single-GPU run only.
    workloads = None
    if not args.no_workloads and ranks.world == 1 and args.workload == "interior" and not args.res:
        import copy
        print("[bench] other workloads", file=sys.stderr, flush=True)
        workloads = {"plain_box": guarded("box", box_rate, flush)}
        sa = copy.copy(args)
        sa.trav_rays, sa.steps, sa.warmup, sa.no_cpu_baseline = 10_000_000, 5, 2, True
        workloads["traversal_2m"] = pick(guarded("traversal", run_traversal_study, sa), (
            "scene", "rays", "ms", "mrays_per_s", "interior_nodes_per_ray", "triangles_per_ray", "alg_gbs",
            "hbm_frac"))
        sa = copy.copy(args)
        sa.fd_params, sa.diff_grid, sa.diff_res, sa.diff_spp = 24, 1024, 512, 64
        workloads["adjoint_terrain"] = pick(guarded("adjoint", run_adjoint_study, sa), (
            "workload", "spp", "primal_mpaths_per_s", "adjoint_mpaths_per_s", "gradient_entries", "fd_params",
            "rel_err_median", "frac_significant_within_1e-3_rel", "n_significant"))
        sa = copy.copy(args)
        sa.batch_scenes, sa.batch_res, sa.batch_max_tris, sa.batch_relmse = 64, 0, 2e6, False
        t0 = time.perf_counter()
        workloads["batch_64_scenes"] = dict(pick(guarded("batch", run_batch_study, sa), (
            "scenes", "spp", "max_depth", "paths", "triangles_total", "tuning", "batch_mpaths_per_s",
            "graph_replay_mpaths_per_s", "sequential_mpaths_per_s")), wall_s=time.perf_counter() - t0)
    print("[bench] device runs done; CPU baseline next", file=sys.stderr, flush=True)
    cpu = cpu_baseline_reference(desc) if not args.no_cpu_baseline and ranks.world == 1 else None
    print("[bench] CPU baseline done", file=sys.stderr, flush=True)
    ranks.close()
    if ranks.rank != 0:
        return None
    return {
        "metric": "Mrays/s",
        "value": value,
        "unit": "Mrays/s",
        "n_gpus": ranks.world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": ms_max / args.steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic (seeded procedural scene)",
        "config": {"workload": wl, "mode": args.mode, "paths_per_step": int(paths_all) // max(args.steps, 1),
                   "spp_per_step": spp, "l2": "flushed (256 MiB write) before every timed step",
                   "parallelism": "replicas" if ranks.world > 1 else "1 GPU"},
        "mpaths_per_s": paths_all / (ms_max * 1e-3) / 1e6,
        "rays_per_path": rays / max(paths, 1),
        "gpu_launches": launches,
        "e2e": {"value": e2e_value, "unit": "Mrays/s", "h2d_bytes_per_step": C.sizeof(abi.Camera),
                "d2h_bytes_per_step": H * W * 3 * 4},
        "modes": side,
        "equal_time": equal_time,
        "workloads": workloads,
        "roofline": roofline,
        "roofline_shade": roofline_shade,
        "roofline_shadow": roofline_shadow,
        "cpu_baseline": cpu,
        "clocks": clocks,
    }


def relmse(img: np.ndarray, ref: np.ndarray, eps: float = 1e-2) -> float:
    """Mean of (x - r)^2 / (r^2 + eps) over pixels and channels."""
    d = img.astype(np.float64) - ref
    return float(np.mean(d * d / (ref * ref + eps)))


def relmse_robust(img: np.ndarray, ref: np.ndarray, eps: float = 1e-2, drop: float = 1e-3) -> float:
    """relMSE with the largest 0.1 % of per-pixel errors left out (a few
    fireflies from the sun lobe otherwise decide the mean)."""
    from pathguidingdissertation_gb300 import metrics
    return metrics.relmse_robust(img, ref, eps, drop)


def rrmse_reference_metric(img: np.ndarray, ref: np.ndarray) -> float:
    """Metrics::calculateRRMSE (Metrics.h:48-68): RMSE / (sqrt(sum ref^2) + 1e-2)."""
    d = img.astype(np.float64) - ref
    return float(np.sqrt(np.mean(d * d)) / (np.sqrt(np.sum(ref.astype(np.float64) ** 2)) + 1e-2))


def run_relmse_study(args) -> dict:
    """Equal-time relMSE of guided (learned or QuadTree) vs plain path tracing
    against a converged plain render of the same view.  All times are device
    times of pgx_render (and of the cache build); training frames are part of
    the guided image and of its time."""
    from pathguidingdissertation_gb300 import abi
    from pathguidingdissertation_gb300 import build as pkg_build
    from pathguidingdissertation_gb300.api import Context

    pkg_build.build()
    w, h = (int(x) for x in args.study_res.split("x"))
    desc, depth, _ = make_workload(args.workload)
    desc.camera = dict(desc.camera, width=w, height=h)
    ctx = Context(0)
    ctx.upload(desc)
    ctx.bvh_build()

    def render_ms(frames, mode, seed, **kw):
        ms = 0.0
        left = frames
        while left > 0:
            n = min(left, 256)
            ctx.render(n, mode=mode, seed=seed, max_depth=depth, **kw)
            ms += ctx.render_stats().ms_total
            left -= n
        return ms

    def image():
        rgb, _, spp = ctx.film()
        return rgb.astype(np.float64) / spp

    ctx.clear()
    cache = Path(args.ref_cache) if args.ref_cache else None
    if cache is not None and cache.exists():
        ref = np.load(cache)
        ref_ms = float("nan")
    else:
        ref_ms = render_ms(args.ref_spp, abi.MODE_PLAIN, 1000)
        ref = image()
        if cache is not None:
            np.save(cache, ref)
    metric = relmse_robust if args.metric == "robust" else relmse

    # Plain: its error at plain_spp and the time it takes.
    ctx.clear()
    plain_ms = render_ms(args.plain_spp, abi.MODE_PLAIN, 7)
    plain_img = image()
    plain_err = metric(plain_img, ref)
    other = relmse if metric is relmse_robust else relmse_robust

    ctx.clear()
    train_ms = 0.0
    train_spp = 0
    extra = {}
    if args.guide == "mlp":
        # Learned guide: online training on the first `train_frames` frames
        # (`mlp_steps` Adam steps per frame, batch 2^18), which stay in the image.
        ctx.mlp_init(3)
        ctx.mlp_configure(lr=args.mlp_lr, decay=args.mlp_decay, batch=args.mlp_batch, steps=args.mlp_steps,
                          direct=not args.mlp_indirect)
        mode = abi.MODE_GUIDED_MLP
        if args.mlp_cache_frames > 0:
            # QuadTree fallback: a radiance cache from unguided frames (kept in
            # the image) guides the regions the network has not learned yet.
            ctx.guide_configure(region_records=args.qt_region, refine_fraction=args.qt_refine,
                                clamp_median=args.qt_clamp, uniform_share=args.qt_uniform,
                                compensate=args.qt_compensate, glossy_alpha=args.qt_glossy_alpha)
            train_ms += render_ms(args.mlp_cache_frames, abi.MODE_PLAIN, 9 + args.study_seed,
                                  record_paths=args.mlp_cache_frames)
            train_ms += ctx.cache_stats().build_ms
            train_spp += args.mlp_cache_frames
            ctx.mlp_set_fallback(args.mlp_fallback)
        train_ms += render_ms(args.train_frames, mode, 13 + args.study_seed, guide_fraction=args.guide_fraction,
                              train_guide=True,
                              guide_depth=args.guide_depth)
        train_spp += args.train_frames
        extra = {"train_frames": args.train_frames, "cache_frames": args.mlp_cache_frames,
                 "fallback_min_samples": args.mlp_fallback if args.mlp_cache_frames > 0 else None,
                 "lr": args.mlp_lr, "lr_decay": args.mlp_decay,
                 "adam_steps_per_frame": args.mlp_steps, "batch": args.mlp_batch, "guide_depth": args.guide_depth,
                 "target": "indirect" if args.mlp_indirect else "full incident radiance"}
    else:
        # QuadTree (directions) or PSS (primary samples): train the cache over
        # `train_iters` iterations of train_first x 1, 2, 4, ... frames (the
        # first unguided, the rest guided by the previous cache; every
        # iteration's records rebuild the cache, in the domain of the mode
        # that recorded them, weighted by Lum(Li) |cos| / pdf), all timed.
        # The training frames are unbiased samples too and stay in the image.
        mode = abi.MODE_GUIDED_PSS if args.guide == "pss" else abi.MODE_GUIDED_QUADTREE
        ctx.guide_configure(region_records=args.qt_region, refine_fraction=args.qt_refine,
                            clamp_median=args.qt_clamp, uniform_share=args.qt_uniform,
                            compensate=args.qt_compensate, glossy_alpha=args.qt_glossy_alpha)
        builds = []
        for it in range(args.train_iters):
            n = args.train_first << it
            m = abi.MODE_PLAIN if (it == 0 and args.guide == "quadtree") else mode
            train_ms += render_ms(n, m, 11 + it + args.study_seed, record_paths=n,
                                  guide_fraction=args.guide_fraction)
            builds.append(ctx.cache_stats().build_ms)
            train_ms += builds[-1]
            train_spp += n
        extra = {"train_iters": args.train_iters, "train_first": args.train_first,
                 "cache_records": ctx.cache_stats().records, "cache_build_ms": builds,
                 "guide_params": ctx.guide_params()}
    guided_ms = 0.0
    curve = []
    reached_ms = reached_chunk_ms = reached_other_seen = None
    chunk = max(1, args.plain_spp // 32)
    total = train_spp
    while total < 4 * args.plain_spp:
        guided_ms += render_ms(chunk, mode, 17 + total + args.study_seed, guide_fraction=args.guide_fraction,
                               guide_depth=args.guide_depth)
        total += chunk
        img = image()
        err = metric(img, ref)
        curve.append((total, train_ms + guided_ms, err, other(img, ref)))
        if reached_ms is None and err <= plain_err:
            reached_ms = train_ms + guided_ms
            if len(curve) >= 2:
                # between the last two points, 1 / relMSE grows linearly in
                # time (relMSE ~ 1 / t): the crossing inside this chunk
                (_, t0, e0, _), (_, t1, e1, _) = curve[-2], curve[-1]
                if e0 > plain_err > 0 and e1 > 0:
                    f = (1.0 / plain_err - 1.0 / e0) / (1.0 / e1 - 1.0 / e0)
                    reached_ms = t0 + f * (t1 - t0)
            reached_chunk_ms = train_ms + guided_ms
        if reached_other_seen is None and curve[-1][3] <= other(plain_img, ref):
            reached_other_seen = total
        if train_ms + guided_ms >= 2.0 * plain_ms and reached_ms is not None and reached_other_seen is not None:
            break
        if train_ms + guided_ms >= 4.0 * plain_ms:
            break
    # Guided error at the plain render's wall time (linear between points).
    eq_err = None
    for (s0, t0, e0, _), (s1, t1, e1, _) in zip(curve, curve[1:]):
        if t0 <= plain_ms <= t1:
            eq_err = e0 + (e1 - e0) * (plain_ms - t0) / max(t1 - t0, 1e-9)
    # the same ratio under the other metric (robust <-> plain relMSE)
    plain_other = other(plain_img, ref)
    reached_other = None
    for k, (_, t, _, e) in enumerate(curve):
        if e <= plain_other:
            reached_other = t
            if k > 0 and curve[k - 1][3] > plain_other > 0 and e > 0:
                t0, e0 = curve[k - 1][1], curve[k - 1][3]
                reached_other = t0 + (1.0 / plain_other - 1.0 / e0) / (1.0 / e - 1.0 / e0) * (t - t0)
            break
    guided_img = image()
    if args.save_images:
        d = Path(args.save_images)
        d.mkdir(parents=True, exist_ok=True)
        np.save(d / f"plain_{args.plain_spp}spp.npy", plain_img.astype(np.float32))
        np.save(d / f"guided_{args.guide}.npy", guided_img.astype(np.float32))
    ctx.close()
    return {
        "study": f"equal-time relMSE, {args.guide}-guided vs plain GPU path tracing",
        "metric": "relMSE (x-r)^2/(r^2+0.01)" + (", largest 0.1% pixel errors left out" if args.metric == "robust"
                                                else ""),
        "workload": f"{args.workload} {w}x{h}, depth {depth}",
        "reference": {"spp": args.ref_spp, "ms": ref_ms},
        "plain": {"spp": args.plain_spp, "ms": plain_ms, "relmse": plain_err, "relmse_other_metric": plain_other,
                  "rrmse_metrics_h": rrmse_reference_metric(plain_img, ref)},
        "guided": dict(extra, guide=args.guide, train_spp=train_spp, train_ms=train_ms,
                       guide_fraction=args.guide_fraction, spp_rendered=total,
                       ms_to_plain_error=reached_ms, ms_to_plain_error_chunk_end=reached_chunk_ms,
                       relmse_at_plain_time=eq_err,
                       rrmse_metrics_h_final=rrmse_reference_metric(guided_img, ref),
                       curve=[{"spp": a, "ms": b, "relmse": c, "relmse_other_metric": d} for a, b, c, d in curve]),
        "time_ratio_guided_over_plain": (reached_ms / plain_ms) if reached_ms else None,
        "time_ratio_other_metric": (reached_other / plain_ms) if reached_other else None,
    }


def run_adjoint_study(args) -> dict:
    """Differentiable rendering of the fBm heightfield (2,093,058 triangles,
    32 GGX conductor materials, 512x256 environment, 512x512): a target at
    256 spp from parameters perturbed by N(0, 0.05), the L2 loss of a 64-spp
    render, its gradient with respect to every environment texel and the 32
    albedo (rgb) and 32 roughness values by the adjoint kernel, and central
    finite differences (h = 1e-3) of the same renderer on random parameters."""
    import time
    from pathguidingdissertation_gb300 import build as pkg_build
    from pathguidingdissertation_gb300 import scenes
    from pathguidingdissertation_gb300.api import Context

    pkg_build.build()
    # --diff-grid / --diff-res / --diff-spp shrink the case (profiler captures)
    desc = scenes.terrain(grid=args.diff_grid, width=args.diff_res, height=args.diff_res)
    ctx = Context(0)
    ctx.upload(desc)
    ctx.bvh_build()
    nm = len(desc.materials)
    rng = np.random.default_rng(1)
    depth, spp, seed = 8, args.diff_spp, 11
    env0 = desc.env.astype(np.float32)
    rough0 = desc.materials["roughness"].astype(np.float32)
    ctx.diff_set_params(env=(env0 + rng.normal(0, 0.05, env0.shape) * np.maximum(env0, 1e-3)).astype(np.float32)
                        .clip(0.0, None),
                        albedo_offset=rng.normal(0, 0.05, (nm, 3)).astype(np.float32),
                        roughness=np.clip(rough0 + rng.normal(0, 0.05, nm), 0.02, 1.0).astype(np.float32))
    t0 = time.perf_counter()
    target = ctx.diff_render(256, seed=99, max_depth=depth)
    target_s = time.perf_counter() - t0
    ctx.diff_set_params()
    t0 = time.perf_counter()
    img = ctx.diff_render(spp, seed, depth)
    primal_s = time.perf_counter() - t0
    loss = float(np.sum((img - target) ** 2))
    dimg = (2.0 * (img - target)).astype(np.float32)
    t0 = time.perf_counter()
    g_env, g_alb, g_rough = ctx.diff_adjoint(dimg, spp, seed, depth)
    adjoint_s = time.perf_counter() - t0
    h = 1e-3
    env_step = 0.1
    n_fd = args.fd_params
    kinds = rng.choice(3, n_fd, p=[0.5, 0.25, 0.25])
    res = []
    t0 = time.perf_counter()
    used = np.unique(desc.triangles["material"])
    nz_env = np.flatnonzero(np.abs(g_env).ravel() > 0)
    for k in kinds:
        step = h
        if k == 0:
            # The image is linear in every texel (sampling is detached), so the
            # loss is quadratic in it and the central difference is exact at
            # any step, up to the float32 rounding of each path's radiance: a
            # dim texel moved by 1e-3 changes a path that also carries the
            # sun lobe by little more than that rounding.  The step is
            # therefore 0.1 x max(1, texel).
            idx = int(rng.choice(nz_env))
            step = env_step * max(1.0, abs(float(env0.ravel()[idx])))
            e1 = env0.copy().ravel(); e1[idx] += step
            e2 = env0.copy().ravel(); e2[idx] -= step
            lp = (dict(env=e1.reshape(env0.shape)), dict(env=e2.reshape(env0.shape)))
            g = float(g_env.ravel()[idx]); name = f"env[{idx}]"
        elif k == 1:
            m, c = int(rng.choice(used)), int(rng.integers(3))

            def lp_at(hh, m=m, c=c):
                a = np.zeros((nm, 3), np.float32); a[m, c] = hh
                return dict(albedo_offset=a), dict(albedo_offset=-a)
            g = float(g_alb[m, c]); name = f"albedo[{m},{c}]"
        else:
            m = int(rng.choice(used))

            def lp_at(hh, m=m):
                r1 = rough0.copy(); r1[m] += hh
                r2 = rough0.copy(); r2[m] -= hh
                return dict(roughness=r1), dict(roughness=r2)
            g = float(g_rough[m]); name = f"roughness[{m}]"

        def central(pair, st):
            vals = []
            for kw in pair:
                ctx.diff_set_params(**kw)
                vals.append(float(np.sum((ctx.diff_render(spp, seed, depth) - target) ** 2)))
            return (vals[0] - vals[1]) / (2 * st)

        if k == 0:
            res.append((name, central(lp, step), g, None))
        else:
            # Albedo and roughness enter the image nonlinearly (GGX D and G
            # in roughness; products of albedos along a path), so the
            # central difference carries an h^2 truncation term; Richardson
            # extrapolation of the differences at h and h/2 cancels it.
            d1 = central(lp_at(h), h)
            d2 = central(lp_at(h / 2), h / 2)
            res.append((name, (4.0 * d2 - d1) / 3.0, g, d1))
    fd_s = time.perf_counter() - t0
    ctx.diff_set_params()
    ctx.close()
    if not res:  # --fd-params 0: timing only
        res = [("none", 1.0, 1.0, None)]
    fd = np.array([r[1] for r in res])
    ad = np.array([r[2] for r in res])
    rel = np.abs(ad - fd) / np.maximum(np.abs(fd), 1e-30)
    # the plain h = 1e-3 central difference for albedo and roughness, beside
    raw = np.array([r[3] if r[3] is not None else r[1] for r in res])
    rel_raw = np.abs(ad - raw) / np.maximum(np.abs(raw), 1e-30)
    scale = np.abs(fd).max()
    significant = np.abs(fd) > 1e-3 * scale
    paths = args.diff_res * args.diff_res * spp
    return {
        "study": "adjoint gradients vs central finite differences, fBm heightfield",
        "fd_step": "albedo offsets and roughness: central differences at h = 1e-3 and 5e-4 combined by Richardson "
                   "extrapolation; environment texels: 0.1 x max(1, texel) (exact: the loss is quadratic in a texel)",
        "workload": f"terrain {desc.ntris} tris, {nm} materials, env 512x256, {args.diff_res}x{args.diff_res}, "
                    f"depth {depth}",
        "loss": loss, "spp": spp, "target_spp": 256,
        "primal_s": primal_s, "adjoint_s": adjoint_s, "target_s": target_s,
        "primal_mpaths_per_s": paths / primal_s / 1e6, "adjoint_mpaths_per_s": paths / adjoint_s / 1e6,
        "gradient_entries": int(g_env.size + g_alb.size + g_rough.size),
        "fd_params": n_fd, "fd_s": fd_s,
        "rel_err_median": float(np.median(rel)), "rel_err_max_significant": float(rel[significant].max()),
        "frac_within_1e-3_rel": float(np.mean(rel <= 1e-3)),
        "frac_significant_within_1e-3_rel": float(np.mean(rel[significant] <= 1e-3)),
        "n_significant": int(significant.sum()),
        "frac_significant_within_1e-3_rel_plain_h": float(np.mean(rel_raw[significant] <= 1e-3)),
        "worst": [r[:3] for r in sorted(res, key=lambda r: -abs(r[2] - r[1]) / max(abs(r[1]), 1e-30))[:5]],
    }


def run_batch_study(args) -> dict:
    """Batched rendering: `batch_scenes` Cornell-box scenes (the plain
    configuration's generator) with triangle counts log-uniform in 1k-2M and
    resolutions from {128^2, 256^2, 512^2, 1024^2}, 32 spp, depth 8, in one
    persistent graph-captured launch (autotuned), against rendering the
    scenes one after another with pgx_render; per-scene relMSE of the batch
    image and of the reference CPU renderer's image (same spp) against a
    converged GPU image, for the scenes small enough for the CPU."""
    import time
    from pathguidingdissertation_gb300 import abi, scenes
    from pathguidingdissertation_gb300 import build as pkg_build
    from pathguidingdissertation_gb300.api import Batch, Context

    pkg_build.build()
    rng = np.random.default_rng(0)
    n = args.batch_scenes
    spp, depth = 32, 8
    specs = []
    for i in range(n):
        tris = int(np.exp(rng.uniform(np.log(1e3), np.log(args.batch_max_tris))))
        res = int(rng.choice([128, 256, 512, 1024])) if args.batch_res == 0 else args.batch_res
        specs.append(dict(seed=i + 1, width=res, height=res, target_tris=tris))
    t0 = time.perf_counter()
    descs = [scenes.cornell_box(**sp) for sp in specs]
    gen_s = time.perf_counter() - t0
    ctxs = []
    build_ms = 0.0
    for d in descs:
        c = Context(0)
        c.upload(d)
        c.bvh_build()
        build_ms += c.bvh_stats().build_ms
        ctxs.append(c)
    b = Batch(ctxs)
    tuning = b.autotune(spp=1, max_depth=depth)
    for c in ctxs:
        c.clear()
    b.render(spp, seed=1, max_depth=depth)
    st = b.stats()
    batch_ms = st.ms
    paths = st.paths
    # replay of the captured graph (another 32 spp), timed separately
    imgs = [c.film()[0].astype(np.float64) / spp for c in ctxs]
    b.render(spp, seed=2, max_depth=depth)
    replay_ms = b.stats().ms
    seq_ms = 0.0
    for c in ctxs:
        c.clear()
        left = spp
        while left > 0:
            k = min(left, 256)
            c.render(k, mode=abi.MODE_PLAIN, seed=1, max_depth=depth)
            seq_ms += c.render_stats().ms_total
            left -= k
    per_scene = []
    ref = None
    try:
        from oracle.ffi import Reference, reference_available
        if reference_available():
            ref = Reference(variant="plain_fast")
    except Exception:
        ref = None
    for i, (sp, d, c) in enumerate(zip(specs, descs, ctxs)):
        row = dict(tris=int(d.ntris), res=sp["width"])
        if getattr(args, "batch_relmse", True) and sp["width"] <= 256 and d.ntris <= 300_000:
            c.clear()
            c.render(1024, mode=abi.MODE_PLAIN, seed=77, max_depth=depth)
            conv = c.film()[0].astype(np.float64) / 1024
            row["relmse_batch"] = relmse(imgs[i], conv)
            if ref is not None:
                rs = ref.scene(d, threads=os.cpu_count() or 1)
                film, _, _ = rs.render_pcg(False, 1, 0, spp, threads=os.cpu_count() or 1)
                rs.close()
                row["relmse_reference_cpu"] = relmse(film.astype(np.float64) / spp, conv)
        per_scene.append(row)
    b.close()
    for c in ctxs:
        c.close()
    rows = [r for r in per_scene if "relmse_reference_cpu" in r]
    ratio = [r["relmse_batch"] / r["relmse_reference_cpu"] for r in rows if r["relmse_reference_cpu"] > 0]
    return {
        "study": "batched wavefront rendering: one graph-captured launch over many scenes",
        "scenes": n, "spp": spp, "max_depth": depth, "paths": int(paths),
        "resolutions": sorted({sp["width"] for sp in specs}), "max_tris_drawn": args.batch_max_tris,
        "triangles_total": int(sum(d.ntris for d in descs)),
        "tuning": {"wave_paths": tuning.wave_paths, "trace_blocks_per_sm": tuning.trace_blocks_per_sm,
                   "shade_blocks_per_sm": tuning.shade_blocks_per_sm},
        "batch_ms": batch_ms, "batch_mpaths_per_s": paths / batch_ms / 1e3,
        "graph_replay_ms": replay_ms, "graph_replay_mpaths_per_s": paths / replay_ms / 1e3,
        "sequential_ms": seq_ms, "sequential_mpaths_per_s": paths / seq_ms / 1e3,
        "scene_generation_s": gen_s, "bvh_build_ms_total": build_ms,
        "relmse_checked_scenes": len(rows),
        "relmse_batch_over_reference_median": float(np.median(ratio)) if ratio else None,
        "per_scene": per_scene,
    }


def run_traversal_study(args) -> dict:
    """Incoherent secondary-ray closest-hit traversal on the ~2M-triangle
    interior: 10^7 rays whose origins are 1-spp first hits and whose
    directions are cosine-distributed about the geometric normal (seed 7)."""
    import torch

    from pathguidingdissertation_gb300 import abi, scenes
    from pathguidingdissertation_gb300 import build as pkg_build
    from pathguidingdissertation_gb300.api import Context

    pkg_build.build()
    desc = scenes.interior(seed=2, target_tris=2_000_000, env_width=64, env_height=32)
    ctx = Context(0)
    ctx.upload(desc)
    t0 = time.perf_counter()
    ctx.bvh_build()
    build_s = time.perf_counter() - t0
    bst = ctx.bvh_stats()
    rng = np.random.default_rng(7)
    n = args.trav_rays
    W, H = desc.camera["width"], desc.camera["height"]
    px = (rng.random(n) * W).astype(np.float32)
    py = (rng.random(n) * H).astype(np.float32)
    cam = ctx.camera_rays(px, py)
    first = ctx.trace_closest(cam)
    hit = first["id"] >= 0
    tris = desc.triangles["v"]["p"].astype(np.float64)
    ids = first["id"][hit]
    p = cam["o"][hit] + cam["d"][hit] * first["t"][hit][:, None]
    e1 = tris[ids, 2] - tris[ids, 1]
    e2 = tris[ids, 0] - tris[ids, 2]
    ng = np.cross(e1, e2)
    ng /= np.linalg.norm(ng, axis=1, keepdims=True)
    ng = np.where((np.einsum("ij,ij->i", ng, cam["d"][hit]) > 0)[:, None], -ng, ng)
    # cosine-weighted directions about ng
    r1, r2 = rng.random(len(ng)), rng.random(len(ng))
    t = np.where(np.abs(ng[:, 0:1]) > 0.9, [[0.0, 1.0, 0.0]], [[1.0, 0.0, 0.0]])
    u = np.cross(t, ng)
    u /= np.linalg.norm(u, axis=1, keepdims=True)
    v = np.cross(ng, u)
    sr = np.sqrt(r1)
    d = (u * (sr * np.cos(2 * np.pi * r2))[:, None] + v * (sr * np.sin(2 * np.pi * r2))[:, None]
         + ng * np.sqrt(1 - r1)[:, None])
    rays = np.zeros(len(d), abi.RAY)
    rays["o"] = (p + ng * 1e-4).astype(np.float32)
    rays["d"] = d.astype(np.float32)
    rays["tmax"] = np.finfo(np.float32).max
    rays = np.resize(rays, n)  # reuse origins to reach exactly n rays
    drays = torch.from_numpy(rays.view(np.uint8)).cuda()
    dhits = torch.empty(n * 16, dtype=torch.uint8, device="cuda")
    stream = torch.cuda.current_stream()
    times = []
    for it in range(args.warmup + args.steps):
        e0 = torch.cuda.Event(enable_timing=True)
        e1_ = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        ctx.check(ctx.lib.pgx_trace_closest_device(ctx.h, drays.data_ptr(), n, dhits.data_ptr(), stream.cuda_stream))
        e1_.record(stream)
        torch.cuda.synchronize()
        if it >= args.warmup:
            times.append(e0.elapsed_time(e1_))
    iv, tt = ctx.trace_counters()
    hits = dhits.cpu().numpy().view(abi.HIT)
    ms = float(np.median(times))
    alg_bytes = iv * 64 + tt * 48
    peaks = measured_peaks()
    out = {
        "study": "incoherent secondary-ray closest-hit traversal",
        "scene": f"interior, {desc.ntris} triangles, GPU binned-SAH BVH ({bst.nodes} nodes, depth {bst.max_depth}, "
                 f"SAH {bst.sah_cost:.2f}, build {bst.build_ms:.1f} ms)",
        "rays": n,
        "ms": ms,
        "mrays_per_s": n / ms / 1e3,
        "interior_nodes_per_ray": iv / n,
        "triangles_per_ray": tt / n,
        "alg_gbs": alg_bytes / (ms * 1e-3) / 1e9,
        "hbm_frac": alg_bytes / (ms * 1e-3) / 1e9 / peaks["hbm_gbs"],
        "hit_fraction": float(np.mean(hits["id"] >= 0)),
        "bvh_build_s_host_clock": build_s,
    }
    if not args.no_cpu_baseline:
        from oracle.ffi import Oracle
        oracle = Oracle()
        nodes, idx = ctx.bvh_export()
        sub = min(n, 200_000)
        ref, _, _ = oracle.trace_closest(desc.triangles, nodes, idx, rays[:sub])
        out["parity_subset"] = {"rays": sub, "identical": bool(ref.tobytes() == hits[:sub].tobytes())}
        cores = os.cpu_count() or 1
        csub = min(n, 2_000_000)
        try:
            from oracle.ffi import Reference, reference_available
            if not reference_available():
                raise RuntimeError("reference sources not staged")
            world = Reference(variant="fast").world(desc.triangles)  # BVHNode::build on the host
            _, cs = world.trace_closest(rays[:csub], threads=cores)
            world.close()
            kind, what = "reference", "BVHNode::traverse of the reference (-O3) on its own BVH"
        except Exception:  # noqa: BLE001
            t1 = time.perf_counter()
            oracle.trace_closest_mt(desc.triangles, nodes, idx, rays[:csub], cores)
            cs = time.perf_counter() - t1
            kind, what = "port", "the oracle's restatement of BVHNode::traverse on the same tree"
        out["cpu_baseline"] = {"value": csub / cs / 1e6, "unit": "Mrays/s", "cores": cores, "kind": kind,
                               "sample": f"{csub} of the rays through {what}"}
    ctx.close()
    return out


def run_reference(args) -> dict:
    from oracle.ffi import Reference, reference_available
    desc, _, wl = make_workload(args.workload)
    if not reference_available():
        return {"impl": "reference", "unavailable": "reference sources not staged on this machine"}
    ref = Reference(variant="plain_fast")
    cores = os.cpu_count() or 1
    rs = ref.scene(desc, threads=cores)
    if args.warmup:
        rs.render_native(args.warmup)
    rays = 0
    secs = 0.0
    for _ in range(args.steps):
        _, _, r, s = rs.render_native(1)
        rays += r
        secs += s
    rs.close()
    value = rays / secs / 1e6
    return {
        "impl": "reference",
        "metric": "Mrays/s",
        "value": value,
        "unit": "Mrays/s",
        "n_gpus": 1,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": secs * 1e3 / max(args.steps, 1),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic (seeded procedural scene)",
        "config": {"workload": wl + " (reference: its fixed depth 8)", "mode": "plain"},
        "cpu_baseline": {"value": value, "unit": "Mrays/s", "cores": cores, "kind": "reference",
                         "sample": f"{args.steps} frame(s) of RayTracer::render (plain build, -O3)"},
        "e2e": {"value": value, "unit": "Mrays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["pgx", "reference"], default="pgx")
    ap.add_argument("--mode", choices=["plain", "guided_quadtree", "guided_mlp"], default="plain")
    ap.add_argument("--workload", choices=["interior", "cornell"], default="interior")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-side-modes", action="store_true", help="skip the guided and depth-8 side measurements")
    ap.add_argument("--no-equal-time", action="store_true", help="skip the reduced equal-time relMSE study")
    ap.add_argument("--no-workloads", action="store_true",
                    help="skip the box, 2M-triangle traversal and adjoint measurements of the default line")
    ap.add_argument("--res", default=None, help="WxH: render the workload at this image size (profiler captures)")
    ap.add_argument("--spp-per-step", type=int, default=32,
                    help="samples per pixel of one step: one pgx_render call, one wavefront")
    ap.add_argument("--study", choices=["relmse", "traversal", "adjoint", "batch"], default=None,
                    help="instead of the throughput line, run the equal-time relMSE study")
    ap.add_argument("--study-res", default="640x360")
    ap.add_argument("--ref-spp", type=int, default=16384)
    ap.add_argument("--plain-spp", type=int, default=1024)
    ap.add_argument("--train-iters", type=int, default=QT_RECIPE["train_iters"])
    ap.add_argument("--train-first", type=int, default=QT_RECIPE["train_first"],
                    help="QuadTree/PSS study: frames of the first (unguided) cache pass; iteration k renders 2^k x as many")
    ap.add_argument("--guide-fraction", type=float, default=None,
                    help="probability of sampling the guide (default: the guide's recipe, 0.7 QuadTree / PSS, "
                         "0.75 learned)")
    ap.add_argument("--qt-region", type=int, default=QT_RECIPE["qt_region"], help="QuadTree guide: records per region")
    ap.add_argument("--qt-refine", type=float, default=0.01, help="QuadTree guide: flux share that splits a cell")
    ap.add_argument("--qt-clamp", type=float, default=QT_RECIPE["qt_clamp"],
                    help="QuadTree guide: flux clamp x median (0: none)")
    ap.add_argument("--qt-uniform", type=float, default=0.2, help="QuadTree guide: uniform share of its samples")
    ap.add_argument("--qt-compensate", type=float, default=0.0, help="QuadTree guide: MIS compensation (0: off)")
    ap.add_argument("--qt-glossy-alpha", type=float, default=QT_RECIPE["qt_glossy_alpha"],
                    help="QuadTree guide: conductors with a smaller GGX alpha are not guided")
    ap.add_argument("--guide", choices=["mlp", "quadtree", "pss"], default="mlp")
    ap.add_argument("--metric", choices=["robust", "plain"], default="robust")
    ap.add_argument("--train-frames", type=int, default=64)
    ap.add_argument("--mlp-lr", type=float, default=5e-3)
    ap.add_argument("--mlp-decay", type=float, default=0.998)
    ap.add_argument("--mlp-steps", type=int, default=4)
    ap.add_argument("--mlp-batch", type=int, default=1 << 18, help="learned guide: radiance samples per Adam step")
    ap.add_argument("--mlp-cache-frames", type=int, default=0,
                    help="learned guide: unguided frames recorded into a QuadTree cache before training (its fallback)")
    ap.add_argument("--mlp-fallback", type=int, default=256,
                    help="learned guide: regions with fewer training samples than this use the QuadTree")
    ap.add_argument("--ref-cache", default=None, help="npy file keeping the converged image between study runs")
    ap.add_argument("--save-images", default=None, help="directory for the study's final plain and guided images")
    ap.add_argument("--guide-depth", type=int, default=0, help="guide the first N bounces only (0: all)")
    ap.add_argument("--study-seed", type=int, default=0, help="relMSE study: offset of the guided renders' seeds")
    ap.add_argument("--mlp-indirect", action="store_true", help="train the learned guide on indirect light only")
    ap.add_argument("--trav-rays", type=int, default=10_000_000)
    ap.add_argument("--fd-params", type=int, default=256)
    ap.add_argument("--diff-grid", type=int, default=1024, help="adjoint study: heightfield vertices per side")
    ap.add_argument("--diff-res", type=int, default=512, help="adjoint study: image width and height")
    ap.add_argument("--diff-spp", type=int, default=64, help="adjoint study: samples per pixel of the loss render")
    ap.add_argument("--batch-scenes", type=int, default=64)
    ap.add_argument("--batch-res", type=int, default=0, help="0: resolutions drawn from {128,256,512,1024}")
    ap.add_argument("--batch-max-tris", type=float, default=2e6)
    args = ap.parse_args()
    if args.guide_fraction is None:
        args.guide_fraction = MLP_RECIPE["guide_fraction"] if args.guide == "mlp" else QT_RECIPE["guide_fraction"]
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if args.gpus != world:
        if rank == 0:
            print(json.dumps({"impl": args.impl, "unavailable": f"--gpus {args.gpus} needs one process per GPU "
                                                                "(torchrun --nproc-per-node N)"}))
        return
    if world > 1 and (args.impl == "reference" or args.study):
        # the reference arm and the studies run on rank 0 alone
        if rank != 0:
            return
    if args.warmup < 0 or args.steps < 1:
        raise SystemExit("--steps must be >= 1 and --warmup >= 0")
    if args.study == "relmse":
        print(json.dumps(run_relmse_study(args)))
        return
    if args.study == "traversal":
        print(json.dumps(run_traversal_study(args)))
        return
    if args.study == "adjoint":
        print(json.dumps(run_adjoint_study(args)))
        return
    if args.study == "batch":
        print(json.dumps(run_batch_study(args)))
        return
    out = run_reference(args) if args.impl == "reference" else run_pgx(args)
    if out is not None:
        print(json.dumps(out))


if __name__ == "__main__":
    main()
