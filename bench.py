#!/usr/bin/env python3
"""Throughput of the GB300 wavefront path tracer on the dense-mesh workload.

One step = one full render of the dense-mesh scene: a displaced icosphere of
1,310,720 triangles in the 0.55 m Cornell room, 1024 x 1024 pixels, 64 spp,
max depth 12, Russian roulette from depth 3, NEE + MIS, policy none (the
reference's per-bounce loop, src/render/WavefrontRenderer.cpp:94-399).
Inputs (scene, BVH, camera) are resident in HBM; synthetic data.

value  Mrays/s = (closest-hit + shadow rays) / device time of K steps,
       measured with CUDA events on the library's stream (wf_timer_*),
       barrier + synchronize on both sides, max over ranks.
e2e    the same metric through wf_render with host buffers: render
       parameters copied in, the averaged image (12.6 MB) copied out every
       step, wall time.
--impl reference  the reference's loop on the host cores: the CPU oracle port
       (the reference's own C++ needs Embree/TBB, absent on the GPU host) on a
       bounded window of the same workload, all host threads.

Multi-GPU: the path shards by image/sample with no exchange; N > 1 runs N
independent replicas (one per rank, weak scaling).
"""
from __future__ import annotations

import argparse
import importlib.util
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent

WORKLOADS = {
    "c1": dict(config=1, width=1024, height=1024, spp=64, depth=12,
               name="c1_icosphere_1310720tri_1024x1024_64spp_depth12"),
    "c0": dict(config=0, width=256, height=256, spp=16, depth=8,
               name="c0_cornell_36tri_256x256_16spp_depth8"),
}
METRIC = "Mrays/s (closest-hit + shadow rays) at equal MSE vs FP64 oracle"

# Algorithmic bytes of the closest-hit kernel (k_trace_render) per ray:
# read origin + direction (24 B); a hit writes its hit record (ray index,
# leaf triangle, t, u, v: 20 B); a miss reads throughput + pixel (16 B) and
# read-modify-writes its pixel's RGB sum (24 B).  BVH and triangle fetches are
# scene-dependent and excluded (ncu DRAM bytes are reported beside).
BYTES_RAY = 24
BYTES_HIT = 20
BYTES_MISS = 16 + 24


def load_pkg():
    if "wavefront_gb300" in sys.modules:
        return sys.modules["wavefront_gb300"]
    spec = importlib.util.spec_from_file_location("wavefront_gb300", ROOT / "wavefront-renderer_gb300" / "__init__.py")
    mod = importlib.util.module_from_spec(spec)
    sys.modules["wavefront_gb300"] = mod
    spec.loader.exec_module(mod)
    if not mod.LIB_PATH.exists():
        spec_b = importlib.util.spec_from_file_location("wf_build", ROOT / "wavefront-renderer_gb300" / "build.py")
        b = importlib.util.module_from_spec(spec_b)
        spec_b.loader.exec_module(b)
        b.build()
    mod.load_library()
    return mod


def measured_peaks() -> tuple[float, str]:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            return float(json.loads(p.read_text())["hbm_gbs"]), "measured"
        except Exception:
            pass
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines: list[str] = []
        self.t = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return
        self.t = threading.Thread(target=self._read, daemon=True)
        self.t.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.t:
            self.t.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        load = [x for x in sm if x > 0.5 * max(sm)] or sm
        return {"sm_mhz": statistics.median(load), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_init():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("gloo")
        return world, rank, local, dist
    return 1, 0, 0, None


def allreduce_max(dist, x: float) -> float:
    if dist is None:
        return x
    import torch

    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def allreduce_sum(dist, x: float) -> float:
    if dist is None:
        return x
    import torch

    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def barrier(dist):
    if dist is not None:
        dist.barrier()


def cpu_sample(pkg, wl, threads: int, rows: int, spp: int, seed: int):
    """The oracle port over a centred band of the workload (rank 0 only)."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle

    scene = pkg.HostScene(wl["config"])
    port = oracle.Port(scene.desc)
    W, H = wl["width"], wl["height"]
    cam = scene.camera(W, H)
    p = pkg.render_params(W, H, spp, wl["depth"], cam, seed=seed)
    y0 = (H - rows) // 2
    t0 = time.perf_counter()
    _, cnt = port.render_window(p, 0, y0, W, rows, threads)
    dt = time.perf_counter() - t0
    rays = cnt["closest_rays"] + cnt["shadow_rays"]
    return rays, dt, f"{W}x{rows} px centre band x {spp} spp of {wl['name']} ({W * rows * spp} paths)"


def run_reference(args, wl):
    world, rank, local, dist = dist_init()
    if rank != 0:
        return 0
    pkg = load_pkg()
    threads = os.cpu_count() or 1
    rows, spp = args.ref_rows, args.ref_spp
    for _ in range(args.warmup):
        cpu_sample(pkg, wl, threads, rows, spp, seed=17)
    total_rays, total_s = 0, 0.0
    sample = ""
    for k in range(args.steps):
        rays, dt, sample = cpu_sample(pkg, wl, threads, rows, spp, seed=100 + k)
        total_rays += rays
        total_s += dt
    value = total_rays / total_s / 1e6
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "Mrays/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000 * total_s / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": wl["name"], "policy": "none", "sample": sample},
        "cpu_baseline": {"value": value, "unit": "Mrays/s", "cores": threads, "kind": "port",
                         "sample": sample + "; oracle port of the reference loop (Embree/TBB absent on the host)"},
        "e2e": {"value": value, "unit": "Mrays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def main() -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="c1", choices=sorted(WORKLOADS))
    ap.add_argument("--policy", default="none", choices=["none", "material", "texture", "costBenefit"])
    ap.add_argument("--ray-sort", type=int, default=0)
    ap.add_argument("--spp-per-wave", type=int, default=0)
    ap.add_argument("--spp", type=int, default=0, help="override the workload's spp (profiling runs only)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--trace-variant", type=int, default=-1)
    ap.add_argument("--blocks-per-sm", type=int, default=0)
    ap.add_argument("--ref-rows", type=int, default=32)
    ap.add_argument("--ref-spp", type=int, default=8)
    args = ap.parse_args()
    args.warmup = max(args.warmup, 0)
    wl = dict(WORKLOADS[args.workload])
    if args.spp > 0:
        wl["spp"] = args.spp
        wl["name"] = wl["name"].replace(f"_{WORKLOADS[args.workload]['spp']}spp", f"_{args.spp}spp")
    if args.impl == "reference":
        return run_reference(args, wl)

    world, rank, local, dist = dist_init()
    pkg = load_pkg()
    ctx = pkg.Context(local)
    scene = pkg.HostScene(wl["config"])
    info = ctx.upload(scene.desc)
    if args.trace_variant >= 0 or args.blocks_per_sm > 0:
        ctx.set_tuning(max(args.trace_variant, 0), args.blocks_per_sm)
    W, H = wl["width"], wl["height"]
    cam = scene.camera(W, H)
    policy = pkg.POLICIES[args.policy]

    def params(seed):
        return pkg.render_params(W, H, wl["spp"], wl["depth"], cam, policy=policy, ray_sort=bool(args.ray_sort),
                                 seed=seed, spp_per_wave=args.spp_per_wave)

    for w in range(max(args.warmup, 0)):
        ctx.render_device(params(1000 + w))

    # ---- device-resident timed region ----
    sampler = ClockSampler(local)
    sampler.start()
    barrier(dist)
    ctx.timer_begin()
    stats = []
    for k in range(args.steps):
        stats.append(ctx.render_device(params(rank * 100000 + k)))
    ms = ctx.timer_end()
    barrier(dist)
    clocks = sampler.stop()
    ms_max = allreduce_max(dist, ms)
    rays_local = sum(s["closest_rays"] + s["shadow_rays"] for s in stats)
    rays_all = allreduce_sum(dist, rays_local)
    value = rays_all / (ms_max / 1e3) / 1e6
    samples_all = world * args.steps * W * H * wl["spp"]

    # ---- end to end through the C ABI with host buffers ----
    barrier(dist)
    e2e_rays = 0
    t0 = time.perf_counter()
    for k in range(args.steps):
        _, st = ctx.render(params(rank * 100000 + 50000 + k))
        e2e_rays += st["closest_rays"] + st["shadow_rays"]
    e2e_s = allreduce_max(dist, time.perf_counter() - t0)
    e2e_value = allreduce_sum(dist, e2e_rays) / e2e_s / 1e6

    # ---- roofline of the closest-hit kernel ----
    closest = sum(s["closest_rays"] for s in stats)
    hits = sum(s["shaded_hits"] for s in stats)
    misses = sum(s["misses"] for s in stats)
    trace_ms = sum(s["ms_intersect"] for s in stats)
    launches = sum(s["bounces"] for s in stats)
    alg_bytes = closest * BYTES_RAY + hits * BYTES_HIT + misses * BYTES_MISS
    achieved = alg_bytes / (trace_ms / 1e3) / 1e9
    peak, peak_kind = measured_peaks()
    traffic = None
    tp = ROOT / "profiles" / "traffic.json"
    if tp.exists():
        try:
            traffic = json.loads(tp.read_text()).get(wl["name"])
        except Exception:
            traffic = None

    line = {
        "metric": METRIC, "value": value, "unit": "Mrays/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": wl["name"], "policy": args.policy, "ray_sort": bool(args.ray_sort),
                   "triangles": info.num_triangles, "spp_per_wave": args.spp_per_wave or "auto",
                   "l2": "inputs larger than L2 (ray queues ~0.9 GB per wave, BVH+triangles ~130 MB)",
                   "parallelism": f"replicas x{world}"},
        "samples_per_s": samples_all / (ms_max / 1e3),
        "closest_rays_per_step": stats[0]["closest_rays"], "shadow_rays_per_step": stats[0]["shadow_rays"],
        "stage_ms_per_step": {k: sum(s[k] for s in stats) / args.steps for k in
                              ("ms_intersect", "ms_shade", "ms_schedule", "ms_ray_sort", "ms_total")},
        "roofline": {"bound": "hbm", "kernel": "k_trace_render", "achieved": achieved, "peak": peak,
                     "unit": "GB/s", "frac": achieved / peak, "peak_kind": peak_kind,
                     "traffic": traffic, "launches": launches,
                     "alg_bytes_per_launch": alg_bytes / max(launches, 1),
                     "avg_launch_ms": trace_ms / max(launches, 1)},
        "e2e": {"value": e2e_value, "unit": "Mrays/s", "h2d_bytes_per_step": 128,
                "d2h_bytes_per_step": W * H * 3 * 4},
        "clocks": clocks,
        "gpu_launches": int(sum(s["kernel_launches"] for s in stats)),
        "bvh_build_ms": info.bvh_build_ms,
        "tuning": ctx.get_tuning(),
    }
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        rays, dt, sample = cpu_sample(pkg, wl, os.cpu_count() or 1, rows=48, spp=8, seed=7)
        line["cpu_baseline"] = {"value": rays / dt / 1e6, "unit": "Mrays/s", "cores": os.cpu_count() or 1,
                                "kind": "port", "sample": sample}
    if rank == 0:
        print(json.dumps(line), flush=True)
    ctx.close()
    if dist is not None:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
