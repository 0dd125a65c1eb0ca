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
    "c1": dict(config=1, width=1024, height=1024, spp=64, depth=12, triangles=1310732,
               name="c1_icosphere_1310720tri_1024x1024_64spp_depth12"),
    "c0": dict(config=0, width=256, height=256, spp=16, depth=8, triangles=36,
               name="c0_cornell_36tri_256x256_16spp_depth8"),
    "c2": dict(config=2, width=2048, height=2048, spp=32, depth=8, triangles=15127922,
               name="c2_lattice_4096meshes_15127922tri_256mat_64tex_hdri_2048x2048_32spp_depth8"),
}
METRIC = "Mrays/s (closest-hit + shadow rays) at equal MSE vs FP64 oracle"

# Algorithmic bytes per unit of work (the fixed per-unit model of the path):
# per closest-hit ray the compulsory inter-kernel state it moves — ray state
# written and read (2 x 48 B), hit record written and read (2 x 20 B) and the
# accumulator read-modify-write of an emission or miss (24 B): 160 B; per
# shadow ray 2 x 44 B + 24 B = 112 B.  BVH and triangle fetches depend on the
# scene and are excluded (ncu's DRAM bytes are reported beside as `traffic`).
# The roofline of the dominant kernel (k_trace_render, the closest-hit
# traversal) is 160 B x its rays / its measured time; the whole step's figure
# applies both per-unit numbers to the step time.
PIPE_BYTES_CLOSEST = 160
PIPE_BYTES_SHADOW = 112
# The closest-hit kernel's own reads and writes per ray (a narrower model,
# reported beside): origin + direction read (24 B); a hit writes its record
# (ray index, leaf triangle, t, u, v: 20 B); a miss reads throughput + pixel
# (16 B) and read-modify-writes its pixel's RGB sum (24 B).
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


_CPU_SCENES: dict = {}

# The CPU legs (the GPU arm's cpu_baseline and --impl reference) time the same
# bounded sample of the workload: a centred band of REF_ROWS rows of the full
# image at REF_SPP samples per pixel.
REF_ROWS = 256
REF_SPP = 16


def _oracle():
    """The CPU oracle (oracle/oracle.py): the reference's loop restated in C++,
    with its own copy of the procedural scene generator; it loads no GPU
    library."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle

    return oracle


def cpu_sample(wl, threads: int, rows: int, spp: int, seed: int):
    """The oracle port over a centred band of the workload (rank 0 only).
    The scene and the port's BVH are built once per workload, untimed."""
    oracle = _oracle()
    if wl["config"] not in _CPU_SCENES:
        sc = oracle.HostScene(wl["config"])
        _CPU_SCENES[wl["config"]] = (sc, oracle.Port(sc.desc))
    scene, port = _CPU_SCENES[wl["config"]]
    W, H = wl["width"], wl["height"]
    cam = scene.camera(W, H)
    p = oracle.render_params(W, H, spp, wl["depth"], cam, seed=seed)
    y0 = (H - rows) // 2
    t0 = time.perf_counter()
    _, cnt = port.render_window(p, 0, y0, W, rows, threads)
    dt = time.perf_counter() - t0
    rays = cnt["closest_rays"] + cnt["shadow_rays"]
    return rays, dt, (f"{W}x{rows} px centre band x {spp} spp of {wl['name']} ({W * rows * spp} paths); "
                      f"the oracle port of the reference loop on {threads} host threads")


def workload_config(wl, args, world: int) -> dict:
    """The `config` object of both arms' lines (identical by construction)."""
    W, H = wl["width"], wl["height"]
    wave_paths = W * H * min(wl["spp"], max(1, (1 << 27) // (W * H)))
    return {"workload": wl["name"], "policy": args.policy, "ray_sort": bool(args.ray_sort),
            "env_nee": bool(args.env_nee), "adaptive": bool(args.adaptive), "cost_aware_rr": bool(args.cost_rr),
            "triangles": wl["triangles"],
            "l2": f"inputs larger than L2 (ray queues {wave_paths * 112 / 1e9:.1f} GB per wave; "
                  f"BVH + triangles {wl['triangles'] * 68 / 1e6:.0f} MB)",
            "parallelism": f"replicas x{world}"}


def run_reference(args, wl):
    world, rank, local, dist = dist_init()
    if rank != 0:
        return 0
    threads = os.cpu_count() or 1
    rows, spp = args.ref_rows, args.ref_spp
    for _ in range(args.warmup):
        cpu_sample(wl, threads, rows, spp, seed=17)
    total_rays, total_s = 0, 0.0
    sample = ""
    for k in range(args.steps):
        rays, dt, sample = cpu_sample(wl, threads, rows, spp, seed=100 + k)
        total_rays += rays
        total_s += dt
    value = total_rays / total_s / 1e6
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "Mrays/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000 * total_s / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": workload_config(wl, args, world),
        "cpu_baseline": {"value": value, "unit": "Mrays/s", "cores": threads, "kind": "port",
                         "sample": sample + " (Embree and TBB, which the reference's own build needs, are absent "
                                            "on the GPU host)"},
        "e2e": {"value": value, "unit": "Mrays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def image_mse(img, wl, spp):
    """MSE of the fixture window of a rendered image against the reference's
    FP64 mean of that window (tests/golden/c<config>_fp64_crop.npz), and what
    the per-sample variance predicts for it: sigma^2 (1/spp + 1/oracle_spp)."""
    p = ROOT / "tests" / "golden" / f"c{wl['config']}_fp64_crop.npz"
    if not p.exists():
        return None
    g = np.load(p)
    if tuple(int(v) for v in g["image_size"]) != (wl["width"], wl["height"]) or int(g["max_depth"]) != wl["depth"]:
        return None
    x0, y0, w, h = (int(v) for v in g["window"])
    win = img[y0:y0 + h, x0:x0 + w].astype(np.float64)
    mean = g["mean"].astype(np.float64)
    exp = float((g["sigma"].astype(np.float64) ** 2 * (1.0 / spp + 1.0 / float(g["spp"]))).mean())
    mse = float(((win - mean) ** 2).mean())
    return {"value": mse, "expected": exp, "ratio": mse / exp, "window": [x0, y0, w, h], "spp": spp,
            "oracle": f"the reference's renderScene, FP64 mean over {int(g['spp'])} spp of the window",
            "image": "the last end-to-end step's image"}


def percentile(xs, q):
    return float(np.percentile(np.asarray(xs, dtype=np.float64), q)) if len(xs) else None


def c3_jobs(pkg, ctx, n, seed):
    """Config 3: n seeded variants of the Cornell box, each its own resident
    scene, resolution from {64^2, 128^2, 256^2}, spp from {4, 16, 64}, depth 8."""
    rng = np.random.default_rng(seed)
    jobs = []
    for k in range(n):
        hs = pkg.HostScene(3, seed=k)
        sid = ctx.add_scene(hs.desc)
        res = int(rng.choice([64, 128, 256]))
        spp = int(rng.choice([4, 16, 64]))
        jobs.append(pkg.make_job(sid, res, res, spp, 8, hs.camera(res, res), seed=10_000 + k))
    return jobs


def batched_block(pkg, ctx, n_jobs: int, trace_variant: int) -> dict:
    """Config 3: n_jobs jobs rendered in one call (all jobs' rays share
    waves, the bounce chain replays a captured CUDA graph) against the plain
    loop: each job rendered alone, its bounces issued back to back with
    device-side counts (the single-job render's form; no graph).  Also the
    jobs one at a time with graph replay, for reference."""
    tv = max(trace_variant, 0)
    jobs = c3_jobs(pkg, ctx, n_jobs, seed=2026)
    paths = sum(j.width * j.height * j.samples_per_pixel for j in jobs)

    def one_by_one(graph_mode):
        ctx.set_tuning(tv, graph_mode=graph_mode)
        ctx.timer_begin()
        rays = 0
        for j in jobs:
            _, st = ctx.render_batch([j], want_images=False)
            rays += st["closest_rays"] + st["shadow_rays"]
        return rays, ctx.timer_end()

    # warm-up: both single-job forms and the batched graph capture
    for gm in (2, 0):
        ctx.set_tuning(tv, graph_mode=gm)
        for j in jobs[:8]:
            ctx.render_batch([j], want_images=False)
    ctx.set_tuning(tv, graph_mode=0)
    ctx.render_batch(jobs[:32], want_images=False)
    plain_rays, plain_ms = one_by_one(2)
    graph_rays, graph_ms = one_by_one(0)
    ctx.set_tuning(tv, graph_mode=0)
    ctx.timer_begin()
    _, st = ctx.render_batch(jobs, want_images=False)
    ms = ctx.timer_end()
    ctx.set_tuning(tv)
    rays = st["closest_rays"] + st["shadow_rays"]
    value = rays / ms / 1e3
    plain = plain_rays / plain_ms / 1e3
    return {"workload": f"c3_batched_{len(jobs)}_jobs_cornell_variants_64-256px_4-64spp_depth8",
            "value": value, "unit": "Mrays/s", "ms": ms, "paths": paths, "waves": st["waves"],
            "samples_per_s": paths / (ms / 1e3), "gpu_launches": st["kernel_launches"],
            "form": "all jobs in shared waves, bounce chain replayed from a CUDA graph",
            "plain_loop": {"value": plain, "unit": "Mrays/s", "ms": plain_ms,
                           "form": "one job per render, bounces issued back to back with device-side counts"},
            "one_job_per_call_graph_replay": {"value": graph_rays / graph_ms / 1e3, "unit": "Mrays/s",
                                              "ms": graph_ms},
            "speedup_vs_plain_loop": value / plain}


def run_batched(args) -> int:
    world, rank, local, dist = dist_init()
    pkg = load_pkg()
    ctx = pkg.Context(local)
    b = batched_block(pkg, ctx, args.jobs, args.trace_variant)
    line = {
        "metric": METRIC, "value": b["value"], "unit": "Mrays/s", "n_gpus": world, "steps": 1, "warmup": 1,
        "ms_per_step": b["ms"], "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic", "config": {"workload": b["workload"], "paths": b["paths"], "form": b["form"]},
        "plain_loop": b["plain_loop"], "speedup_vs_plain_loop": b["speedup_vs_plain_loop"],
        "samples_per_s": b["samples_per_s"], "waves": b["waves"], "gpu_launches": b["gpu_launches"],
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    return 0


def _c0_oracle():
    p = ROOT / "tests" / "golden" / "c0_fp64.npz"
    if not p.exists():
        return None
    g = np.load(p)
    return {k: g[k] for k in ("mean", "sigma", "spp")}


def serving_block(pkg, ctx, duration: float, rate: float, budget_gb: float, drain: float,
                  trace_variant: int, wave_paths: int = 0) -> dict:
    """Config 4: Poisson arrivals over resident scenes of configs 0, 1 and
    16 config-3 variants; admission by an HBM budget; progressive frames every
    8 spp.  Time to first frame (TTFF) and to completion (TTC) are taken over
    every submitted job: a job without a frame (or not done) when the run ends
    counts at the end time (censored), and the censored counts are given.
    Jobs on the config-0 scene are 256 x 256 at depth 8, so each has an FP64
    oracle (the reference's 16384-spp mean); their final images give a
    per-job MSE.  Other jobs: resolution log-uniform in [128^2, 1024^2],
    spp from {8, 32, 128}, depth 4-12.  Beside it, the plain loop on the same
    stream: its first jobs rendered one per call, and the same jobs served by
    a fresh server to the end (identical work for both forms)."""
    rng = np.random.default_rng(4242)
    scenes = []
    for cfg in (0, 1):
        hs = pkg.HostScene(cfg)
        scenes.append((ctx.add_scene(hs.desc), hs))
    for k in range(16):
        hs = pkg.HostScene(3, seed=k)
        scenes.append((ctx.add_scene(hs.desc), hs))
    ctx.set_tuning(max(trace_variant, 0))
    srv = pkg.Server(ctx, hbm_budget_bytes=int(budget_gb * (1 << 30)), frame_spp=8, max_paths_per_wave=wave_paths)
    for sid, hs in scenes[:3]:  # warm-up: one small job per scene kind
        srv.submit(pkg.make_job(sid, 64, 64, 8, 8, hs.camera(64, 64), seed=1))
    for _ in range(20):
        if srv.step()["running"] == 0:
            break
    arrivals = []
    t = 0.0
    while t < duration:
        t += rng.exponential(1.0 / rate)
        side = int(round(np.exp(rng.uniform(np.log(128), np.log(1024)))))
        spp = int(rng.choice([8, 32, 128]))
        depth = int(rng.integers(4, 13))
        kind = int(rng.integers(0, 3))
        if kind == 0:
            side, depth = 256, 8
        sid, hs = scenes[kind] if kind < 2 else scenes[2 + int(rng.integers(0, 16))]
        arrivals.append((t, kind, pkg.make_job(sid, side, side, spp, depth, hs.camera(side, side),
                                               seed=int(rng.integers(1, 2**31)))))
    ids, kinds = [], []
    rays, dev_ms = 0, 0.0
    base = srv.clock()
    k = 0
    terminal = (pkg.JOB_DONE, pkg.JOB_REJECTED, pkg.JOB_CANCELLED)
    while True:
        now = srv.clock() - base
        while k < len(arrivals) and arrivals[k][0] <= now:
            ids.append(srv.submit(arrivals[k][2]))
            kinds.append(arrivals[k][1])
            k += 1
        if now > duration:
            if now > duration + drain or all(srv.status(i)["state"] in terminal for i in ids):
                break
        info = srv.step()
        rays += info["rays_traced"]
        dev_ms += info["step_ms"]
    wall = srv.clock() - base
    t_end = base + wall
    st = [srv.status(i) for i in ids]
    ttff = [(s["t_first_frame"] if s["t_first_frame"] >= 0 else t_end) - s["t_submit"] for s in st]
    ttc = [(s["t_done"] if s["state"] == pkg.JOB_DONE else t_end) - s["t_submit"] for s in st]
    done_ttc = [s["t_done"] - s["t_submit"] for s in st if s["state"] == pkg.JOB_DONE]
    g = _c0_oracle()
    mses = []
    if g is not None:
        for jid, kind, s, arr in zip(ids, kinds, st, arrivals):
            if kind == 0 and s["state"] == pkg.JOB_DONE:
                img = srv.image(jid, 256, 256).astype(np.float64)
                spp = arr[2].samples_per_pixel
                mse = float(((img - g["mean"]) ** 2).mean())
                exp = float((g["sigma"].astype(np.float64) ** 2 * (1.0 / spp + 1.0 / float(g["spp"]))).mean())
                mses.append((mse / exp, spp))
    srv.close()
    # the plain loop on the same stream: the first arrivals rendered one job per
    # call in the fastest single-job form (bounces back to back with
    # device-side counts), up to ~1.5 G paths
    ctx.set_tuning(max(trace_variant, 0), graph_mode=2)
    plain_jobs, plain_paths = [], 0
    for _, _, job in arrivals:
        if plain_paths > 1.5e9 or len(plain_jobs) >= 256:
            break
        plain_jobs.append(job)
        plain_paths += job.width * job.height * job.samples_per_pixel
    ctx.render_batch(plain_jobs[:2], want_images=False)  # warm-up
    ctx.timer_begin()
    plain_rays = 0
    for job in plain_jobs:
        _, pst = ctx.render_batch([job], want_images=False)
        plain_rays += pst["closest_rays"] + pst["shadow_rays"]
    plain_ms = ctx.timer_end()
    ctx.set_tuning(max(trace_variant, 0))
    plain = plain_rays / plain_ms / 1e3
    # the served form on exactly that work: the same jobs submitted at once to
    # a fresh server and served until every one is done
    srv2 = pkg.Server(ctx, hbm_budget_bytes=int(budget_gb * (1 << 30)), frame_spp=8, max_paths_per_wave=wave_paths)
    s_rays, s_dev = 0, 0.0
    t_s = srv2.clock()
    for job in plain_jobs:
        srv2.submit(job)
    while True:
        info = srv2.step()
        s_rays += info["rays_traced"]
        s_dev += info["step_ms"]
        if info["running"] == 0 and info["queued"] == 0:
            break
    s_wall = srv2.clock() - t_s
    srv2.close()
    ratio = [m for m, _ in mses]
    return {
        "workload": "c4_serving_poisson", "rate_per_s": rate, "duration_s": duration, "drain_s": drain,
        "hbm_budget_gb": budget_gb, "frame_spp": 8, "server_wave_paths": wave_paths or "library default",
        "scenes": "config 0 (jobs 256^2, depth 8), config 1 (1.31 M tris), 16 config-3 variants",
        "value": rays / wall / 1e6, "unit": "Mrays/s", "wall_s": wall,
        "device_busy_mrays_per_s": rays / (dev_ms / 1e3) / 1e6 if dev_ms else None,
        "plain_loop": {"value": plain, "unit": "Mrays/s", "jobs": len(plain_jobs), "paths": plain_paths,
                       "form": "the stream's first jobs one per call, bounces back to back with device-side counts"},
        "served_same_jobs": {"value": s_rays / s_wall / 1e6, "unit": "Mrays/s",
                             "device_busy_mrays_per_s": s_rays / (s_dev / 1e3) / 1e6 if s_dev else None,
                             "speedup_vs_plain_loop": (s_rays / s_wall / 1e6) / plain if plain > 0 else None,
                             "form": "the plain loop's jobs submitted at once to a fresh server, served to the end"},
        "submitted": len(ids), "completed": len(done_ttc),
        "with_first_frame": sum(1 for s in st if s["t_first_frame"] >= 0),
        "rejected": sum(1 for s in st if s["state"] == pkg.JOB_REJECTED),
        "censored_ttff": sum(1 for s in st if s["t_first_frame"] < 0),
        "censored_ttc": sum(1 for s in st if s["state"] != pkg.JOB_DONE),
        "ttff_s": {"p50": percentile(ttff, 50), "p99": percentile(ttff, 99),
                   "over": "all submitted jobs; jobs without a frame count at the end time"},
        "ttc_s": {"p50": percentile(ttc, 50), "p99": percentile(ttc, 99),
                  "over": "all submitted jobs; unfinished jobs count at the end time"},
        "ttc_completed_only_s": {"p50": percentile(done_ttc, 50), "p99": percentile(done_ttc, 99)},
        "c0_job_mse": {"jobs": len(mses),
                       "mse_over_expected_median": float(np.median(ratio)) if ratio else None,
                       "mse_over_expected_max": float(np.max(ratio)) if ratio else None,
                       "oracle": "the reference's 16384-spp FP64 mean of config 0 at 256^2 (tests/golden/c0_fp64.npz)",
                       "expected": "sigma^2 (1/spp + 1/16384) per pixel, from the oracle's per-sample variance"},
    }


def run_serving(args) -> int:
    world, rank, local, dist = dist_init()
    pkg = load_pkg()
    ctx = pkg.Context(local)
    b = serving_block(pkg, ctx, args.duration, args.rate, args.budget_gb, args.drain, args.trace_variant,
                      args.server_wave_paths)
    line = {
        "metric": METRIC, "value": b["value"], "unit": "Mrays/s", "n_gpus": world, "steps": 1,
        "warmup": 1, "ms_per_step": b["wall_s"] * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {k: b[k] for k in ("workload", "rate_per_s", "duration_s", "drain_s", "hbm_budget_gb",
                                     "frame_spp", "scenes")},
        **{k: v for k, v in b.items() if k not in ("value", "unit", "workload", "rate_per_s", "duration_s",
                                                   "drain_s", "hbm_budget_gb", "frame_spp", "scenes")},
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    return 0


def main() -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="c1", choices=sorted(WORKLOADS) + ["c3", "c4"])
    ap.add_argument("--jobs", type=int, default=512, help="config 3: number of jobs")
    ap.add_argument("--duration", type=float, default=20.0, help="config 4: seconds of arrivals")
    ap.add_argument("--rate", type=float, default=200.0, help="config 4: arrivals per second")
    ap.add_argument("--budget-gb", type=float, default=60.0, help="config 4: HBM budget")
    ap.add_argument("--server-wave-paths", type=int, default=0,
                    help="config 4: paths per served wave (0 = the library's default)")
    ap.add_argument("--drain", type=float, default=0.0,
                    help="config 4: seconds to keep serving after the last arrival until all jobs are done")
    ap.add_argument("--policy", default="none", choices=["none", "material", "texture", "costBenefit"])
    ap.add_argument("--ray-sort", type=int, default=0)
    ap.add_argument("--env-nee", type=int, default=0, help="environment NEE + MIS (same mean, lower variance)")
    ap.add_argument("--spp-per-wave", type=int, default=0)
    ap.add_argument("--spp", type=int, default=0, help="override the workload's spp (profiling runs only)")
    ap.add_argument("--res", type=int, default=0, help="override the workload's resolution (profiling runs only)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--trace-variant", type=int, default=-1)
    ap.add_argument("--blocks-per-sm", type=int, default=0)
    ap.add_argument("--ref-rows", type=int, default=REF_ROWS, help="CPU legs: rows of the timed band")
    ap.add_argument("--ref-spp", type=int, default=REF_SPP, help="CPU legs: samples per pixel of the timed band")
    ap.add_argument("--bvh", default="ploc", choices=["ploc", "lbvh", "ploc4", "ploc_sah"])
    ap.add_argument("--autotune", type=int, default=0, help="run wf_autotune on the workload before timing")
    ap.add_argument("--adaptive", type=int, default=0, help="the reference's adaptive sampling (threshold 0.05)")
    ap.add_argument("--ray-sort-bits", type=int, default=0, help="key bits of the loop's ray sort (0 = 33)")
    ap.add_argument("--cost-rr", type=int, default=0, help="cost-aware RR fed by the live device CostTracker")
    ap.add_argument("--batched-jobs", type=int, default=512,
                    help="config-3 jobs of the batched block of the default line (0 = skip)")
    ap.add_argument("--serve-seconds", type=float, default=10.0,
                    help="seconds of config-4 arrivals in the serving block of the default line (0 = skip)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 0)
    if args.impl == "reference" and args.workload in ("c3", "c4"):
        print(json.dumps({"impl": "reference", "unavailable": "the reference has no batched or served form: its "
                          "loop renders one scene per call (src/render/WavefrontRenderer.cpp:94-399)"}), flush=True)
        return 0
    if args.workload == "c3":
        return run_batched(args)
    if args.workload == "c4":
        return run_serving(args)
    wl = dict(WORKLOADS[args.workload])
    if args.spp > 0:
        wl["spp"] = args.spp
        wl["name"] = wl["name"].replace(f"_{WORKLOADS[args.workload]['spp']}spp", f"_{args.spp}spp")
    if args.res > 0:
        r0 = WORKLOADS[args.workload]["width"]
        wl["width"] = wl["height"] = args.res
        wl["name"] = wl["name"].replace(f"_{r0}x{r0}_", f"_{args.res}x{args.res}_")
    if args.impl == "reference":
        return run_reference(args, wl)

    world, rank, local, dist = dist_init()
    pkg = load_pkg()
    ctx = pkg.Context(local)
    scene = pkg.HostScene(wl["config"])
    ctx.set_tuning(max(args.trace_variant, 0), args.blocks_per_sm,
                   bvh_builder={"ploc": 0, "lbvh": 1, "ploc4": 3, "ploc_sah": 4}[args.bvh],
                   ray_sort_bits=args.ray_sort_bits)
    info = ctx.upload(scene.desc)
    W, H = wl["width"], wl["height"]
    cam = scene.camera(W, H)
    policy = pkg.POLICIES[args.policy]

    def params(seed):
        return pkg.render_params(W, H, wl["spp"], wl["depth"], cam, policy=policy, ray_sort=bool(args.ray_sort),
                                 seed=seed, spp_per_wave=args.spp_per_wave, env_nee=bool(args.env_nee),
                                 adaptive=bool(args.adaptive), cost_aware_rr=bool(args.cost_rr),
                                 cost_tracking=bool(args.cost_rr))

    tune_ms = None
    if args.autotune:
        _, tune_ms = ctx.autotune(params(999))
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
    if args.adaptive:  # pixels stop early: the last step's per-pixel counts stand for every step
        samples_all = world * args.steps * int(ctx.sample_counts(W, H).sum())

    # ---- end to end through the C ABI with host buffers ----
    # the image comes back into page-locked host memory (wf_host_alloc)
    image_host = pkg.host_array(W * H * 3)
    barrier(dist)
    e2e_rays = 0
    t0 = time.perf_counter()
    for k in range(args.steps):
        _, st = ctx.render(params(rank * 100000 + 50000 + k), out=image_host)
        e2e_rays += st["closest_rays"] + st["shadow_rays"]
    e2e_s = allreduce_max(dist, time.perf_counter() - t0)
    e2e_value = allreduce_sum(dist, e2e_rays) / e2e_s / 1e6
    mse = image_mse(np.asarray(image_host).reshape(H, W, 3), wl, wl["spp"])

    # ---- roofline of the closest-hit kernel ----
    closest = sum(s["closest_rays"] for s in stats)
    hits = sum(s["shaded_hits"] for s in stats)
    misses = sum(s["misses"] for s in stats)
    trace_ms = sum(s["ms_intersect"] for s in stats)
    launches = sum(s["bounces"] for s in stats)
    alg_bytes = closest * PIPE_BYTES_CLOSEST
    achieved = alg_bytes / (trace_ms / 1e3) / 1e9
    io_bytes = closest * BYTES_RAY + hits * BYTES_HIT + misses * BYTES_MISS
    io_achieved = io_bytes / (trace_ms / 1e3) / 1e9
    shadow = sum(s["shadow_rays"] for s in stats)
    step_ms = sum(s["ms_total"] for s in stats)
    pipe_achieved = (closest * PIPE_BYTES_CLOSEST + shadow * PIPE_BYTES_SHADOW) / (step_ms / 1e3) / 1e9
    peak, peak_kind = measured_peaks()
    # DRAM bytes per closest-hit ray of k_trace_render, measured by ncu over
    # every launch of a smaller render of the same scene (profiles/) with the
    # default tree (binary PLOC); scaled to this run's average launch by its
    # rays.  Other trees have no measured figure.
    traffic = None
    tp = ROOT / "profiles" / "traffic.json"
    if tp.exists() and info.bvh_builder == 0:
        try:
            per_ray = json.loads(tp.read_text())[f"config{wl['config']}"]["dram_bytes_per_closest_ray"]
            traffic = per_ray * closest / max(launches, 1)
        except (KeyError, ValueError, TypeError):
            traffic = None

    line = {
        "metric": METRIC, "value": value, "unit": "Mrays/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": workload_config(wl, args, world),
        "spp_per_wave": args.spp_per_wave or "auto",
        "samples_per_s": samples_all / (ms_max / 1e3),
        "closest_rays_per_step": stats[0]["closest_rays"], "shadow_rays_per_step": stats[0]["shadow_rays"],
        "stage_ms_per_step": {k: sum(s[k] for s in stats) / args.steps for k in
                              ("ms_intersect", "ms_shade", "ms_schedule", "ms_ray_sort", "ms_total")},
        "roofline": {"bound": "hbm", "kernel": "k_trace_render", "achieved": achieved, "peak": peak,
                     "unit": "GB/s", "frac": achieved / peak, "peak_kind": peak_kind,
                     "traffic": traffic, "launches": launches,
                     "alg_bytes_per_launch": alg_bytes / max(launches, 1),
                     "alg_bytes_per_unit": {"closest_hit_ray": PIPE_BYTES_CLOSEST},
                     "avg_launch_ms": trace_ms / max(launches, 1),
                     "kernel_io_model": {
                         "bytes": "24 B ray read + 20 B hit record or 40 B miss (sky + accumulator)",
                         "bytes_per_launch": io_bytes / max(launches, 1), "achieved": io_achieved,
                         "frac": io_achieved / peak},
                     "pipeline_model": {
                         "bytes_per_closest_ray": PIPE_BYTES_CLOSEST, "bytes_per_shadow_ray": PIPE_BYTES_SHADOW,
                         "achieved": pipe_achieved, "frac": pipe_achieved / peak,
                         "over": "the whole step (all kernels of the bounce loop)"}},
        "e2e": {"value": e2e_value, "unit": "Mrays/s", "h2d_bytes_per_step": 128,
                "d2h_bytes_per_step": W * H * 3 * 4},
        "clocks": clocks,
        "gpu_launches": int(sum(s["kernel_launches"] for s in stats)),
        "bvh_build_ms": info.bvh_build_ms,
        "bvh": {"builder": {0: "ploc", 1: "lbvh", 3: "ploc4", 4: "ploc_sah_leaves"}[info.bvh_builder],
                "nodes": info.bvh_nodes,
                "depth": info.bvh_depth},
        "tuning": dict(ctx.get_tuning(), autotuned=bool(args.autotune), autotune_wave_ms=tune_ms),
    }
    if mse is not None:
        line["mse"] = mse
    # the systems forms beside the plain loop (config 3 batched, config 4
    # served), one GPU, after the timed region of the headline workload
    if world == 1 and args.workload == "c1" and args.policy == "none" and not args.adaptive:
        if args.batched_jobs > 0:
            line["batched"] = batched_block(pkg, ctx, args.batched_jobs, args.trace_variant)
        if args.serve_seconds > 0:
            line["serving"] = serving_block(pkg, ctx, args.serve_seconds, args.rate, args.budget_gb, 0.0,
                                            args.trace_variant)
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        # the same band as --impl reference, repeated for >= 10 s of CPU work
        threads = os.cpu_count() or 1
        rays, dt, k = 0, 0.0, 0
        while dt < 10.0 and k < 16:
            r, t, sample = cpu_sample(wl, threads, args.ref_rows, args.ref_spp, seed=100 + k)
            rays, dt, k = rays + r, dt + t, k + 1
        line["cpu_baseline"] = {"value": rays / dt / 1e6, "unit": "Mrays/s", "cores": threads, "kind": "port",
                                "sample": f"{k} runs of the {sample}"}
    if rank == 0:
        print(json.dumps(line), flush=True)
    ctx.close()
    if dist is not None:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
