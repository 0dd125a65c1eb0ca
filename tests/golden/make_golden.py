"""Generates the golden fixtures of tests/golden from the reference itself.

The reference's own C++ sources, compiled in place with shims
(oracle/_ref/libwfref.so, see oracle/Makefile), produce every fixture here;
the reference checkout must be present (it is not on GPU hosts, which only
read the committed .npz files).

  python tests/golden/make_golden.py small   camera, hits, schedules (seconds)
  python tests/golden/make_golden.py fp64    16384-spp FP64 mean of config 0
                                             (the reference's renderScene,
                                             256 batches x 64 spp; ~1 h on 8
                                             cores, resumable)
  python tests/golden/make_golden.py hits1   dense-mesh scene (config 1):
                                             closest hits and occlusion
  python tests/golden/make_golden.py hits2   lattice scene (config 2), same
  python tests/golden/make_golden.py crop1   FP64 mean of a 128 x 128 window
                                             of the 1024^2 dense-mesh render
                                             (16384 spp, depth 12; ~30 min)
  python tests/golden/make_golden.py crop2   FP64 mean of a 128 x 128 window
                                             of the 2048^2 lattice render
                                             (8192 spp, depth 8, HDRI)
  python tests/golden/make_golden.py fp104   FP64 mean of config 104 (config 0
                                             with a directional light and a
                                             glass box), 128 x 128, 16384 spp

Inputs are seeded; the workload scenes come from the procedural generator
compiled into the oracle (the same source as the GPU library's), fed
identically to the reference.  A window of a W x H render is rendered by the
reference with the camera moved onto that window (Camera's public
topLeftCorner / horizontal / vertical, include/core/Camera.h:8-11), which
gives pixel (x0 + i, y0 + j) of the full image the same ray formula.
"""
from __future__ import annotations

import importlib.util
import sys
import time
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path.insert(0, str(ROOT / "oracle"))
import oracle as O  # noqa: E402

wf = O.wf


def small() -> None:
    scene = O.HostScene(0)
    ref = O.Ref(scene.desc, True)
    # Camera (Camera::Camera) and Camera::getRay on a grid of (u, v)
    cam12 = O.ref_camera([0, 0.275, 0.8], [0, 0.275, 0], [0, 1, 0], 40.0, 256, 256)
    uv = np.stack(np.meshgrid(np.linspace(0, 1, 17, dtype=np.float32), np.linspace(0, 1, 17, dtype=np.float32)), -1).reshape(-1, 2)
    ro, rd = zip(*[O.ref_camera_get_ray(cam12, float(u), float(v)) for u, v in uv])
    np.savez_compressed(HERE / "c0_camera.npz", cam12=cam12, uv=uv, origins=np.array(ro), dirs=np.array(rd))
    # Hits: EmbreeAccelerator::intersect4 mapping over the shimmed BVH, and
    # Scene::hit brute force; both are the reference's code paths.
    rng = np.random.default_rng(20261203)
    n = 8192
    o = rng.uniform([-0.27, 0.01, -0.54], [0.27, 0.54, -0.01], size=(n, 3)).astype(np.float32)
    d = rng.normal(size=(n, 3))
    d = (d / np.linalg.norm(d, axis=1, keepdims=True)).astype(np.float32)
    h4 = ref.trace(o, d, mode=1)
    brute = O.Ref(scene.desc, False).trace(o, d, mode=0)
    np.savez_compressed(HERE / "c0_hits.npz", o=o, d=d, **{f"i4_{k}": v for k, v in h4.items()},
                        **{f"bf_{k}": v for k, v in brute.items()})
    # Occlusion
    maxd = rng.uniform(0.002, 0.8, size=n).astype(np.float32)
    np.savez_compressed(HERE / "c0_occluded.npz", o=o, d=d, maxd=maxd, occluded=ref.occluded(o, d, maxd))
    # RayQueue::schedule
    m = 20000
    ro_ = rng.uniform(-12, 12, size=(m, 3)).astype(np.float32)
    rd_ = rng.normal(size=(m, 3)).astype(np.float32)
    rd_[:200, 1] = 0.0
    ro_[500:800] = ro_[500]
    bmin, bmax = np.array([-10, -10, -10], np.float32), np.array([10, 10, 10], np.float32)
    perm, keys = O.ref_ray_schedule(ro_, rd_, bmin, bmax)
    np.savez_compressed(HERE / "ray_schedule.npz", o=ro_, d=rd_, bmin=bmin, bmax=bmax, perm=perm, keys=keys)
    # ShadingQueue::schedule, four policies, trackers fed with cost samples
    types = [0, 1, 4, 5, 0, 1, 4, 2, 0, 5, 1, 3]
    mats = [wf.WfMaterial(type=t, albedo=(0.5, 0.5, 0.5), roughness=0.3, emission=1.0, ior=1.5,
                          texture_id=(i % 5 if i % 3 else -1)) for i, t in enumerate(types)]
    tex_wh = np.array([[512, 512], [256, 256], [512, 512], [64, 64], [0, 0]], np.int32)
    k = 6000
    mids = rng.integers(0, len(mats), k).astype(np.int32)
    tids = np.array([mats[x].texture_id for x in mids], np.int32)
    tids[rng.random(k) < 0.1] = -1
    thr = rng.uniform(0, 1, size=(k, 3)).astype(np.float32)
    thr[rng.random(k) < 0.2] = 1.0
    pts = rng.uniform(-3, 3, size=(k, 3)).astype(np.float32)
    ms_ids = rng.integers(0, len(mats), 4000).astype(np.int32)
    ms_ns = rng.uniform(10, 50, 4000)
    ts_ids = rng.integers(0, 5, 600).astype(np.int32)
    ts_ns = rng.uniform(5, 9, 600)
    perms = {f"perm_{p}": O.ref_shading_schedule(p, mids, tids, thr, pts, mats, tex_wh, (ms_ids, ms_ns), (ts_ids, ts_ns))
             for p in range(4)}
    rc_mat = O.cost_tracker_relative(len(mats), ms_ids, ms_ns, ref=True)
    rc_tex = O.cost_tracker_relative(5, ts_ids, ts_ns, ref=True)
    mat_arr = np.array([[m.type, *m.albedo, m.roughness, m.emission, m.texture_id, m.ior] for m in mats], np.float64)
    np.savez_compressed(HERE / "shading_schedule.npz", mids=mids, tids=tids, thr=thr, pts=pts, mats=mat_arr,
                        tex_wh=tex_wh, rc_mat=rc_mat, rc_tex=rc_tex, ms_ids=ms_ids, ms_ns=ms_ns, ts_ids=ts_ids,
                        ts_ns=ts_ns, **perms)
    print("small fixtures written")


def fp64(batches: int = 256, spp: int = 64, threads: int = 8) -> None:
    """Per-pixel FP64 mean and per-sample standard deviation of config 0 from
    the reference's renderScene: batch b renders `spp` samples with seed b
    (adaptive sampling and cost-aware RR off, policy none, firefly 10)."""
    W = H = 256
    out = HERE / "c0_fp64.npz"
    scene = O.HostScene(0)
    ref = O.Ref(scene.desc, True)
    cam12 = scene.camera(W, H).as_array()
    s1 = np.zeros((H, W, 3), np.float64)
    s2 = np.zeros((H, W, 3), np.float64)
    done = 0
    part = HERE / "c0_fp64.partial.npz"
    if part.exists():
        z = np.load(part)
        s1, s2, done = z["s1"], z["s2"], int(z["done"])
    t0 = time.time()
    for b in range(done, batches):
        img = ref.render(cam12, W, H, spp, 8, policy=0, ray_sort=False, firefly=10.0, seed=1 + b, threads=threads)
        s1 += img
        s2 += img.astype(np.float64) ** 2
        done = b + 1
        if done % 8 == 0 or done == batches:
            np.savez(part, s1=s1, s2=s2, done=done)
            print(f"batch {done}/{batches} {time.time() - t0:.0f}s", flush=True)
    mean = s1 / done
    var_batch = np.maximum(s2 / done - mean ** 2, 0.0) * done / max(done - 1, 1)
    sigma_sample = np.sqrt(var_batch * spp)  # std of a single-sample estimate
    np.savez_compressed(out, mean=mean.astype(np.float32), sigma=sigma_sample.astype(np.float32),
                        spp=np.int64(done * spp), batches=np.int64(done), batch_spp=np.int64(spp),
                        mean_f64_channel=mean.mean(axis=(0, 1)))
    print("written", out, "spp", done * spp)


def crop_camera(cam12: np.ndarray, W: int, H: int, x0: int, y0: int, w: int, h: int) -> np.ndarray:
    """The camera whose w x h image is pixels [x0, x0 + w) x [y0, y0 + h) of
    the W x H image of `cam12` (origin, topLeftCorner, horizontal, vertical):
    the reference's pixel (x, y) uses u = (x + a) / (W - 1) and
    v = 1 - (y + b) / (H - 1) (src/render/WavefrontRenderer.cpp:401-457)."""
    o, tl, hor, ver = np.asarray(cam12, np.float32).reshape(4, 3)
    tl2 = tl + hor * np.float32(x0 / (W - 1)) + ver * np.float32(1.0 - (y0 + h - 1) / (H - 1))
    return np.concatenate([o, tl2, hor * np.float32((w - 1) / (W - 1)),
                           ver * np.float32((h - 1) / (H - 1))]).astype(np.float32)


def hits(config: int, n: int = 8192, brute_n: int = 128) -> None:
    """Closest hits (EmbreeAccelerator::intersect4 mapping) and occlusion of
    a workload scene from the reference's code: a quarter camera rays through
    random image positions, a quarter secondary rays leaving first hits in
    random directions, a quarter aimed at triangle vertices and a quarter at
    edge midpoints (shared edges) from random points inside the scene bounds.
    `brute_n` of them also through Scene::hit's brute force."""
    scene = O.HostScene(config)
    ref = O.Ref(scene.desc, True)
    rng = np.random.default_rng(20261204 + config)
    W = H = {1: 1024, 2: 2048}[config]
    cam12 = scene.camera(W, H).as_array()
    q = n // 4
    uv = rng.uniform(0, 1, size=(2 * q, 2)).astype(np.float32)
    ro, rd = map(np.array, zip(*[O.ref_camera_get_ray(cam12, float(u), float(v)) for u, v in uv]))
    first = ref.trace(ro[q:], rd[q:], mode=1)
    hitmask = first["prim_id"] >= 0
    pts = np.stack([first["point_x"], first["point_y"], first["point_z"]], 1)
    sd = rng.normal(size=(q, 3))
    sd = (sd / np.linalg.norm(sd, axis=1, keepdims=True)).astype(np.float32)
    so = np.where(hitmask[:, None], pts, ro[q:]).astype(np.float32)
    # rays at vertices and edge midpoints of random triangles
    d = scene.desc
    ni = d.num_indices
    idx = np.ctypeslib.as_array(d.indices, (ni,))
    P = np.stack([np.ctypeslib.as_array(a, (d.num_vertices,)) for a in (d.positions_x, d.positions_y, d.positions_z)], 1)
    bmin, bmax = ref.bounds()
    tri = rng.integers(0, ni // 3, 2 * q)
    corner = rng.integers(0, 3, 2 * q)
    a = P[idx[3 * tri + corner]]
    b = P[idx[3 * tri + (corner + 1) % 3]]
    target = np.concatenate([a[:q], 0.5 * (a[q:] + b[q:])]).astype(np.float32)
    org = rng.uniform(bmin, bmax, size=(2 * q, 3)).astype(np.float32)
    td = target - org
    td = (td / np.linalg.norm(td, axis=1, keepdims=True)).astype(np.float32)
    o = np.concatenate([ro[:q], so, org]).astype(np.float32)
    dd = np.concatenate([rd[:q], sd, td]).astype(np.float32)
    h4 = ref.trace(o, dd, mode=1)
    sel = rng.choice(n, brute_n, replace=False)
    brute = O.Ref(scene.desc, False).trace(o[sel], dd[sel], mode=0)
    for k in ("prim_id", "distance", "material_id"):
        assert np.array_equal(brute[k], h4[k][sel]), k
    np.savez_compressed(HERE / f"c{config}_hits.npz", o=o, d=dd, **{f"i4_{k}": v for k, v in h4.items()})
    # occlusion: maxd below and above the closest hit distance
    t = np.where(h4["prim_id"] >= 0, h4["distance"], 1e3).astype(np.float32)
    maxd = (t * rng.choice([0.5, 0.999, 1.001, 2.0], n)).astype(np.float32)
    occ = ref.occluded(o, dd, maxd)
    np.savez_compressed(HERE / f"c{config}_occluded.npz", o=o, d=dd, maxd=maxd, occluded=occ)
    print(f"config {config}: {int((h4['prim_id'] >= 0).sum())} of {n} rays hit, {int(occ.sum())} occluded")


def fp64_window(name: str, config: int, W: int, H: int, window, depth: int, batches: int, batch_spp: int,
                threads: int = 8) -> None:
    """Per-pixel FP64 mean and per-sample standard deviation of a window of
    the W x H render of `config` from the reference's renderScene: batch b
    renders `batch_spp` samples with seed b (adaptive sampling and cost-aware
    RR off, policy none, firefly 10).  Resumable."""
    x0, y0, w, h = window
    scene = O.HostScene(config)
    ref = O.Ref(scene.desc, True)
    cam12 = crop_camera(scene.camera(W, H).as_array(), W, H, x0, y0, w, h)
    env = O.scene_environment(scene.desc)
    env_path = None
    if env is not None:
        env_path = HERE / f"{name}.env.partial.pfm"
        O.write_pfm(env_path, env)
    out = HERE / f"{name}.npz"
    part = HERE / f"{name}.partial.npz"
    s1 = np.zeros((h, w, 3), np.float64)
    s2 = np.zeros((h, w, 3), np.float64)
    done = 0
    if part.exists():
        z = np.load(part)
        s1, s2, done = z["s1"], z["s2"], int(z["done"])
    t0 = time.time()
    unresolved = 0
    for b in range(done, batches):
        img = ref.render(cam12, w, h, batch_spp, depth, policy=0, ray_sort=False, firefly=10.0, seed=1 + b,
                         threads=threads, env_path=env_path)
        unresolved += O.ref_front_face_stats()[0]
        s1 += img
        s2 += img.astype(np.float64) ** 2
        done = b + 1
        if done % 8 == 0 or done == batches:
            np.savez(part, s1=s1, s2=s2, done=done)
            print(f"{name}: batch {done}/{batches} {time.time() - t0:.0f}s", flush=True)
    assert unresolved == 0, "frontFace of a rebuilt hit record not resolved"
    mean = s1 / done
    var_batch = np.maximum(s2 / done - mean ** 2, 0.0) * done / max(done - 1, 1)
    sigma_sample = np.sqrt(var_batch * batch_spp)
    np.savez_compressed(out, mean=mean.astype(np.float32), sigma=sigma_sample.astype(np.float32),
                        spp=np.int64(done * batch_spp), batches=np.int64(done), batch_spp=np.int64(batch_spp),
                        cam12=cam12, window=np.array(window, np.int64), image_size=np.array([W, H], np.int64),
                        max_depth=np.int64(depth), config=np.int64(config))
    if env_path is not None:
        env_path.unlink()
    print("written", out, "spp", done * batch_spp)


if __name__ == "__main__":
    what = sys.argv[1] if len(sys.argv) > 1 else "small"
    if what == "small":
        small()
    elif what == "fp64":
        fp64(batches=int(sys.argv[2]) if len(sys.argv) > 2 else 256)
    elif what in ("hits1", "hits2"):
        hits(int(what[-1]))
    elif what == "crop1":
        fp64_window("c1_fp64_crop", 1, 1024, 1024, (256, 384, 128, 128), 12, 256, 64)
    elif what == "crop2":
        fp64_window("c2_fp64_crop", 2, 2048, 2048, (960, 1536, 128, 128), 8, 256, 32)
    elif what == "fp104":
        fp64_window("c104_fp64", 104, 128, 128, (0, 0, 128, 128), 8, 256, 64)
    else:
        raise SystemExit(__doc__)
