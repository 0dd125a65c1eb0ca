"""The per-bounce stages on device-resident queues (GPU).

The reference's loop body (WavefrontRenderer::renderScene, src/render/
WavefrontRenderer.cpp:141-268) driven from the host one stage at a time:
generatePrimaryRays, RayQueue::schedule/materialize, intersectAll,
ShadingQueue::schedule/materialize, shadeAll, the occluded() calls and the
miss loop, each a call on queues that stay in device memory.

* The loop renders wf_render's image (same random streams; pixel sums differ
  only by the order of float additions: 1e-4 relative on 99.9% of pixels), and
  its per-bounce counts add up to wf_render's ray, hit and shadow-ray counts.
* Each stage's output equals the entry point that the reference-made fixtures
  pin: the ShadingQueue's columns equal wf_trace_closest_host on the same
  rays; the two schedules' permutations equal wf_ray_schedule_host and
  wf_shading_schedule_host on the same columns.
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import report

pytestmark = pytest.mark.gpu


def _staged_render(wf, ctx, p, *, misses=True, policy=0, ray_sort=False, bounds=None, checks=None):
    W, H, spp = p.width, p.height, p.samples_per_pixel
    cap = W * H * spp
    rays, nxt = wf.RayQueue(ctx, cap), wf.RayQueue(ctx, cap)
    miss_q = wf.RayQueue(ctx, cap) if misses else None
    hits = wf.ShadingQueue(ctx, cap)
    shadows = wf.ShadowQueue(ctx, 3 * cap)
    ctx.stage_begin(p)
    ctx.stage_generate_primary(0, spp, rays)
    counts = []
    try:
        for depth in range(p.max_depth):
            n = rays.size()
            if n == 0:
                break
            if ray_sort:
                perm = rays.schedule(*bounds)
                if checks is not None and depth == 1:
                    checks["ray_schedule"] = (rays.download(), perm)
                rays.materialize()
            ctx.intersect(rays, hits, miss_q)
            if checks is not None and depth == 1:
                checks["hits"] = (rays.download(), hits.download())
            if policy:
                perm = hits.schedule(policy)
                if checks is not None and depth == 1:
                    checks["shading_schedule"] = (hits.download(), perm)
                hits.materialize()
            ctx.shade(hits, nxt, shadows)
            ctx.occluded(shadows)
            if miss_q is not None:
                ctx.miss(miss_q)
            counts.append((n, hits.size(), shadows.size(), miss_q.size() if miss_q else n - hits.size()))
            rays, nxt = nxt, rays
        img = ctx.stage_image()
    finally:
        for q in (rays, nxt, miss_q, hits, shadows):
            if q is not None:
                q.close()
    return img, counts


@pytest.mark.parametrize("which", ["c0", "c2small"])
@pytest.mark.parametrize("misses", [True, False])
def test_stages_render_the_loops_image(wf, ctx, scene0, scene_c2small, which, misses):
    scene = scene0 if which == "c0" else scene_c2small
    ctx.upload(scene.desc)
    W = H = 48
    p = wf.render_params(W, H, 8, 8, scene.camera(W, H), seed=5)
    img, counts = _staged_render(wf, ctx, p, misses=misses)
    ref, st = ctx.render(p)
    agree = np.isclose(img, ref, rtol=1e-4, atol=1e-6).all(axis=2).mean()
    rays = sum(c[0] for c in counts)
    hits = sum(c[1] for c in counts)
    shadow = sum(c[2] for c in counts)
    report(f"stages_{which}_misses{int(misses)}", agree=float(agree), bounces=len(counts), rays=rays,
           render_rays=st["closest_rays"], hits=hits, render_hits=st["shaded_hits"], shadow=shadow,
           render_shadow=st["shadow_rays"])
    assert agree >= 0.999, agree
    assert rays == st["closest_rays"] and hits == st["shaded_hits"] and shadow == st["shadow_rays"]
    assert all(c[0] == c[1] + c[3] for c in counts)  # every ray either hit or missed


def test_stage_outputs_equal_the_pinned_entry_points(wf, ctx, scene_c2small):
    """Bounce 1 of a render with the ray sort and the material policy: the
    queues' contents against the host entry points on the same columns."""
    sc = scene_c2small
    info = ctx.upload(sc.desc)
    W = H = 32
    p = wf.render_params(W, H, 8, 8, sc.camera(W, H), seed=11)
    bounds = (np.array(info.bounds_min, np.float32), np.array(info.bounds_max, np.float32))
    checks: dict = {}
    img, counts = _staged_render(wf, ctx, p, policy=wf.POLICY_MATERIAL, ray_sort=True, bounds=bounds,
                                 checks=checks)
    ref, st = ctx.render(p)
    assert np.isclose(img, ref, rtol=1e-4, atol=1e-6).all(axis=2).mean() >= 0.999
    # RayQueue::schedule on the device queue == wf_ray_schedule_host
    rq, perm = checks["ray_schedule"]
    o = np.stack([rq["origins_x"], rq["origins_y"], rq["origins_z"]], 1)
    d = np.stack([rq["dirs_x"], rq["dirs_y"], rq["dirs_z"]], 1)
    want, _ = ctx.ray_schedule(o, d, *bounds)
    assert np.array_equal(perm, want)
    # intersectAll: the ShadingQueue's hits == wf_trace_closest_host of the rays that hit
    rq, (hcols, hrays) = checks["hits"]
    o = np.stack([rq["origins_x"], rq["origins_y"], rq["origins_z"]], 1)
    d = np.stack([rq["dirs_x"], rq["dirs_y"], rq["dirs_z"]], 1)
    full = ctx.trace_closest(o, d)
    hit_rays = np.nonzero(full["prim_id"] >= 0)[0]
    assert len(hit_rays) == len(hcols["prim_id"])
    order = np.lexsort((hrays["sample_indices"], hrays["pixel_indices"]))
    ref_order = np.lexsort((rq["sample_indices"][hit_rays], rq["pixel_indices"][hit_rays]))
    for k in ("geom_id", "prim_id", "distance", "point_x", "point_y", "point_z", "normal_x", "normal_y", "normal_z",
              "front_face", "u", "v", "material_id", "texture_id"):
        assert np.array_equal(hcols[k][order], full[k][hit_rays][ref_order]), k
    # ShadingQueue::schedule (MaterialAware) == wf_shading_schedule_host on its columns
    (hc, hr), perm = checks["shading_schedule"]
    mats = [sc.desc.materials[i] for i in range(sc.desc.num_materials)]
    tex_bytes = np.array([sc.desc.textures[t].width * sc.desc.textures[t].height * 12
                          for t in range(sc.desc.num_textures)], np.int64)
    thr = np.stack([hr["throughputs_r"], hr["throughputs_g"], hr["throughputs_b"]], 1)
    pts = np.stack([hc["point_x"], hc["point_y"], hc["point_z"]], 1)
    want = ctx.shading_schedule(wf.POLICY_MATERIAL, hc["material_id"], hc["texture_id"], thr, pts, mats, tex_bytes)
    assert np.array_equal(perm, want)
    report("stage_outputs", bounce1_rays=int(len(o)), bounce1_hits=int(len(hit_rays)))
