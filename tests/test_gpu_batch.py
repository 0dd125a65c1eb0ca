"""Batched jobs (config 3) and the serving loop (config 4) on the GPU.

A job's random streams are keyed by its own seed and (pixel, sample, depth),
so the paths it traces do not depend on which other jobs share its waves; only
the order of the float additions into its pixels does (atomics).  Tolerance:
the image of a job in a mix equals its image alone within 1e-4 relative +
1e-6 absolute on at least 99.9% of pixels.
"""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RES = [(24, 16), (32, 32), (48, 40), (64, 64)]


def _jobs(wf, ctx, n, seed0=100, scenes=None):
    """n config-3 jobs on their own resident scene variants."""
    jobs, hosts = [], []
    rng = np.random.default_rng(seed0)
    for k in range(n):
        hs = wf.HostScene(3, seed=seed0 + k)
        sid = ctx.add_scene(hs.desc)
        w, h = RES[k % len(RES)]
        spp = int(rng.choice([2, 4, 8]))
        cam = hs.camera(w, h)
        jobs.append(wf.make_job(sid, w, h, spp, 8, cam, seed=7000 + k))
        hosts.append(hs)
    return jobs, hosts


def _same(a, b):
    return np.isclose(a, b, rtol=1e-4, atol=1e-6).all(axis=2).mean()


@pytest.mark.parametrize("variant", [0, 1])
def test_batch_job_equals_job_alone(wf, ctx, variant):
    """Variant 1 runs the multi-job traversal at 9 resident blocks per SM."""
    ctx.set_tuning(trace_variant=variant)
    try:
        jobs, hosts = _jobs(wf, ctx, 12)
        imgs, st = ctx.render_batch(jobs)
    finally:
        ctx.set_tuning()
    assert st["closest_rays"] > 0 and st["waves"] >= 1
    for j, hs, img in zip(jobs, hosts, imgs):
        ctx.upload(hs.desc)  # slot 0: the single-scene path
        alone, _ = ctx.render(wf.render_params(j.width, j.height, j.samples_per_pixel, j.max_depth, j.camera,
                                               seed=j.seed_lo))
        assert _same(img, alone) >= 0.999


def test_batch_with_dense_scene_equals_jobs_alone(wf, ctx):
    """A wave over the dense mesh (1.31 M triangles, tree + triangles above
    16 MB) runs the multi-job traversal at 9 blocks per SM and writes the
    next rays grouped by direction octant; its jobs still equal their images
    rendered alone."""
    from conftest import report

    dense = wf.HostScene(1)
    sid = ctx.add_scene(dense.desc)
    try:
        jobs, hosts = _jobs(wf, ctx, 3, seed0=500)
        jobs.append(wf.make_job(sid, 48, 40, 8, 12, dense.camera(48, 40), seed=9100))
        hosts.append(dense)
        imgs, st = ctx.render_batch(jobs)
        agree = []
        for j, hs, img in zip(jobs, hosts, imgs):
            ctx.upload(hs.desc)
            alone, _ = ctx.render(wf.render_params(j.width, j.height, j.samples_per_pixel, j.max_depth, j.camera,
                                                   seed=j.seed_lo))
            agree.append(float(_same(img, alone)))
        report("batch_dense_scene", agree=agree, rays=st["closest_rays"], waves=st["waves"])
        assert st["closest_rays"] > 0
        assert min(agree) >= 0.999, agree
    finally:
        ctx.remove_scene(sid)


def test_batch_job_matches_oracle(wf, orc, ctx):
    """Jobs of a batch against the port rendering each alone (same random
    streams); the agreement is reported before it is asserted."""
    from conftest import report

    jobs, hosts = _jobs(wf, ctx, 3, seed0=300)
    imgs, _ = ctx.render_batch(jobs)
    for k, (j, hs, img) in enumerate(zip(jobs, hosts, imgs)):
        port = orc.Port(hs.desc)
        p = wf.render_params(j.width, j.height, j.samples_per_pixel, j.max_depth, j.camera, seed=j.seed_lo)
        acc, _ = port.render_window(p, 0, 0, j.width, j.height)
        close = np.isclose(img, acc / j.samples_per_pixel, rtol=1e-3, atol=1e-4).all(axis=2)
        agree = float(close.mean())
        report(f"batch_job{k}_paths", agree=agree, disagreeing_pixels=int((~close).sum()), pixels=int(close.size))
        assert agree >= 0.97


def test_graph_replay_equals_host_loop(wf, ctx, scene_small):
    ctx.upload(scene_small.desc)
    cam = scene_small.camera(48, 48)
    p = wf.render_params(48, 48, 8, 12, cam, seed=11, spp_per_wave=3)
    ctx.set_tuning(graph_mode=2)
    host, st_h = ctx.render(p)
    ctx.set_tuning(graph_mode=1)
    graph, st_g = ctx.render(p)
    ctx.set_tuning()
    assert _same(graph, host) >= 0.999
    assert st_g["closest_rays"] == st_h["closest_rays"]
    assert st_g["shadow_rays"] == st_h["shadow_rays"]


def test_server_progressive_frames_and_final_images(wf, ctx):
    jobs, hosts = _jobs(wf, ctx, 10, seed0=500)
    for j in jobs:
        j.samples_per_pixel = 16
    srv = wf.Server(ctx, hbm_budget_bytes=64 << 20, frame_spp=4, max_paths_per_wave=1 << 16)
    ids = [srv.submit(j) for j in jobs]
    saw_progressive = False
    for _ in range(200):
        info = srv.step()
        assert info["budget_used_bytes"] <= 64 << 20
        for i, j in zip(ids, jobs):
            st = srv.status(i)
            if st["state"] == wf.JOB_RUNNING and 0 < st["samples_done"] < 16:
                srv.image(i, j.width, j.height)  # a progressive frame is readable
                saw_progressive = True
        if info["running"] == 0 and info["queued"] == 0:
            break
    assert saw_progressive
    for i, j, hs in zip(ids, jobs, hosts):
        st = srv.status(i)
        assert st["state"] == wf.JOB_DONE and st["samples_done"] == 16 and st["frames"] == 4
        assert st["t_submit"] <= st["t_admit"] <= st["t_first_frame"] <= st["t_done"]
        final = srv.image(i, j.width, j.height)
        ctx.upload(hs.desc)
        alone, _ = ctx.render(wf.render_params(j.width, j.height, 16, j.max_depth, j.camera, seed=j.seed_lo))
        assert _same(final, alone) >= 0.999
    srv.close()


def test_server_admission_respects_budget(wf, ctx):
    jobs, hosts = _jobs(wf, ctx, 6, seed0=700)
    for j in jobs:
        j.width, j.height, j.samples_per_pixel = 64, 64, 8
    wave = 1 << 14
    # the streaming queue (two RayQueues, a hit queue, the shadow queue), then
    # the sums: two jobs' and the frame share (6 floats per queued path here)
    per_path = 2 * 14 * 4 + 5 * 4 + 3 * 12 * 4
    budget = wave * per_path + 4 * (2 * 64 * 64 * 3 + 6 * wave)
    srv = wf.Server(ctx, hbm_budget_bytes=budget, frame_spp=8, max_paths_per_wave=wave)
    ids = [srv.submit(j) for j in jobs]
    big = wf.make_job(jobs[0].scene_id, 512, 512, 4, 8, jobs[0].camera)
    big_id = srv.submit(big)
    assert srv.status(big_id)["state"] == wf.JOB_REJECTED
    max_running = 0
    for _ in range(100):
        info = srv.step()
        # running: admitted and not yet handed over (a finished job's image is
        # handed over during the next step, its sums freed at the end of this one)
        max_running = max(max_running, info["running"])
        assert info["budget_used_bytes"] <= budget
        if info["running"] == 0 and info["queued"] == 0:
            break
    assert max_running <= 2
    assert all(srv.status(i)["state"] == wf.JOB_DONE for i in ids)
    srv.close()


def test_server_streams_frames_larger_than_its_queue(wf, ctx, scene_small):
    """A job whose frames hold more paths than the streaming queue (64 x 64
    x 4 spp = 16384 paths through a queue of 4096): paths that end are
    replaced by new camera rays bounce by bounce.  Every progressive image is
    the job's first k frames exactly (equal to a render of its first
    k * frame_spp samples, same random streams), and the final image equals
    the job rendered alone."""
    sid = ctx.add_scene(scene_small.desc)
    cam = scene_small.camera(64, 64)
    job = wf.make_job(sid, 64, 64, 16, 8, cam, seed=77)
    srv = wf.Server(ctx, hbm_budget_bytes=64 << 20, frame_spp=4, max_paths_per_wave=4096)
    jid = srv.submit(job)
    seen = {}
    for _ in range(400):
        info = srv.step()
        assert info["paths_in_wave"] <= 8 * 4096
        st = srv.status(jid)
        if st["state"] == wf.JOB_RUNNING and st["samples_done"] > 0 and st["samples_done"] not in seen:
            seen[st["samples_done"]] = srv.image(jid, 64, 64).copy()
        if st["state"] == wf.JOB_DONE:
            break
    st = srv.status(jid)
    assert st["state"] == wf.JOB_DONE and st["frames"] == 4
    assert seen, "no progressive frame observed"
    final = srv.image(jid, 64, 64)
    srv.close()
    ctx.upload(scene_small.desc)
    for spp, img in seen.items():
        ref, _ = ctx.render(wf.render_params(64, 64, spp, 8, cam, seed=77))
        assert _same(img, ref) >= 0.999, spp
    alone, _ = ctx.render(wf.render_params(64, 64, 16, 8, cam, seed=77))
    assert _same(final, alone) >= 0.999


def test_server_mixes_textured_and_plain_scenes(wf, ctx, scene_c2small):
    """A job on a scene with textures and an environment map arrives while
    jobs on plain scenes run: the server's captured step is redone with the
    full shading instance (the lean one, used while no queued scene needs
    them, compiles texture and environment lookups out), and every job equals
    its render alone."""
    jobs, hosts = _jobs(wf, ctx, 3, seed0=1300)
    sid = ctx.add_scene(scene_c2small.desc)
    cam = scene_c2small.camera(40, 32)
    tex_job = wf.make_job(sid, 40, 32, 8, 8, cam, seed=515)
    srv = wf.Server(ctx, hbm_budget_bytes=64 << 20, frame_spp=4, max_paths_per_wave=1 << 14)
    ids = [srv.submit(j) for j in jobs]
    srv.step()
    tid = srv.submit(tex_job)
    for _ in range(200):
        info = srv.step()
        if info["running"] == 0 and info["queued"] == 0:
            break
    assert all(srv.status(i)["state"] == wf.JOB_DONE for i in ids + [tid])
    imgs = [srv.image(i, j.width, j.height) for i, j in zip(ids + [tid], jobs + [tex_job])]
    srv.close()
    for j, hs, img in zip(jobs, hosts, imgs):
        ctx.upload(hs.desc)
        alone, _ = ctx.render(wf.render_params(j.width, j.height, j.samples_per_pixel, j.max_depth, j.camera,
                                               seed=j.seed_lo))
        assert _same(img, alone) >= 0.999
    ctx.upload(scene_c2small.desc)
    alone, _ = ctx.render(wf.render_params(40, 32, 8, 8, cam, seed=515))
    assert _same(imgs[-1], alone) >= 0.999


@pytest.mark.parametrize("ask", ["image", "cancel"])
def test_server_hands_over_a_finished_job_on_request(wf, ctx, ask):
    """After the step in which a job's last frame ends, the job still counts as
    running (its image is being copied out); wf_server_image hands it over at
    once, and wf_server_cancel finds it complete, not cancelled."""
    jobs, hosts = _jobs(wf, ctx, 1, seed0=950)
    j, hs = jobs[0], hosts[0]
    j.samples_per_pixel = 8
    srv = wf.Server(ctx, hbm_budget_bytes=64 << 20, frame_spp=4, max_paths_per_wave=1 << 16)
    try:
        jid = srv.submit(j)
        img = None
        for _ in range(100):
            info = srv.step()
            st = srv.status(jid)
            if st["state"] == wf.JOB_RUNNING and st["samples_done"] == 8:
                if ask == "cancel":
                    srv.cancel(jid)
                img = srv.image(jid, j.width, j.height)
                assert srv.status(jid)["state"] == wf.JOB_DONE
                break
            if info["running"] == 0 and info["queued"] == 0:
                break
        assert img is not None  # the job was seen between its last frame and its hand-over
        ctx.upload(hs.desc)
        alone, _ = ctx.render(wf.render_params(j.width, j.height, 8, j.max_depth, j.camera, seed=j.seed_lo))
        assert _same(img, alone) >= 0.999
    finally:
        srv.close()


def test_server_cancel(wf, ctx):
    jobs, hosts = _jobs(wf, ctx, 3, seed0=900)
    srv = wf.Server(ctx, hbm_budget_bytes=64 << 20, frame_spp=2, max_paths_per_wave=1 << 14)
    ids = [srv.submit(j) for j in jobs]
    srv.step()
    srv.cancel(ids[0])
    for _ in range(50):
        info = srv.step()
        if info["running"] == 0 and info["queued"] == 0:
            break
    assert srv.status(ids[0])["state"] == wf.JOB_CANCELLED
    assert all(srv.status(i)["state"] == wf.JOB_DONE for i in ids[1:])
    srv.close()


def test_batch_env_nee_job_equals_job_alone(wf, ctx, scene_c2small):
    """A job with environment NEE among jobs without it (per-ray job flags)."""
    sid = ctx.add_scene(scene_c2small.desc)
    jobs, hosts = _jobs(wf, ctx, 3, seed0=1100)
    cam = scene_c2small.camera(40, 32)
    nee = wf.make_job(sid, 40, 32, 4, 8, cam, seed=4242, env_nee=True)
    imgs, _ = ctx.render_batch(jobs + [nee])
    ctx.upload(scene_c2small.desc)
    alone, _ = ctx.render(wf.render_params(40, 32, 4, 8, cam, seed=4242, env_nee=True))
    assert _same(imgs[-1], alone) >= 0.999
