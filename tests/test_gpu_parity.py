"""Parity of the CUDA path (through the C ABI) with the CPU oracle.

Integer and index results are compared bit for bit; float results of basic
IEEE arithmetic (camera rays, Moller-Trumbore t, hit points, Morton keys) are
compared bit for bit as well, because the device build uses no fused
multiply-add (-fmad=false).  Rendered images use the same random streams on
both sides, so they agree pixel by pixel except where a transcendental
(cosf, sinf, powf: CUDA's and glibc's differ in the last ulp) nudges a path;
the tolerance for that is written in each test.
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import rays_in_box

pytestmark = pytest.mark.gpu

HIT_KEYS_EXACT = ["prim_id", "material_id", "texture_id", "front_face", "distance", "point_x", "point_y",
                  "point_z", "normal_x", "normal_y", "normal_z", "u", "v"]


def _od(cols):
    o = np.stack([cols["ox"], cols["oy"], cols["oz"]], 1)
    d = np.stack([cols["dx"], cols["dy"], cols["dz"]], 1)
    return o, d


def test_camera_rays_bit_exact(wf, orc, ctx, scene0):
    """generatePrimaryRays + Camera::getRay, same Philox jitter: all columns equal."""
    W, H = 256, 256
    cam = scene0.camera(W, H)
    g = ctx.generate_primary(cam, W, H, seed=0x1234_5678_9ABC, first_sample=5, nspp=2)
    c = orc.generate_primary(cam, W, H, 0x1234_5678_9ABC, 5, 2)
    for k in ("ox", "oy", "oz", "dx", "dy", "dz", "pixel", "sample"):
        assert np.array_equal(g[k], c[k]), k


@pytest.mark.parametrize("which", ["c0", "small", "c2small"])
def test_trace_closest_matches_oracle(wf, orc, ctx, scene0, scene_small, scene_c2small, which):
    scene = {"c0": scene0, "small": scene_small, "c2small": scene_c2small}[which]
    ctx.upload(scene.desc)
    port = orc.Port(scene.desc)
    rng = np.random.default_rng(11)
    cam = scene.camera(128, 128)
    prim = orc.generate_primary(cam, 128, 128, 3, 0, 1)
    o1, d1 = _od(prim)
    if which == "c2small":  # 16 x 16 lattice on the ground plane, meshes below y = 0.9
        o2, d2 = rays_in_box(rng, 50000, [0.0, 0.01, 0.0], [16.0, 0.9, 16.0])
    else:
        o2, d2 = rays_in_box(rng, 50000, [-0.27, 0.01, -0.54], [0.27, 0.54, -0.01])
    o = np.concatenate([o1, o2])
    d = np.concatenate([d1, d2])
    g = ctx.trace_closest(o, d)
    c = port.trace_closest(o, d)
    hit = c["prim_id"] >= 0
    assert hit.mean() > 0.5
    # geomID: the GPU reports it; the oracle's geom id is the mesh index too
    assert np.array_equal(g["geom_id"], c["geom_id"])
    for k in HIT_KEYS_EXACT:
        assert np.array_equal(g[k], c[k]), k  # misses included: ids -1, other columns 0
    assert np.array_equal(g["prim_id"] < 0, ~hit)


def test_trace_closest_equals_brute_force(wf, orc, ctx, scene0):
    """The BVH result equals the reference's brute-force Scene::hit order."""
    ctx.upload(scene0.desc)
    port = orc.Port(scene0.desc)
    rng = np.random.default_rng(5)
    o, d = rays_in_box(rng, 20000, [-0.27, 0.01, -0.54], [0.27, 0.54, -0.01])
    g = ctx.trace_closest(o, d)
    b = port.trace_closest(o, d, brute=True)
    assert np.array_equal(g["prim_id"], b["prim_id"])
    assert np.array_equal(g["geom_id"], b["geom_id"])
    assert np.array_equal(g["distance"], b["distance"])


def test_trace_closest_t_range(wf, orc, ctx, scene0):
    """tmin / tmax cut-offs (EmbreeTest HitBeyondMaxDistanceReturnsFalse)."""
    ctx.upload(scene0.desc)
    port = orc.Port(scene0.desc)
    rng = np.random.default_rng(8)
    o, d = rays_in_box(rng, 4000, [-0.27, 0.01, -0.54], [0.27, 0.54, -0.01])
    for tmin, tmax in [(0.001, 0.05), (0.1, 0.3), (0.0, 1e9)]:
        g = ctx.trace_closest(o, d, tmin, tmax)
        c = port.trace_closest(o, d, tmin, tmax)
        assert np.array_equal(g["prim_id"], c["prim_id"])
        assert np.array_equal(g["distance"], c["distance"])


def test_trace_occluded_matches_oracle(wf, orc, ctx, scene_small):
    ctx.upload(scene_small.desc)
    port = orc.Port(scene_small.desc)
    rng = np.random.default_rng(2)
    o, d = rays_in_box(rng, 40000, [-0.27, 0.01, -0.54], [0.27, 0.54, -0.01])
    maxd = rng.uniform(0.002, 0.8, size=40000).astype(np.float32)
    g = ctx.trace_occluded(o, d, maxd)
    c = port.trace_occluded(o, d, maxd)
    assert np.array_equal(g, c)
    assert 0.05 < g.mean() < 0.95


def test_embree_known_answers_on_gpu(wf, ctx):
    """tests/accelerator/EmbreeTest.cpp cases, run through the GPU."""
    def quad_scene(verts, mats):
        pass

    # single quad at z = -1 (EmbreeTest buildSingleQuadScene)
    px = np.array([-1, 1, 1, -1], np.float32)
    py = np.array([-1, -1, 1, 1], np.float32)
    pz = np.array([-1, -1, -1, -1], np.float32)
    idx = np.array([0, 1, 2, 0, 2, 3], np.int32)
    desc, keep = _desc(wf, [(px, py, pz, idx, 0)], [wf.WfMaterial(type=0, albedo=(0.8, 0.8, 0.8), texture_id=-1)])
    ctx.upload(desc)
    o = np.array([[0, 0, 0], [0, 0, 0], [5, 5, 0]], np.float32)
    d = np.array([[0, 0, -1], [0, 0, 1], [0, 0, -1]], np.float32)
    h = ctx.trace_closest(o, d)
    assert h["prim_id"][0] >= 0 and abs(h["distance"][0] - 1.0) < 1e-3
    assert h["material_id"][0] == 0 and h["normal_z"][0] > 0 and h["front_face"][0] == 1
    assert h["prim_id"][1] == -1 and h["prim_id"][2] == -1
    h = ctx.trace_closest(o[:1], d[:1], 0.001, 0.5)
    assert h["prim_id"][0] == -1
    # nearest of two meshes (MultiMeshSceneHitsCorrectMaterial)
    tri = np.array([0, 1, 2], np.int32)
    A = (np.array([-1, 1, 0], np.float32), np.array([-1, -1, 1], np.float32), np.full(3, -2, np.float32), tri, 0)
    B = (np.array([-1, 1, 0], np.float32), np.array([-1, -1, 1], np.float32), np.full(3, -1, np.float32), tri, 1)
    mats = [wf.WfMaterial(type=0, albedo=(1, 0, 0), texture_id=-1), wf.WfMaterial(type=0, albedo=(0, 1, 0), texture_id=-1)]
    desc, keep = _desc(wf, [A, B], mats)
    ctx.upload(desc)
    h = ctx.trace_closest(o[:1], d[:1])
    assert h["material_id"][0] == 1 and abs(h["distance"][0] - 1.0) < 1e-2
    # empty scene (EmptySceneReturnsNoHit)
    desc, keep = _desc(wf, [], mats)
    ctx.upload(desc)
    assert ctx.trace_closest(o[:1], d[:1])["prim_id"][0] == -1
    assert ctx.trace_occluded(o[:1], d[:1], np.array([10.0], np.float32))[0] == 0


def _desc(wf, meshes, materials):
    """Flat scene description from (px, py, pz, local indices, material) meshes."""
    px, py, pz, idx, off, cnt, mat = [], [], [], [], [], [], []
    base = 0
    for (x, y, z, i, m) in meshes:
        off.append(sum(len(a) for a in idx))
        cnt.append(len(i))
        idx.append(np.asarray(i, np.int32) + base)
        px.append(x); py.append(y); pz.append(z)
        mat.append(m)
        base += len(x)
    cat = lambda L, t: np.ascontiguousarray(np.concatenate(L) if L else np.zeros(0, t), dtype=t)
    arrs = dict(px=cat(px, np.float32), py=cat(py, np.float32), pz=cat(pz, np.float32),
                idx=cat(idx, np.int32), off=np.array(off, np.int32), cnt=np.array(cnt, np.int32),
                mat=np.array(mat, np.int32))
    marr = (wf.WfMaterial * len(materials))(*materials)
    import ctypes as C
    d = wf.WfSceneDesc()
    d.num_vertices = len(arrs["px"])
    d.positions_x, d.positions_y, d.positions_z = wf.ptr(arrs["px"]), wf.ptr(arrs["py"]), wf.ptr(arrs["pz"])
    d.num_indices = len(arrs["idx"])
    d.indices = wf.ptr(arrs["idx"], C.c_int32)
    d.num_meshes = len(meshes)
    d.mesh_index_offsets = wf.ptr(arrs["off"], C.c_int32)
    d.mesh_index_counts = wf.ptr(arrs["cnt"], C.c_int32)
    d.mesh_material_ids = wf.ptr(arrs["mat"], C.c_int32)
    d.num_materials = len(materials)
    d.materials = marr
    d.environment.intensity_scale = 1.0
    return d, (arrs, marr)


def test_ray_schedule_matches_oracle(wf, orc, ctx):
    rng = np.random.default_rng(21)
    n = 100_000
    o = rng.uniform(-12, 12, size=(n, 3)).astype(np.float32)  # some outside the bounds (clamped)
    d = rng.normal(size=(n, 3)).astype(np.float32)
    d[:500, 0] = 0.0  # +0 direction components go to the positive octant
    o[1000:1500] = o[1000]  # identical keys: the stable order must hold
    bmin, bmax = np.array([-10, -10, -10], np.float32), np.array([10, 10, 10], np.float32)
    perm, keys = ctx.ray_schedule(o, d, bmin, bmax)
    assert np.array_equal(keys, orc.ray_sort_keys(o, d, bmin, bmax))
    assert np.array_equal(perm, orc.ray_schedule(o, d, bmin, bmax))
    # flat scene: zero extent on an axis (SceneTest RayQueueScheduleDoesNotDivideByZeroOnFlatScene)
    bmin2, bmax2 = np.array([-1, -1, 0], np.float32), np.array([1, 1, 0], np.float32)
    perm2, _ = ctx.ray_schedule(o[:1000], d[:1000], bmin2, bmax2)
    assert np.array_equal(perm2, orc.ray_schedule(o[:1000], d[:1000], bmin2, bmax2))


def test_ray_schedule_known_answers(wf, ctx):
    """tests/scheduling/RayQueueTest.cpp:132-171 through the GPU."""
    bmin, bmax = np.array([-10, -10, -10], np.float32), np.array([10, 10, 10], np.float32)
    o = np.zeros((4, 3), np.float32)
    d = np.array([[1, 1, 1], [-1, -1, -1], [1, 1, 1], [-1, -1, -1]], np.float32)
    perm, _ = ctx.ray_schedule(o, d, bmin, bmax)
    pix = np.array([10, 20, 11, 21])[perm]
    assert sorted(pix[:2]) in ([10, 11], [20, 21]) and sorted(pix[2:]) in ([10, 11], [20, 21])
    o = np.array([[5, 0, 0], [-5, 0, 0], [0, 0, 0]], np.float32)
    d = np.tile(np.array([[0, 0, 1]], np.float32), (3, 1))
    perm, _ = ctx.ray_schedule(o, d, bmin, bmax)
    assert list(np.array([100, 200, 300])[perm]) == [200, 300, 100]


def _materials(wf):
    mk = wf.WfMaterial
    return [mk(type=0, albedo=(1, 1, 1), roughness=1, texture_id=-1),
            mk(type=1, albedo=(1, 1, 1), roughness=0.5, texture_id=-1),
            mk(type=2, albedo=(1, 1, 1), emission=1, texture_id=-1),
            mk(type=3, albedo=(1, 1, 1), emission=1, spot_outer_deg=45, spot_falloff_deg=30, texture_id=-1),
            mk(type=4, albedo=(1, 1, 1), ior=1.5, texture_id=-1),
            mk(type=5, albedo=(1, 1, 1), roughness=0.5, texture_id=-1)]


def test_shading_schedule_known_answers(wf, ctx):
    """tests/scheduling/ShadingQueueTest.cpp:73-200 through the GPU."""
    mats = _materials(wf)
    tb = np.array([12, 48, 192], np.int64)  # Texture(1,1), (2,2), (4,4) memoryBytes
    def run(policy, mids, tids=None):
        n = len(mids)
        tids = np.zeros(n, np.int32) if tids is None else np.asarray(tids, np.int32)
        return ctx.shading_schedule(policy, np.asarray(mids, np.int32), tids, np.ones((n, 3), np.float32),
                                    np.zeros((n, 3), np.float32), mats, tb)
    m = np.array([2, 0, 1])
    assert list(m[run(0, m)]) == [2, 0, 1]          # none keeps arrival order
    assert list(m[run(1, m)]) == [2, 1, 0]          # material: ties -> higher type first
    m = np.array([1, 0, 1, 0, 1])
    assert list(m[run(1, m)]) == [1, 1, 1, 0, 0]    # grouping by count
    t = np.array([0, 2, 1])
    assert list(t[run(2, [0, 1, 0], t)]) == [2, 1, 0]  # texture bytes descending
    assert list(run(1, [5])) == [0]
    assert list(np.array([42, 99])[run(1, [1, 0])]) == [42, 99]


@pytest.mark.parametrize("policy", [0, 1, 2, 3])
def test_shading_schedule_matches_oracle(wf, orc, ctx, policy):
    rng = np.random.default_rng(100 + policy)
    mk = wf.WfMaterial
    types = [0, 1, 4, 5, 0, 1, 4, 2, 0, 5, 1, 3]
    mats = [mk(type=t, albedo=(0.5, 0.5, 0.5), roughness=0.3, emission=1.0, ior=1.5,
               texture_id=(i % 5 if i % 3 else -1)) for i, t in enumerate(types)]
    tex_bytes = np.array([12 * 512 * 512, 12 * 256 * 256, 12 * 512 * 512, 12 * 64 * 64, 0], np.int64)
    n = 30000
    mids = rng.integers(0, len(mats), n).astype(np.int32)
    tids = np.array([mats[m].texture_id for m in mids], np.int32)
    tids[rng.random(n) < 0.1] = -1  # queue texture ids need not match the material
    thr = rng.uniform(0, 1, size=(n, 3)).astype(np.float32)
    thr[rng.random(n) < 0.2] = 1.0
    pts = rng.uniform(-3, 3, size=(n, 3)).astype(np.float32)
    ids = rng.integers(0, len(mats), 4000)
    rc_mat = orc.cost_tracker_relative(len(mats), ids, rng.uniform(10, 50, 4000))
    rc_tex = orc.cost_tracker_relative(5, rng.integers(0, 5, 600), rng.uniform(5, 9, 600))
    g = ctx.shading_schedule(policy, mids, tids, thr, pts, mats, tex_bytes, rc_mat, rc_tex)
    c = orc.shading_schedule(policy, mids, tids, thr, pts, mats, tex_bytes, rc_mat, rc_tex)
    assert np.array_equal(g, c)
    assert sorted(g) == list(range(n))


def _path_agreement(name, img, ref):
    """Fraction of pixels within 1e-3 relative + 1e-4 absolute of the port's
    (same random streams), reported with the exact-equality fraction, the
    count of disagreeing pixels and the largest difference before any
    assertion, so a divergence below the threshold is visible."""
    from conftest import report

    close = np.isclose(img, ref, rtol=1e-3, atol=1e-4).all(axis=2)
    agree = float(close.mean())
    report(name, agree=agree, exact=float((img == ref).all(axis=2).mean()), disagreeing_pixels=int((~close).sum()),
           pixels=int(close.size), max_abs_diff=float(np.abs(img - ref).max()),
           channel_mean_gpu=[float(x) for x in img.mean(axis=(0, 1))],
           channel_mean_port=[float(x) for x in ref.mean(axis=(0, 1))])
    return agree


def _mean_close(a, b, rel):
    ma, mb = a.mean(axis=(0, 1)), b.mean(axis=(0, 1))
    return np.all(np.abs(ma - mb) <= rel * np.abs(mb))


@pytest.mark.parametrize("which", ["c0", "small", "c2small"])
def test_render_matches_oracle_paths(wf, orc, ctx, scene0, scene_small, scene_c2small, which):
    """Same seed, same random streams: pixels agree except where a
    transcendental's last ulp moves a path.  Tolerance: 98% of pixels within
    1e-3 relative + 1e-4 absolute, channel means within 1%."""
    scene = {"c0": scene0, "small": scene_small, "c2small": scene_c2small}[which]
    ctx.upload(scene.desc)
    port = orc.Port(scene.desc)
    W = H = 64
    spp = 8
    cam = scene.camera(W, H)
    p = wf.render_params(W, H, spp, 8 if which == "c0" else 12, cam, seed=99)
    img, st = ctx.render(p)
    acc, cnt = port.render_window(p, 0, 0, W, H)
    ref = acc / spp
    agree = _path_agreement(f"paths_{which}", img, ref)
    assert agree >= 0.98, agree
    assert _mean_close(img, ref, 0.01)
    assert st["closest_rays"] == cnt["closest_rays"] or abs(st["closest_rays"] - cnt["closest_rays"]) < 0.01 * cnt["closest_rays"]


@pytest.mark.parametrize("which", ["small", "c2small"])
def test_render_is_order_independent(wf, ctx, scene_small, scene_c2small, which):
    """Ray sort, policies and wave size change only the order of work: with
    path-keyed random streams the image is the same up to float-add order
    (atomic accumulation); tolerance 1e-4 relative on 99.9% of pixels."""
    scene = scene_small if which == "small" else scene_c2small
    ctx.upload(scene.desc)
    W = H = 48
    cam = scene.camera(W, H)
    base, _ = ctx.render(wf.render_params(W, H, 8, 12, cam, seed=5))
    assert np.isfinite(base).all()
    for kw in [dict(ray_sort=True), dict(policy=1), dict(policy=2), dict(policy=3), dict(spp_per_wave=3)]:
        img, _ = ctx.render(wf.render_params(W, H, 8, 12, cam, seed=5, **kw))
        agree = np.isclose(img, base, rtol=1e-4, atol=1e-6).all(axis=2).mean()
        assert agree >= 0.999, (kw, agree)
    # launch tuning: occupancy variant, grid size, graph replay and the
    # sort-or-skip threshold change no pixel beyond that.
    # The base render issues its bounces back to back with device-side counts;
    # a sort-or-skip threshold sends policy none through the loop that waits
    # for each bounce's counts on the host, graph_mode=1 through graph replay.
    try:
        for tune, kw in [(dict(trace_variant=1), {}),
                         (dict(ray_sort_bits=16), dict(ray_sort=True)),
                         (dict(persistent_blocks_per_sm=4), {}), (dict(graph_mode=1), {}),
                         (dict(sort_min_queue=6000), dict(policy=1, ray_sort=True)),
                         (dict(sort_min_queue=6000), dict(ray_sort=True))]:
            ctx.set_tuning(**tune)
            img, _ = ctx.render(wf.render_params(W, H, 8, 12, cam, seed=5, **kw))
            agree = np.isclose(img, base, rtol=1e-4, atol=1e-6).all(axis=2).mean()
            assert agree >= 0.999, (tune, agree)
    finally:
        ctx.set_tuning()


@pytest.mark.parametrize("builder", [3, 4])
def test_tree_formats_render_the_same_image(wf, ctx, scene_c2small, builder):
    """The 4-wide and surface-area-leaf trees return the binary tree's hits, so a render
    over them (plain launches, graph replay, every launch variant) gives the
    binary tree's image up to float-add order (1e-4 relative, 99.9% of
    pixels).  A context of its own: the resident scenes of one context share
    one tree format."""
    W = H = 48
    cam = scene_c2small.camera(W, H)
    ctx.upload(scene_c2small.desc)
    base, st0 = ctx.render(wf.render_params(W, H, 8, 8, cam, seed=13))
    other = wf.Context(0)
    try:
        other.set_tuning(bvh_builder=builder)
        info = other.upload(scene_c2small.desc)
        assert info.bvh_builder == builder
        for tune in [{}, dict(graph_mode=1), dict(trace_variant=1)]:
            other.set_tuning(bvh_builder=builder, **tune)
            img, st = other.render(wf.render_params(W, H, 8, 8, cam, seed=13))
            agree = np.isclose(img, base, rtol=1e-4, atol=1e-6).all(axis=2).mean()
            assert agree >= 0.999, (tune, agree)
            assert st["closest_rays"] == st0["closest_rays"], tune
    finally:
        other.close()


def test_tuning_rejects_removed_options(wf, ctx):
    """The options taken out after measuring slower everywhere are refused,
    not silently ignored: trace variants beyond 1, the compressed 8-wide tree
    (bvh_builder 2) and non-zero reserved fields."""
    try:
        for bad in [dict(trace_variant=2), dict(trace_variant=3), dict(bvh_builder=2), dict(bvh_builder=5)]:
            with pytest.raises(wf.WfError):
                ctx.set_tuning(**bad)
        for t in (wf.WfTuning(0, 0, 0, 0, 0, 1, 0, 0), wf.WfTuning(0, 0, 0, 0, 0, 0, 1, 0)):  # reserved2, reserved
            rc = wf.load_library().wf_set_tuning(ctx._h, wf.C.byref(t))
            assert wf.ERRORS.get(rc) == "WF_ERR_INVALID_ARGUMENT", rc
        ctx.set_tuning(bvh_builder=4)  # still valid
    finally:
        ctx.set_tuning()


def test_autotune_picks_a_valid_tuning(wf, ctx, scene_small):
    ctx.upload(scene_small.desc)
    cam = scene_small.camera(64, 64)
    p = wf.render_params(64, 64, 4, 8, cam, seed=2, policy=1)
    try:
        tuning, ms = ctx.autotune(p)
        assert ms > 0
        assert tuning["trace_variant"] in (0, 1) and tuning["persistent_blocks_per_sm"] in (4, 8, 12, 16, 24)
        assert tuning["sort_min_queue"] in (0, 1 << 18, 1 << 20, 1 << 22, 2**31 - 1)
        assert ctx.get_tuning() == tuning
        img, _ = ctx.render(p)
        assert np.isfinite(img).all()
    finally:
        ctx.set_tuning()


def test_render_accumulate_and_device_paths(wf, ctx, scene0):
    ctx.upload(scene0.desc)
    W = H = 32
    cam = scene0.camera(W, H)
    p = wf.render_params(W, H, 4, 8, cam, seed=3)
    img, _ = ctx.render(p)
    acc, _ = ctx.render(p, accumulate=True)
    assert np.allclose(acc / 4.0, img, rtol=1e-6, atol=1e-7)
    st = ctx.render_device(p)
    img2 = ctx.image_download(W, H)
    assert np.allclose(img2, img, rtol=1e-5, atol=1e-6)
    assert st["kernel_launches"] > 0


def test_errors_are_reported(wf, ctx, scene0):
    ctx.upload(scene0.desc)
    cam = scene0.camera(8, 8)
    with pytest.raises(wf.WfError):
        ctx.render(wf.render_params(1, 8, 1, 8, cam))
    with pytest.raises(wf.WfError):
        ctx.render(wf.render_params(8, 8, 0, 8, cam))
    with pytest.raises(wf.WfError):
        ctx.render(wf.render_params(8, 8, 1, 8, cam, policy=7))
    c2 = wf.Context(0)
    with pytest.raises(wf.WfError, match="STATE"):
        c2.render(wf.render_params(8, 8, 1, 8, cam))
    c2.close()


# ------------------------------------------------ against the golden fixtures ---
# (made by the reference's own sources, tests/golden/make_golden.py)

def test_gpu_golden_hits(wf, ctx, scene0):
    from conftest import GOLDEN
    g = np.load(GOLDEN / "c0_hits.npz")
    ctx.upload(scene0.desc)
    h = ctx.trace_closest(g["o"], g["d"])
    for k in ("prim_id", "material_id", "texture_id", "distance", "point_x", "point_y", "point_z", "normal_x",
              "normal_y", "normal_z", "front_face", "u", "v"):
        assert np.array_equal(h[k], g["i4_" + k]), k
    z = np.load(GOLDEN / "c0_occluded.npz")
    assert np.array_equal(ctx.trace_occluded(z["o"], z["d"], z["maxd"]), z["occluded"])


def test_gpu_golden_camera(wf, ctx, scene0):
    from conftest import GOLDEN
    g = np.load(GOLDEN / "c0_camera.npz")
    cam = scene0.camera(256, 256)
    assert np.allclose(cam.as_array(), g["cam12"], rtol=0, atol=1e-7)


def test_gpu_golden_schedules(wf, ctx):
    from conftest import GOLDEN
    from test_oracle import golden_materials
    g = np.load(GOLDEN / "ray_schedule.npz")
    perm, keys = ctx.ray_schedule(g["o"], g["d"], g["bmin"], g["bmax"])
    assert np.array_equal(keys, g["keys"]) and np.array_equal(perm, g["perm"])
    s = np.load(GOLDEN / "shading_schedule.npz")
    mats = golden_materials(wf, s["mats"])
    tb = s["tex_wh"][:, 0].astype(np.int64) * s["tex_wh"][:, 1] * 12
    for policy in range(4):
        perm = ctx.shading_schedule(policy, s["mids"], s["tids"], s["thr"], s["pts"], mats, tb, s["rc_mat"], s["rc_tex"])
        assert np.array_equal(perm, s[f"perm_{policy}"]), policy


def test_gpu_render_within_fp64_band(wf, ctx, scene0):
    """Config 0 at its full size (256x256, 16 spp, depth 8) against the
    reference's 16k-spp FP64 per-pixel mean (conftest.fp64_band: bias,
    variance, tail, MSE, channel means)."""
    from conftest import GOLDEN, fp64_band
    path = GOLDEN / "c0_fp64.npz"
    if not path.exists():
        pytest.skip("FP64 oracle fixture not generated")
    g = np.load(path)
    ctx.upload(scene0.desc)
    W = H = 256
    spp = 16
    img, st = ctx.render(wf.render_params(W, H, spp, 8, scene0.camera(W, H), seed=31337))
    out = fp64_band(img, spp, g)
    print(f"MSE vs FP64 oracle {out['mse']:.4e} (variance predicts {out['expected_mse']:.4e}), {out}")


# ------------------------------------ environment NEE (GPU addition) -------

def test_gpu_env_nee_matches_analytic_irradiance(wf, orc, ctx):
    """The GPU's environment NEE converges to the exact cosine-weighted
    integral of the map (plane under the config-102 HDRI, sun lobe 1e4):
    within 4 standard errors of 8 runs + 1e-3 relative."""
    from conftest import PlaneUnderSky

    hs = wf.HostScene(102)  # owns the map scene_environment copies
    sky = PlaneUnderSky(wf, orc.scene_environment(hs.desc))
    ctx.upload(sky.desc)
    W = H = 64
    spp, N = 256, 8
    cam = sky.camera(wf, W, H)
    X = np.array([ctx.render(wf.render_params(W, H, spp, 2, cam, seed=900 + k, env_nee=True))[0]
                  for k in range(N)], np.float64).mean(axis=(1, 2))
    m, se = X.mean(0), X.std(0, ddof=1) / np.sqrt(N)
    assert np.all(np.abs(m - sky.expected) <= 4 * se + 1e-3 * sky.expected), (m, se, sky.expected)


def test_render_matches_oracle_plastic_spotlight(wf, orc, ctx):
    """The plastic lobes (Schlick-chosen fuzzy mirror or cosine lobe) and the
    spotlight's cone (full inside the falloff angle, smoothstep to the outer
    angle, dark beyond) against the port on the same random streams: the
    Cornell box with its white box turned plastic (roughness 0.2) and its
    ceiling light a spotlight (falloff 35, outer 65 degrees); without an
    environment map, textures or a directional light it runs the lean
    shading instance.  Tolerance as for the other path-level checks."""
    scene = wf.HostScene(0)  # a copy of its own: the materials are edited in place
    mats = scene.desc.materials
    kinds = [mats[i].type for i in range(scene.desc.num_materials)]
    light = kinds.index(wf.MATERIAL_EMISSIVE)
    mats[light].type = wf.MATERIAL_SPOTLIGHT
    mats[light].spot_falloff_deg = 35.0
    mats[light].spot_outer_deg = 65.0
    box = scene.desc.num_materials - 1  # the white Lambert box
    assert kinds[box] == wf.MATERIAL_DIFFUSE
    mats[box].type = wf.MATERIAL_PLASTIC
    mats[box].roughness = 0.2
    ctx.upload(scene.desc)
    port = orc.Port(scene.desc)
    W = H = 64
    spp = 8
    cam = scene.camera(W, H)
    p = wf.render_params(W, H, spp, 8, cam, seed=41)
    img, st = ctx.render(p)
    acc, cnt = port.render_window(p, 0, 0, W, H)
    ref = acc / spp
    assert ref.mean() > 0.0
    agree = _path_agreement("paths_plastic_spotlight", img, ref)
    assert agree >= 0.98, agree
    assert _mean_close(img, ref, 0.01)


def test_gpu_env_nee_matches_oracle_paths(wf, orc, ctx, scene_c2small):
    """Environment NEE on the textured 16 x 16 lattice: the GPU's paths are
    the port's (same alias table, same random streams); tolerance as for the
    other path-level checks."""
    ctx.upload(scene_c2small.desc)
    port = orc.Port(scene_c2small.desc)
    W = H = 64
    spp = 8
    cam = scene_c2small.camera(W, H)
    p = wf.render_params(W, H, spp, 8, cam, seed=77, env_nee=True)
    img, st = ctx.render(p)
    acc, cnt = port.render_window(p, 0, 0, W, H)
    ref = acc / spp
    agree = _path_agreement("paths_env_nee", img, ref)
    assert agree >= 0.98, agree
    assert _mean_close(img, ref, 0.01)
    assert abs(int(st["shadow_rays"]) - int(cnt["shadow_rays"])) <= 0.01 * cnt["shadow_rays"]


# ------------------------------------------------ adaptive sampling --------

@pytest.mark.parametrize("spw", [0, 4, 16])
def test_gpu_adaptive_matches_oracle(wf, orc, ctx, scene0, spw):
    """AdaptiveSampler on the GPU: each pixel's sample count and image equal
    the port's (same random streams; the Welford inputs differ only by the
    order of float additions, so a stop may move by one check on a few
    pixels).  spw 0 runs samples 0-31 as one wave and then waves of 16 (the
    per-sample slots of a 32-slot buffer used from slot 16 on alternate
    waves); 4 and 16 run fixed waves.  Tolerance: counts equal on 99% of pixels, image within 1e-3
    relative + 1e-4 on 98%."""
    ctx.upload(scene0.desc)
    port = orc.Port(scene0.desc)
    W = H = 64
    spp = 64
    cam = scene0.camera(W, H)
    p = wf.render_params(W, H, spp, 8, cam, seed=31, adaptive=True, adaptive_threshold=0.1, spp_per_wave=spw)
    img, st = ctx.render(p)
    counts = ctx.sample_counts(W, H)
    acc, _, pc = port.render_window(p, 0, 0, W, H, counts=True)
    assert (counts == pc).mean() >= 0.99
    assert (counts < spp).mean() > 0.2
    ref = acc / np.maximum(pc, 1)[..., None]
    assert np.isclose(img, ref, rtol=1e-3, atol=1e-4).all(axis=2).mean() >= 0.98
    assert st["samples_run"] == spp or (counts < spp).all()
    assert st["active_pixels"] <= int((counts == spp).sum())


def test_gpu_adaptive_off_counts_are_spp(wf, ctx, scene0):
    ctx.upload(scene0.desc)
    cam = scene0.camera(16, 16)
    ctx.render(wf.render_params(16, 16, 4, 8, cam, seed=3))
    assert (ctx.sample_counts(16, 16) == 4).all()


# ------------------------------------------------ live CostTracker ---------

def test_gpu_cost_tracker_replay_matches_oracle(wf, orc, ctx):
    """The device CostTracker update (run after every bounce) is the
    reference's record/relativeCost: replaying per-step cycle sums gives the
    port's relative costs bit for bit (EMA weight 0.05, 50-record floor)."""
    rng = np.random.default_rng(5)
    items, steps = 7, 160
    counts = rng.integers(0, 40, size=(steps, items)).astype(np.uint32)
    counts[rng.random((steps, items)) < 0.3] = 0
    per_call = rng.integers(200, 5000, size=items)
    sums = (counts * per_call[None, :] * rng.uniform(0.5, 1.5, size=(steps, items))).astype(np.uint64)
    got = ctx.cost_tracker_replay(sums, counts)
    ids, costs = [], []
    for k in range(steps):
        for i in range(items):
            if counts[k, i]:
                ids.append(i)
                costs.append(float(sums[k, i]) / float(counts[k, i]))
    want = orc.cost_tracker_relative(items, ids, costs)
    assert np.array_equal(got, want)
    assert (got != 1.0).any()


def test_gpu_live_cost_aware_rr_is_unbiased(wf, ctx, scene0):
    """Cost-aware RR driven by live device timings changes which paths
    survive but not the expectation: channel means of 8 runs with and
    without it agree within 4 standard errors."""
    ctx.upload(scene0.desc)
    W = H = 64
    cam = scene0.camera(W, H)
    def runs(**kw):
        return np.array([ctx.render(wf.render_params(W, H, 32, 8, cam, seed=100 + k, **kw))[0].mean(axis=(0, 1))
                         for k in range(8)], np.float64)
    a = runs()
    b = runs(cost_aware_rr=True, cost_tracking=True)
    se = np.sqrt(a.var(0, ddof=1) / 8 + b.var(0, ddof=1) / 8)
    assert np.all(np.abs(a.mean(0) - b.mean(0)) <= 4 * se + 1e-6)
    rel_m, _ = ctx.cost_tracker_state(scene0.desc.num_materials, scene0.desc.num_textures)
    assert np.all(rel_m > 0) and (rel_m != 1.0).any()


@pytest.mark.parametrize("policy", [1, 3])
def test_gpu_live_costs_only_reorder_shading(wf, ctx, scene_c2small, policy):
    """With cost-aware RR off, live costs only change the material /
    costBenefit orders: the image is the plain render's up to float-add
    order."""
    ctx.upload(scene_c2small.desc)
    W = H = 48
    cam = scene_c2small.camera(W, H)
    base, _ = ctx.render(wf.render_params(W, H, 4, 8, cam, seed=9))
    img, st = ctx.render(wf.render_params(W, H, 4, 8, cam, seed=9, policy=policy, cost_tracking=True))
    assert np.isclose(img, base, rtol=1e-4, atol=1e-6).all(axis=2).mean() >= 0.999
    rel_m, rel_t = ctx.cost_tracker_state(scene_c2small.desc.num_materials, scene_c2small.desc.num_textures)
    assert np.all(rel_m > 0) and np.all(rel_t > 0)


# ------------------------------------------------ BVH builders -------------

@pytest.mark.parametrize("which", ["c0", "small", "c2small"])
def test_bvh_builders_give_identical_hits(wf, orc, ctx, scene0, scene_small, scene_c2small, which):
    """The binary PLOC tree (default leaves), the LBVH, the 4-wide PLOC tree
    and the PLOC tree with surface-area leaves return the same closest hits
    and occlusion bit for bit (and the port's), and each passes the build's
    structural check."""
    scene = {"c0": scene0, "small": scene_small, "c2small": scene_c2small}[which]
    rng = np.random.default_rng(21)
    lo, hi = ([0.0, 0.01, 0.0], [16.0, 0.9, 16.0]) if which == "c2small" else \
        ([-0.27, 0.01, -0.54], [0.27, 0.54, -0.01])
    o, d = rays_in_box(rng, 60000, lo, hi)
    maxd = rng.uniform(0.01, 2.0, len(o)).astype(np.float32)
    port = orc.Port(scene.desc)
    want = port.trace_closest(o, d)
    want_occ = port.trace_occluded(o, d, maxd)
    infos = []
    try:
        for builder in (0, 1, 3, 4):
            ctx.set_tuning(bvh_builder=builder)
            infos.append(ctx.upload(scene.desc))
            got = ctx.trace_closest(o, d)
            for k in HIT_KEYS_EXACT:
                assert np.array_equal(got[k], want[k]), (builder, k)
            assert np.array_equal(ctx.trace_occluded(o, d, maxd), want_occ), builder
    finally:
        ctx.set_tuning()
    assert [i.bvh_builder for i in infos] == [0, 1, 3, 4]
    assert infos[2].bvh_nodes < infos[0].bvh_nodes  # the 4-wide tree has fewer nodes
    assert infos[2].bvh_depth < infos[0].bvh_depth


@pytest.mark.parametrize("ntri", [1, 2, 4, 5, 9, 33])
def test_bvh_builders_on_tiny_scenes(wf, orc, ntri):
    """Trees of a few triangles — the whole tree one leaf (<= 4 triangles),
    the first split, a couple of levels — give the port's hits and occlusion
    under every builder.  A context of its own per format."""
    rng = np.random.default_rng(100 + ntri)
    c = rng.uniform(-0.5, 0.5, size=(ntri, 1, 3))
    v = (c + rng.uniform(-0.3, 0.3, size=(ntri, 3, 3))).reshape(-1, 3).astype(np.float32)
    idx = np.arange(3 * ntri, dtype=np.int32)
    mats = [wf.WfMaterial(type=0, albedo=(0.5, 0.5, 0.5), texture_id=-1)]
    desc, keep = _desc(wf, [(v[:, 0].copy(), v[:, 1].copy(), v[:, 2].copy(), idx, 0)], mats)
    # rays aimed at points on random triangles (a quarter at random points)
    n = 4000
    o = rng.uniform(-1.5, 1.5, size=(n, 3)).astype(np.float32)
    tv = v.reshape(ntri, 3, 3)[rng.integers(0, ntri, n)]
    b = rng.dirichlet([1.0, 1.0, 1.0], n)[:, :, None]
    target = (tv * b).sum(axis=1)
    target[: n // 4] = rng.uniform(-0.8, 0.8, size=(n // 4, 3))
    d = (target - o).astype(np.float32)
    d[:100, 1] = 0.0  # axis-parallel components
    maxd = rng.uniform(0.01, 4.0, n).astype(np.float32)
    port = orc.Port(desc)
    want = port.trace_closest(o, d)
    want_occ = port.trace_occluded(o, d, maxd)
    assert (want["prim_id"] >= 0).mean() > 0.3
    for builder in (0, 1, 3, 4):
        c2 = wf.Context(0)
        try:
            c2.set_tuning(bvh_builder=builder)
            info = c2.upload(desc)
            assert info.bvh_builder == builder
            got = c2.trace_closest(o, d)
            for k in HIT_KEYS_EXACT:
                assert np.array_equal(got[k], want[k]), (builder, k)
            assert np.array_equal(c2.trace_occluded(o, d, maxd), want_occ), builder
        finally:
            c2.close()


def test_scene_file_renders_like_the_original(wf, ctx, scene_c2small, tmp_path):
    """A scene written with wf_scene_save and read back renders the same image
    on the GPU (same arrays, same tree, same random streams)."""
    path = tmp_path / "lattice.wfscene"
    scene_c2small.save(path, [8.0, 4.48, 17.9], [8.0, 0.0, 6.08], [0, 1, 0], 50.0)
    back = wf.HostScene.load(path)
    cam = back.camera(40, 30)
    p = wf.render_params(40, 30, 4, 6, cam, seed=12)
    ctx.upload(scene_c2small.desc)
    a, _ = ctx.render(p)
    ctx.upload(back.desc)
    b, _ = ctx.render(p)
    assert np.isclose(a, b, rtol=1e-4, atol=1e-6).all(axis=2).mean() >= 0.999
