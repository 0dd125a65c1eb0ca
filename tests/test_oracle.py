"""Pins of the CPU oracle (no GPU).

1. The known-answer cases of the reference's own tests (tests/geometry/
   TriangleTest.cpp, tests/scheduling/RayQueueTest.cpp, ShadingQueueTest.cpp,
   tests/accelerator/EmbreeTest.cpp, tests/core/SceneTest.cpp,
   tests/render/CostTrackerTest.cpp, tests/shading/MaterialFeaturesTest.cpp).
2. The golden fixtures made by the reference's own sources (tests/golden).
3. Where the reference checkout exists, the reference compiled in place.
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import GOLDEN, rays_in_box
from test_gpu_parity import _desc


# The oracle's tests load no GPU library: the ABI's structs come from
# include/wf_abi.py and the workload scenes from the generator compiled into
# liboracle.so.
@pytest.fixture(scope="module")
def wf(orc):
    return orc.wf


@pytest.fixture(scope="module")
def scene0(orc):
    return orc.HostScene(0)


@pytest.fixture(scope="module")
def scene_small(orc):
    return orc.HostScene(100, seed=3)


def _tri_scene(wf, v0, v1, v2):
    x, y, z = (np.array(a, np.float32) for a in zip(v0, v1, v2))
    return _desc(wf, [(x, y, z, np.array([0, 1, 2], np.int32), 0)],
                 [wf.WfMaterial(type=0, albedo=(0.8, 0.8, 0.8), texture_id=-1)])


def test_philox_known_answers(orc):
    """Random123 philox4x32-10 known-answer vectors (Salmon et al., SC'11)."""
    assert list(orc.philox([0, 0, 0, 0], [0, 0])) == [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]
    assert list(orc.philox([0xFFFFFFFF] * 4, [0xFFFFFFFF] * 2)) == [0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD]
    assert list(orc.philox([0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344], [0xA4093822, 0x299F31D0])) == \
        [0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1]


def test_triangle_known_answers(wf, orc):
    """TriangleTest.cpp:4-42."""
    desc, keep = _tri_scene(wf, (-1, 0, 0), (1, 0, 0), (0, 1, 0))
    port = orc.Port(desc)
    o = np.array([[0, 0.3, 1], [5, 5, 1], [0, 0.3, 1]], np.float32)
    d = np.array([[0, 0, -1], [0, 0, -1], [1, 0, 0]], np.float32)
    h = port.trace_closest(o, d)
    assert h["prim_id"][0] == 0 and abs(h["distance"][0] - 1.0) < 1e-4
    assert h["prim_id"][1] == -1 and h["prim_id"][2] == -1
    far = port.trace_closest(np.array([[0, 0.3, 5]], np.float32), d[:1], 0.001, 2.0)
    assert far["prim_id"][0] == -1


def test_embree_wrapper_known_answers(wf, orc):
    """EmbreeTest.cpp:28-292 against the oracle's accelerator semantics."""
    px = np.array([-1, 1, 1, -1], np.float32)
    py = np.array([-1, -1, 1, 1], np.float32)
    pz = np.full(4, -1, np.float32)
    quad = (px, py, pz, np.array([0, 1, 2, 0, 2, 3], np.int32), 0)
    desc, keep = _desc(wf, [quad], [wf.WfMaterial(type=0, albedo=(0.8, 0.8, 0.8), texture_id=-1)])
    port = orc.Port(desc)
    o = np.array([[0, 0, 0], [0, 0, 0], [5, 5, 0]], np.float32)
    d = np.array([[0, 0, -1], [0, 0, 1], [0, 0, -1]], np.float32)
    h = port.trace_closest(o, d)
    assert abs(h["distance"][0] - 1.0) < 1e-3 and h["material_id"][0] == 0
    assert h["normal_z"][0] > 0 and h["front_face"][0] == 1
    assert h["prim_id"][1] == -1 and h["prim_id"][2] == -1
    assert port.trace_closest(o[:1], d[:1], 0.001, 0.5)["prim_id"][0] == -1
    # floor scene, packets of four (Intersect4*)
    floor = (np.array([-5, 5, 5, -5], np.float32), np.zeros(4, np.float32), np.array([-5, -5, 5, 5], np.float32),
             np.array([0, 1, 2, 0, 2, 3], np.int32), 0)
    desc2, keep2 = _desc(wf, [floor], [wf.WfMaterial(type=0, albedo=(0.8, 0.8, 0.8), texture_id=-1)])
    p2 = orc.Port(desc2)
    o4 = np.array([[0, 5, 0], [0, 5, 0], [2, 5, 2], [0, 5, 0]], np.float32)
    d4 = np.array([[0, -1, 0], [0, 1, 0], [0, -1, 0], [0, 1, 0]], np.float32)
    mask = p2.trace_closest(o4, d4)["prim_id"] >= 0
    assert list(mask) == [True, False, True, False]
    # nearest of two meshes
    tri = np.array([0, 1, 2], np.int32)
    A = (np.array([-1, 1, 0], np.float32), np.array([-1, -1, 1], np.float32), np.full(3, -2, np.float32), tri, 0)
    B = (np.array([-1, 1, 0], np.float32), np.array([-1, -1, 1], np.float32), np.full(3, -1, np.float32), tri, 1)
    mats = [wf.WfMaterial(type=0, albedo=(1, 0, 0), texture_id=-1), wf.WfMaterial(type=0, albedo=(0, 1, 0), texture_id=-1)]
    desc3, keep3 = _desc(wf, [A, B], mats)
    h = orc.Port(desc3).trace_closest(o[:1], d[:1])
    assert h["material_id"][0] == 1 and abs(h["distance"][0] - 1.0) < 1e-2
    # empty scene
    desc4, keep4 = _desc(wf, [], mats)
    assert orc.Port(desc4).trace_closest(o[:1], d[:1])["prim_id"][0] == -1


def test_scene_bounds_known_answers(wf, orc):
    """SceneTest.cpp:39-80."""
    quad = (np.array([-4, 3, 3, -4], np.float32), np.array([-1, -1, 5, 5], np.float32),
            np.array([-2, -2, 6, 6], np.float32), np.array([0, 1, 2, 0, 2, 3], np.int32), 0)
    desc, keep = _desc(wf, [quad], [wf.WfMaterial(type=0, albedo=(0.8, 0.8, 0.8), texture_id=-1)])
    bmin, bmax = orc.Port(desc).bounds()
    assert list(bmin) == [-4, -1, -2] and list(bmax) == [3, 5, 6]


def test_ray_queue_known_answers(orc):
    """RayQueueTest.cpp:110-215."""
    bmin, bmax = np.array([-10, -10, -10], np.float32), np.array([10, 10, 10], np.float32)
    assert len(orc.ray_schedule(np.zeros((0, 3), np.float32), np.zeros((0, 3), np.float32), bmin, bmax)) == 0
    o = np.zeros((4, 3), np.float32)
    d = np.array([[1, 1, 1], [-1, -1, -1], [1, 1, 1], [-1, -1, -1]], np.float32)
    pix = np.array([10, 20, 11, 21])[orc.ray_schedule(o, d, bmin, bmax)]
    assert sorted(pix[:2]) in ([10, 11], [20, 21]) and sorted(pix[2:]) in ([10, 11], [20, 21])
    o = np.array([[5, 0, 0], [-5, 0, 0], [0, 0, 0]], np.float32)
    d = np.tile(np.array([[0, 0, 1]], np.float32), (3, 1))
    assert list(np.array([100, 200, 300])[orc.ray_schedule(o, d, bmin, bmax)]) == [200, 300, 100]
    o = np.array([[9999, 9999, 9999], [0, 0, 0]], np.float32)
    assert sorted(orc.ray_schedule(o, d[:2], bmin, bmax)) == [0, 1]


def test_shading_queue_known_answers(wf, orc):
    """ShadingQueueTest.cpp:73-200 and MaterialFeaturesTest.cpp:120-178."""
    mk = wf.WfMaterial
    mats = [mk(type=0, albedo=(1, 1, 1), roughness=1, texture_id=-1), mk(type=1, albedo=(1, 1, 1), roughness=0.5, texture_id=-1),
            mk(type=2, albedo=(1, 1, 1), emission=1, texture_id=-1),
            mk(type=3, albedo=(1, 1, 1), emission=1, spot_outer_deg=45, spot_falloff_deg=30, texture_id=-1),
            mk(type=4, albedo=(1, 1, 1), ior=1.5, texture_id=-1), mk(type=5, albedo=(1, 1, 1), roughness=0.5, texture_id=-1)]
    tb = np.array([12, 48, 192], np.int64)

    def run(policy, mids, tids=None):
        n = len(mids)
        tids = np.zeros(n, np.int32) if tids is None else np.asarray(tids, np.int32)
        return orc.shading_schedule(policy, np.asarray(mids, np.int32), tids, np.ones((n, 3), np.float32),
                                    np.zeros((n, 3), np.float32), mats, tb)
    m = np.array([2, 0, 1])
    assert list(m[run(0, m)]) == [2, 0, 1]
    assert list(m[run(1, m)]) == [2, 1, 0]
    m = np.array([1, 0, 1, 0, 1])
    assert list(m[run(1, m)]) == [1, 1, 1, 0, 0]
    t = np.array([0, 2, 1])
    assert list(t[run(2, [0, 1, 0], t)]) == [2, 1, 0]
    assert list(run(1, [5])) == [0]
    assert list(np.array([2, 1, 0])[run(1, [2, 1, 0])]) == [2, 1, 0]
    assert list(np.array([42, 99])[run(1, [1, 0])]) == [42, 99]


def test_cost_tracker_known_answers(orc):
    """CostTrackerTest.cpp:4-47."""
    assert orc.cost_tracker_relative(3, [], [])[0] == 1.0
    assert orc.cost_tracker_relative(2, [0] * 10, [100.0] * 10)[0] == 1.0
    ids = np.array([0, 1] * 60, np.int32)
    r = orc.cost_tracker_relative(2, ids, np.array([10.0, 30.0] * 60))
    assert r[1] > 1.0 and r[0] < 1.0
    r = orc.cost_tracker_relative(2, ids, np.array([15.0, 15.0] * 60))
    assert abs(r[0] - 1.0) < 0.05 and abs(r[1] - 1.0) < 0.05


def test_uv_interpolation_known_answers(wf, orc):
    """MaterialFeaturesTest.cpp:63-97 through the closest-hit mapping."""
    import ctypes as C
    x = np.array([0, 1, 0], np.float32)
    y = np.array([0, 0, 1], np.float32)
    z = np.zeros(3, np.float32)
    desc, keep = _desc(wf, [(x, y, z, np.array([0, 1, 2], np.int32), 0)],
                       [wf.WfMaterial(type=0, albedo=(1, 1, 1), texture_id=-1)])
    o = np.array([[0.3, 0.4, 1.0]], np.float32)
    d = np.array([[0, 0, -1]], np.float32)
    h = orc.Port(desc).trace_closest(o, d)  # no UVs: barycentric pass-through
    assert abs(h["u"][0] - 0.3) < 1e-6 and abs(h["v"][0] - 0.4) < 1e-6
    cu = np.array([0.0, 1.0, 0.0], np.float32)
    cv = np.array([0.0, 0.0, 1.0], np.float32)
    has = np.array([1], np.uint8)
    desc.corner_u, desc.corner_v = wf.ptr(cu), wf.ptr(cv)
    desc.mesh_has_uv = wf.ptr(has, C.c_uint8)
    h = orc.Port(desc).trace_closest(o, d)
    assert abs(h["u"][0] - 0.3) < 1e-6 and abs(h["v"][0] - 0.4) < 1e-6


# ---------------------------------------------------------------- golden ---

def test_golden_camera(wf, orc, scene0):
    g = np.load(GOLDEN / "c0_camera.npz")
    cam = scene0.camera(256, 256)
    assert np.array_equal(cam.as_array(), g["cam12"])  # wf_camera_make == Camera::Camera
    for (u, v), o, d in zip(g["uv"], g["origins"], g["dirs"]):
        po, pd = orc.camera_get_ray(cam, float(u), float(v))
        assert np.array_equal(po, o) and np.array_equal(pd, d)


def test_golden_hits(wf, orc, scene0):
    g = np.load(GOLDEN / "c0_hits.npz")
    port = orc.Port(scene0.desc)
    h = port.trace_closest(g["o"], g["d"])
    for k in ("prim_id", "material_id", "texture_id", "distance", "point_x", "point_y", "point_z", "normal_x",
              "normal_y", "normal_z", "front_face", "u", "v"):
        assert np.array_equal(h[k], g["i4_" + k]), k
    b = port.trace_closest(g["o"], g["d"], brute=True)
    for k in ("prim_id", "distance", "u", "v", "texture_id"):
        assert np.array_equal(b[k], g["bf_" + k]), k
    z = np.load(GOLDEN / "c0_occluded.npz")
    assert np.array_equal(port.trace_occluded(z["o"], z["d"], z["maxd"]), z["occluded"])


def test_golden_ray_schedule(orc):
    g = np.load(GOLDEN / "ray_schedule.npz")
    assert np.array_equal(orc.ray_sort_keys(g["o"], g["d"], g["bmin"], g["bmax"]), g["keys"])
    assert np.array_equal(orc.ray_schedule(g["o"], g["d"], g["bmin"], g["bmax"]), g["perm"])


def golden_materials(wf, arr):
    return [wf.WfMaterial(type=int(r[0]), albedo=(r[1], r[2], r[3]), roughness=r[4], emission=r[5],
                          texture_id=int(r[6]), ior=r[7]) for r in arr]


@pytest.mark.parametrize("policy", [0, 1, 2, 3])
def test_golden_shading_schedule(wf, orc, policy):
    g = np.load(GOLDEN / "shading_schedule.npz")
    mats = golden_materials(wf, g["mats"])
    tb = (g["tex_wh"][:, 0].astype(np.int64) * g["tex_wh"][:, 1] * 12)
    assert np.array_equal(orc.cost_tracker_relative(len(mats), g["ms_ids"], g["ms_ns"]), g["rc_mat"])
    perm = orc.shading_schedule(policy, g["mids"], g["tids"], g["thr"], g["pts"], mats, tb, g["rc_mat"], g["rc_tex"])
    assert np.array_equal(perm, g[f"perm_{policy}"])


@pytest.mark.skipif(not (GOLDEN / "c0_fp64.npz").exists(), reason="FP64 oracle fixture not generated")
def test_golden_fp64_port_render(wf, orc, scene0):
    """The port's config-0 render at 16 spp against the reference's 16k-spp
    FP64 mean (conftest.fp64_band)."""
    from conftest import fp64_band
    g = np.load(GOLDEN / "c0_fp64.npz")
    W = H = 256
    spp = 16
    port = orc.Port(scene0.desc)
    p = wf.render_params(W, H, spp, 8, scene0.camera(W, H), seed=424242)
    acc, _ = port.render_window(p, 0, 0, W, H)
    fp64_band(acc / spp, spp, g)


@pytest.mark.parametrize("config", [1, 2])
def test_golden_workload_window_port_render(wf, orc, config):
    """The port renders the benchmarked workload's fixture window (config 1:
    1024^2 at 64 spp, depth 12; config 2: 2048^2 at 32 spp, depth 8) inside
    the band of the reference's FP64 mean of that window, and agrees with the
    hit fixtures of the same scene bit for bit."""
    from conftest import fp64_band
    g = np.load(GOLDEN / f"c{config}_fp64_crop.npz")
    sc = orc.HostScene(config)
    port = orc.Port(sc.desc)
    h = np.load(GOLDEN / f"c{config}_hits.npz")
    got = port.trace_closest(h["o"], h["d"])
    for k in ("prim_id", "material_id", "texture_id", "distance", "point_x", "normal_z", "front_face", "u", "v"):
        assert np.array_equal(got[k], h["i4_" + k]), k
    z = np.load(GOLDEN / f"c{config}_occluded.npz")
    assert np.array_equal(port.trace_occluded(z["o"], z["d"], z["maxd"]), z["occluded"])
    W, H = (int(v) for v in g["image_size"])
    x0, y0, w, hh = (int(v) for v in g["window"])
    spp = {1: 64, 2: 32}[config]
    p = wf.render_params(W, H, spp, int(g["max_depth"]), sc.camera(W, H), seed=5150)
    acc, _ = port.render_window(p, x0, y0, w, hh)
    fp64_band(acc / spp, spp, g)


def test_golden_directional_port_render(wf, orc):
    """Config 104 (directional light, metal and glass boxes): the port's
    render at 64 spp inside the band of the reference's FP64 mean."""
    from conftest import fp64_band
    g = np.load(GOLDEN / "c104_fp64.npz")
    sc = orc.HostScene(104)
    port = orc.Port(sc.desc)
    W = H = 128
    spp = 64
    p = wf.render_params(W, H, spp, 8, sc.camera(W, H), seed=8080)
    acc, _ = port.render_window(p, 0, 0, W, H)
    fp64_band(acc / spp, spp, g)


# ------------------------------------------------- live reference (x86 dev) ---

def test_port_directional_statistics_match_reference_live(wf, orc):
    """Config 104: the reference's directional NEE (WavefrontRenderer.cpp
    :712-737) and the port's agree pixel by pixel in distribution (24 runs
    each, |z| > 3 on < 1.5% of pixel channels)."""
    if not orc.ref_available():
        pytest.skip("reference checkout not present")
    sc = orc.HostScene(104)
    ref = orc.Ref(sc.desc, True)
    port = orc.Port(sc.desc)
    W = H = 32
    spp, N = 32, 24
    cam = sc.camera(W, H)
    P = np.array([port.render_window(wf.render_params(W, H, spp, 8, cam, seed=900 + k), 0, 0, W, H)[0] / spp
                  for k in range(N)], np.float64)
    R = np.array([ref.render(cam.as_array(), W, H, spp, 8, seed=700 + k) for k in range(N)], np.float64)
    assert orc.ref_front_face_stats()[0] == 0
    z = (P.mean(0) - R.mean(0)) / np.sqrt(P.var(0, ddof=1) / N + R.var(0, ddof=1) / N + 1e-30)
    assert (np.abs(z) > 3).mean() < 0.015
    assert abs(np.median(P.var(0) / (R.var(0) + 1e-30)) - 1.0) < 0.2


def test_port_equals_reference_live(wf, orc, scene_small):
    if not orc.ref_available():
        pytest.skip("reference checkout not present")
    ref = orc.Ref(scene_small.desc, True)
    port = orc.Port(scene_small.desc)
    rng = np.random.default_rng(77)
    o, d = rays_in_box(rng, 20000, [-0.27, 0.01, -0.54], [0.27, 0.54, -0.01])
    h, r = port.trace_closest(o, d), ref.trace(o, d)
    for k in ("prim_id", "material_id", "distance", "point_x", "normal_y", "u", "front_face"):
        assert np.array_equal(h[k], r[k]), k
    maxd = rng.uniform(0.01, 0.5, 20000).astype(np.float32)
    assert np.array_equal(port.trace_occluded(o, d, maxd), ref.occluded(o, d, maxd))
    assert np.array_equal(port.bounds()[0], ref.bounds()[0])


def test_port_render_statistics_match_reference_live(wf, orc, scene0):
    """Same estimator, independent random streams: per-pixel z-scores of the
    mean over 24 runs each are normal (|z| > 3 on < 1.5% of pixel channels)."""
    if not orc.ref_available():
        pytest.skip("reference checkout not present")
    ref = orc.Ref(scene0.desc, True)
    port = orc.Port(scene0.desc)
    W = H = 32
    spp = 32
    N = 24
    cam = scene0.camera(W, H)
    P = np.array([port.render_window(wf.render_params(W, H, spp, 8, cam, seed=900 + k), 0, 0, W, H)[0] / spp
                  for k in range(N)], np.float64)
    R = np.array([ref.render(cam.as_array(), W, H, spp, 8, seed=700 + k) for k in range(N)], np.float64)
    z = (P.mean(0) - R.mean(0)) / np.sqrt(P.var(0, ddof=1) / N + R.var(0, ddof=1) / N + 1e-30)
    assert (np.abs(z) > 3).mean() < 0.015
    assert abs(np.median(P.var(0) / (R.var(0) + 1e-30)) - 1.0) < 0.2


def _c102_clipped(wf, orc, tmp_path):
    """Config 102 (16 x 16 textured, metal and glass meshes under an HDRI)
    with the HDRI clipped at 2.0 (keeps the variance small).  Glass stays in:
    the reference reads HitRecord::frontFace uninitialised after
    ShadingQueue::getHitRecord (include/scheduling/ShadingQueue.h:144-158),
    and the shim (oracle/shims/core/HitRecord.h) gives it the value the
    intersection computed, which is what the port and the GPU carry."""
    hs = orc.HostScene(102)
    d = hs.desc
    env = np.minimum(orc.scene_environment(d), 2.0).astype(np.float32)
    np.ctypeslib.as_array(d.environment.rgb, shape=(env.size,))[:] = env.ravel()
    path = tmp_path / "env.pfm"
    orc.write_pfm(path, env)
    return hs, d, path


def test_port_textured_hdri_statistics_match_reference_live(wf, orc, tmp_path):
    """Textures (RGBA8 sRGB, per-corner UVs) and the equirect environment map:
    per-pixel means of the port and of the reference over 12 runs of 64 spp
    agree (|z| > 3 on < 2% of pixel channels, whole-image means within 3
    standard errors)."""
    if not orc.ref_available():
        pytest.skip("reference checkout not present")
    hs, d, env_path = _c102_clipped(wf, orc, tmp_path)
    port, ref = orc.Port(d), orc.Ref(d, True)
    W = H = 32
    spp, N = 64, 12
    cam = hs.camera(W, H)
    P = np.array([port.render_window(wf.render_params(W, H, spp, 8, cam, seed=900 + k), 0, 0, W, H)[0] / spp
                  for k in range(N)], np.float64)
    R = np.array([ref.render(cam.as_array(), W, H, spp, 8, seed=700 + k, env_path=env_path) for k in range(N)],
                 np.float64)
    var = P.var(0, ddof=1) / N + R.var(0, ddof=1) / N
    live = var > 1e-12  # pixels that see only the sky are deterministic
    z = (P.mean(0) - R.mean(0))[live] / np.sqrt(var[live])
    assert (np.abs(z) > 3).mean() < 0.02
    pm, rm = P.mean(axis=(1, 2, 3)), R.mean(axis=(1, 2, 3))
    assert abs(pm.mean() - rm.mean()) < 3 * np.sqrt(pm.var(ddof=1) / N + rm.var(ddof=1) / N)


# ------------------------------------ environment NEE (GPU addition) -------

@pytest.mark.parametrize("clip", [50.0, None])
def test_port_env_nee_matches_analytic_irradiance(wf, orc, clip):
    """Environment NEE + MIS is unbiased: a Lambertian plane under the
    config-102 HDRI (sun lobe 1e4, or clipped at 50) converges to the exact
    cosine-weighted integral of the map.  Tolerance 4 standard errors of 8
    independent runs (plus 1e-3 relative for the finite plane)."""
    from conftest import PlaneUnderSky

    hs = orc.HostScene(102)  # owns the map scene_environment copies
    env = orc.scene_environment(hs.desc)
    if clip is not None:
        env = np.minimum(env, clip)
    sky = PlaneUnderSky(wf, env)
    port = orc.Port(sky.desc)
    W = H = 32
    spp, N = 256, 8
    cam = sky.camera(orc, W, H)
    X = np.array([port.render_window(wf.render_params(W, H, spp, 2, cam, seed=900 + k, env_nee=True),
                                     0, 0, W, H)[0] / spp for k in range(N)], np.float64)
    per_run = X.mean(axis=(1, 2))
    m, se = per_run.mean(0), per_run.std(0, ddof=1) / np.sqrt(N)
    assert np.all(np.abs(m - sky.expected) <= 4 * se + 1e-3 * sky.expected), (m, se, sky.expected)
    if clip is not None:  # the reference's miss-only estimator, same mean, more noise
        Y = np.array([port.render_window(wf.render_params(W, H, spp, 2, cam, seed=500 + k), 0, 0, W, H)[0] / spp
                      for k in range(N)], np.float64).mean(axis=(1, 2))
        my, sey = Y.mean(0), Y.std(0, ddof=1) / np.sqrt(N)
        assert np.all(np.abs(my - sky.expected) <= 4 * sey + 1e-3 * sky.expected)
        assert np.all(se < sey)


def test_port_env_nee_mean_matches_reference_live(wf, orc, tmp_path):
    """With environment NEE on, the port's per-pixel means still agree with
    the reference's miss-only renderScene (config 102 with its glass, HDRI
    clipped at 2.0 so both estimators are well behaved)."""
    if not orc.ref_available():
        pytest.skip("reference checkout not present")
    hs, d, env_path = _c102_clipped(wf, orc, tmp_path)
    port, ref = orc.Port(d), orc.Ref(d, True)
    W = H = 32
    spp, N = 64, 12
    cam = hs.camera(W, H)
    P = np.array([port.render_window(wf.render_params(W, H, spp, 8, cam, seed=900 + k, env_nee=True), 0, 0, W, H)[0]
                  / spp for k in range(N)], np.float64)
    R = np.array([ref.render(cam.as_array(), W, H, spp, 8, seed=700 + k, env_path=env_path) for k in range(N)],
                 np.float64)
    var = P.var(0, ddof=1) / N + R.var(0, ddof=1) / N
    live = var > 1e-12
    z = (P.mean(0) - R.mean(0))[live] / np.sqrt(var[live])
    assert (np.abs(z) > 3).mean() < 0.02


# ------------------------------------------------ adaptive sampling --------

def test_port_adaptive_statistics_match_reference_live(wf, orc, scene0):
    """The reference's default sampling mode (AdaptiveSampler on): the
    port's per-pixel means over 12 runs agree with the reference's
    (|z| > 3 on < 1.5% of pixel channels, variance ratio within 20%), and
    pixels do stop early."""
    if not orc.ref_available():
        pytest.skip("reference checkout not present")
    ref = orc.Ref(scene0.desc, True)
    port = orc.Port(scene0.desc)
    W = H = 32
    spp, N, thr = 64, 12, 0.1
    cam = scene0.camera(W, H)
    runs = [port.render_window(wf.render_params(W, H, spp, 8, cam, seed=900 + k, adaptive=True,
                                                adaptive_threshold=thr), 0, 0, W, H, counts=True)
            for k in range(N)]
    P = np.array([a / np.maximum(n, 1)[..., None] for a, _, n in runs], np.float64)
    counts = np.array([n for _, _, n in runs])
    assert (counts < spp).mean() > 0.2 and counts.min() >= 32
    assert set(np.unique(counts)) <= {32, 48, 64}
    R = np.array([ref.render_adaptive(cam.as_array(), W, H, spp, 8, thr, seed=700 + k) for k in range(N)],
                 np.float64)
    var = P.var(0, ddof=1) / N + R.var(0, ddof=1) / N
    live = var > 1e-12
    z = (P.mean(0) - R.mean(0))[live] / np.sqrt(var[live])
    assert (np.abs(z) > 3).mean() < 0.015
    assert abs(np.median(P.var(0) / (R.var(0) + 1e-30)) - 1.0) < 0.2
