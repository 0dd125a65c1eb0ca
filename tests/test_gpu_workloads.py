"""Parity on the benchmarked workloads at their full sizes (GPU).

* Closest hits and occlusion of the dense-mesh scene (config 1, 1.31 M
  triangles) and of the lattice (config 2, 15.1 M triangles) against the
  fixtures the reference's own code made (EmbreeAccelerator::intersect4 /
  occluded, src/accelerator/Embree.cpp:180-280, over the shimmed BVH whose
  leaves run the reference's intersectTriangle): bit-exact.
* The benchmarked render itself (config 1: 1024^2, 64 spp, depth 12; config
  2: 2048^2, 32 spp, depth 8), through wf_render:
    - a 128 x 128 window against the reference's FP64 mean of that window
      (renderScene, src/render/WavefrontRenderer.cpp:94-399; 16384 / 8192 spp)
      inside the 3-sigma band, with its MSE;
    - path parity against the oracle port on 64 x 64 windows: the same random
      streams give the same paths, so pixels agree except where a
      transcendental's last ulp moves a path.  The disagreeing fraction is
      measured and reported (WF_PARITY_REPORT), and must stay under 2%.
* Config 104 (config 0 + a directional light + a glass box): the directional
  NEE of WavefrontRenderer.cpp:712-737 on Lambert, metal and glass hits,
  against the port (paths) and the reference's FP64 mean (band).
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import GOLDEN, fp64_band, report

pytestmark = pytest.mark.gpu

HIT_FIELDS = ("prim_id", "material_id", "texture_id", "distance", "point_x", "point_y", "point_z", "normal_x",
              "normal_y", "normal_z", "front_face", "u", "v")

# The lattice's estimator is heavy-tailed: sky misses that find the HDRI's
# sun lobe (1e4 times the sky, unclamped as in the reference's miss loop) are
# rare and huge, so its block z-scores have a heavier tail and spread than a
# normal's even when nothing is biased.  Measured on the port (pinned to the
# reference) over 13 seeds of this window at 32 spp (12 on an x86 host, seed
# 4242 on the GPU host): |z| > 3 on 0.9-3.3% of blocks, winsorized z spread
# 0.86-1.12; the band for it allows 5% and +-0.2.
WORKLOAD = {1: dict(size=1024, spp=64, depth=12, windows=[(256, 384), (480, 560)], band={}),
            2: dict(size=2048, spp=32, depth=8, windows=[(960, 1536), (1024, 1200)],
                    band=dict(tail_max=0.05, std_tol=0.2))}


@pytest.fixture(scope="module")
def scenes(wf):
    return {}


def _scene(wf, scenes, config):
    if config not in scenes:
        scenes.clear()  # one large scene at a time in host memory
        scenes[config] = wf.HostScene(config)
    return scenes[config]


@pytest.mark.parametrize("config", [1, 2])
def test_gpu_workload_hits_match_reference_fixture(wf, ctx, scenes, config):
    g = np.load(GOLDEN / f"c{config}_hits.npz")
    z = np.load(GOLDEN / f"c{config}_occluded.npz")
    sc = _scene(wf, scenes, config)
    ctx.upload(sc.desc)
    h = ctx.trace_closest(g["o"], g["d"])
    diff = {k: int((h[k] != g["i4_" + k]).sum()) for k in HIT_FIELDS}
    occ = ctx.trace_occluded(z["o"], z["d"], z["maxd"])
    report(f"hits_config{config}", rays=len(g["o"]), hits=int((g["i4_prim_id"] >= 0).sum()),
           field_mismatches=diff, occlusion_mismatches=int((occ != z["occluded"]).sum()))
    assert all(v == 0 for v in diff.values()), diff
    assert np.array_equal(occ, z["occluded"])


@pytest.mark.parametrize("config,policy", [(1, "none"), (1, "material"), (2, "none"), (2, "material"),
                                           (2, "texture"), (2, "costBenefit")])
def test_gpu_workload_render_matches_reference_and_port(wf, orc, ctx, scenes, config, policy):
    """The benchmarked render, under each scheduling policy its workload
    compares (dense mesh: none and material; lattice: all four): its paths
    equal to the port's on the fixture window and a second window (the port
    renders the same pixels with the same random streams; a policy only
    reorders the work), and its fixture window inside the band of the
    reference's FP64 mean.  Every figure is reported before anything is
    asserted."""
    w = WORKLOAD[config]
    g = np.load(GOLDEN / f"c{config}_fp64_crop.npz")
    assert int(g["max_depth"]) == w["depth"] and int(g["image_size"][0]) == w["size"]
    sc = _scene(wf, scenes, config)
    ctx.upload(sc.desc)
    W = H = w["size"]
    spp = w["spp"]
    p = wf.render_params(W, H, spp, w["depth"], sc.camera(W, H), seed=4242, policy=wf.POLICIES[policy])
    img, st = ctx.render(p)
    assert np.isfinite(img).all()
    x0, y0, cw, ch = (int(v) for v in g["window"])
    port = orc.Port(sc.desc)
    paths = {}
    port_window = None
    for (wx, wy, ww, wh) in [(x0, y0, cw, ch), (w["windows"][1][0], w["windows"][1][1], 64, 64)]:
        acc, cnt = port.render_window(p, wx, wy, ww, wh)
        ref = acc / spp
        if (wx, wy) == (x0, y0):
            port_window = ref
        got = img[wy:wy + wh, wx:wx + ww]
        close = np.isclose(got, ref, rtol=1e-3, atol=1e-4).all(axis=2)
        paths[f"{wx},{wy},{ww}x{wh}"] = {"disagreeing_pixel_frac": float(1.0 - close.mean()),
                                         "max_abs_diff": float(np.abs(got - ref).max()),
                                         "channel_rel": (got.mean((0, 1)) / ref.mean((0, 1)) - 1).tolist()}
    band, band_error = None, None
    try:
        band = fp64_band(img[y0:y0 + ch, x0:x0 + cw], spp, g, **w["band"])
    except AssertionError as e:
        band_error = str(e)
    try:
        port_band = fp64_band(port_window, spp, g, **w["band"])
    except AssertionError as e:
        port_band = {"failed": str(e)}
    report(f"render_config{config}_{policy}", image=f"{W}x{H}x{spp}spp depth {w['depth']}", fp64_window=band or band_error,
           port_same_seed_fp64_window=port_band, port_windows=paths, closest_rays=st["closest_rays"],
           shadow_rays=st["shadow_rays"])
    for k, v in paths.items():
        assert v["disagreeing_pixel_frac"] <= 0.02, (k, v)
    assert band_error is None, band_error


def test_gpu_directional_light_matches_reference_and_port(wf, orc, ctx):
    """Config 104: directional NEE on Lambert, metal and glass."""
    sc = wf.HostScene(104)
    ctx.upload(sc.desc)
    g = np.load(GOLDEN / "c104_fp64.npz")
    W = H = 128
    spp = 64
    img, st = ctx.render(wf.render_params(W, H, spp, 8, sc.camera(W, H), seed=777))
    band = fp64_band(img, spp, g)
    port = orc.Port(sc.desc)
    p = wf.render_params(64, 64, 8, 8, sc.camera(64, 64), seed=99)
    got, st8 = ctx.render(p)
    acc, cnt = port.render_window(p, 0, 0, 64, 64)
    ref = acc / 8
    frac = 1.0 - np.isclose(got, ref, rtol=1e-3, atol=1e-4).all(axis=2).mean()
    # without the directional light the same render traces fewer shadow rays
    no_sun = wf.HostScene(104)
    no_sun.desc.directional.intensity = 0.0
    ctx.upload(no_sun.desc)
    _, st_off = ctx.render(p)
    report("directional_config104", fp64_band=band, port_disagreeing_pixel_frac=float(frac),
           shadow_rays=st8["shadow_rays"], shadow_rays_without_directional=st_off["shadow_rays"],
           port_shadow_rays=cnt["shadow_rays"])
    assert frac <= 0.02, frac
    assert abs(st8["shadow_rays"] - cnt["shadow_rays"]) <= 0.01 * cnt["shadow_rays"]
    assert st_off["shadow_rays"] < 0.8 * st8["shadow_rays"]
