"""Shared fixtures.  GPU tests are marked `gpu`; everything else runs on CPU.

The oracle (oracle/oracle.py) is the checker only: tests compare the CUDA path
(libwfgpu.so through its C ABI) against it and against the committed golden
fixtures made from the reference's own sources (tests/golden/make_golden.py).
"""
from __future__ import annotations

import importlib.util
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT / "oracle"))
GOLDEN = ROOT / "tests" / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300)")


# Figures the parity tests measure (disagreeing-pixel fractions, MSE against
# the FP64 oracle, ...), keyed by test.  With WF_PARITY_REPORT=<path> they are
# written there as JSON when the session ends.
PARITY_REPORT: dict = {}


def report(name: str, **figures) -> None:
    PARITY_REPORT[name] = {k: (float(v) if isinstance(v, (np.floating, np.integer)) else v)
                           for k, v in figures.items()}


def pytest_sessionfinish(session, exitstatus):
    import json
    import os

    path = os.environ.get("WF_PARITY_REPORT")
    if path and PARITY_REPORT:
        Path(path).parent.mkdir(parents=True, exist_ok=True)
        Path(path).write_text(json.dumps(PARITY_REPORT, indent=1, sort_keys=True))


def _load(name, path):
    if name in sys.modules:
        return sys.modules[name]
    spec = importlib.util.spec_from_file_location(name, path)
    mod = importlib.util.module_from_spec(spec)
    sys.modules[name] = mod
    spec.loader.exec_module(mod)
    return mod


@pytest.fixture(scope="session")
def wf():
    mod = _load("wavefront_gb300", ROOT / "wavefront-renderer_gb300" / "__init__.py")
    if not mod.LIB_PATH.exists():
        _load("wavefront_gb300_build", ROOT / "wavefront-renderer_gb300" / "build.py").build()
    mod.load_library()
    return mod


@pytest.fixture(scope="session")
def orc():
    import oracle

    oracle.port_lib()
    return oracle


@pytest.fixture(scope="session")
def ctx(wf):
    c = wf.Context(0)
    yield c
    c.close()


@pytest.fixture(scope="session")
def scene0(wf):
    return wf.HostScene(0)


@pytest.fixture(scope="session")
def scene_small(wf):
    return wf.HostScene(100, seed=3)


@pytest.fixture(scope="session")
def scene_c2small(wf):
    """16 x 16 meshes, 256 materials (glass, metal, textured Lambert), HDRI."""
    return wf.HostScene(102)


def rays_in_box(rng, n, lo, hi):
    """Random rays from points inside an axis box, directions uniform on the sphere."""
    o = rng.uniform(lo, hi, size=(n, 3)).astype(np.float32)
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    return o, d.astype(np.float32)


def fp64_band(img, spp, golden, block=8, tail_max=0.03, std_tol=0.15):
    """Check (c): an image rendered with `spp` samples against the
    reference's FP64 per-pixel mean (`golden["mean"]`, over `golden["spp"]`
    samples) and per-sample standard deviation (`golden["sigma"]`).

    Per-pixel samples are heavy-tailed (rare paths clamped at the firefly
    threshold of 10; in the lattice scene unclamped sky misses that find a
    1e4 sun lobe), so the 3-sigma band is applied to block means of block x
    block pixels (block*block*spp samples each).  The variance of a difference
    counts both sides: sigma^2/spp for the image and sigma^2/golden_spp for
    the oracle's own mean.  A block where the render drew a rare path that the
    oracle's variance estimate never saw gets an enormous z without any bias,
    so the mean and spread of the z-scores are taken winsorized at |z| = 5
    (a normal z passes 5 with probability 6e-7; the number of blocks beyond is
    reported, and the tail check below still counts them):
      * bias: the mean block z-score is within 3 standard errors of 0;
      * spread: their standard deviation is 1 +- `std_tol` (0.15);
      * tail: |z| > 3 on fewer than `tail_max` of blocks (3%; a normal tail
        gives 0.27%);
      * MSE against the FP64 mean is within 30% of what the variance predicts;
      * each channel's image mean is within 4 standard errors of the oracle's.
    Returns the figures (MSE included) for reporting."""
    H, W, _ = img.shape
    gspp = float(golden["spp"]) if "spp" in golden else 16384.0
    mean, sigma = golden["mean"].astype(np.float64), golden["sigma"].astype(np.float64)
    pix_var = sigma ** 2 * (1.0 / spp + 1.0 / gspp)
    bm = mean.reshape(H // block, block, W // block, block, 3).mean((1, 3))
    bx = img.astype(np.float64).reshape(H // block, block, W // block, block, 3).mean((1, 3))
    bv = pix_var.reshape(H // block, block, W // block, block, 3).sum((1, 3)) / block ** 4
    live = bv > 1e-14  # blocks that see only a constant sky have no variance
    z = (bx - bm)[live] / np.sqrt(bv[live])
    zw = np.clip(z, -5.0, 5.0)
    mse = float(((img - mean) ** 2).mean())
    expected = float(pix_var.mean())
    ch_se = np.sqrt(pix_var.sum((0, 1))) / (H * W)
    ch_diff = img.astype(np.float64).mean((0, 1)) - mean.mean((0, 1))
    out = {"mse": mse, "expected_mse": expected, "z_mean": float(zw.mean()), "z_std": float(zw.std()),
           "z_beyond_5": int((np.abs(z) > 5).sum()), "z_max_abs": float(np.abs(z).max()),
           "tail_frac": float((np.abs(z) > 3).mean()), "blocks": int(z.size),
           "channel_rel": (ch_diff / mean.mean((0, 1))).tolist(), "channel_z": (ch_diff / ch_se).tolist(),
           "spp": spp, "oracle_spp": gspp}
    assert abs(out["z_mean"]) < 3.0 / np.sqrt(z.size), out
    assert abs(out["z_std"] - 1.0) < std_tol, out
    assert out["tail_frac"] < tail_max, out
    assert mse < 1.3 * expected, out
    assert max(abs(c) for c in out["channel_z"]) < 4.0, out
    return out


class PlaneUnderSky:
    """A Lambertian ground quad (albedo 0.5, 2000 x 2000 at y = 0, normal +y)
    under an equirect environment, seen from 1 m above, looking down.  With
    max depth 2 every pixel's expectation is albedo/pi times the
    cosine-weighted integral of the map over the upper hemisphere, which is
    exact per texel row: (2 pi / W) (sin^2 e_hi - sin^2 e_lo) / 2 for the
    row's elevations clipped at the horizon."""

    def __init__(self, wf, env: np.ndarray):
        import ctypes as C

        self.env = np.ascontiguousarray(env, np.float32)
        H, W, _ = self.env.shape
        self.px = np.array([-1000, 1000, 1000, -1000], np.float32)
        self.py = np.zeros(4, np.float32)
        self.pz = np.array([-1000, -1000, 1000, 1000], np.float32)
        self.idx = np.array([0, 2, 1, 0, 3, 2], np.int32)
        self.off, self.cnt, self.mm = (np.array([v], np.int32) for v in (0, 6, 0))
        self.mats = (wf.WfMaterial * 1)(wf.WfMaterial(type=0, albedo=(0.5, 0.5, 0.5), texture_id=-1))
        d = wf.WfSceneDesc()
        d.num_vertices = 4
        d.positions_x, d.positions_y, d.positions_z = wf.ptr(self.px), wf.ptr(self.py), wf.ptr(self.pz)
        d.num_indices = 6
        d.indices = wf.ptr(self.idx, C.c_int32)
        d.num_meshes = 1
        d.mesh_index_offsets = wf.ptr(self.off, C.c_int32)
        d.mesh_index_counts = wf.ptr(self.cnt, C.c_int32)
        d.mesh_material_ids = wf.ptr(self.mm, C.c_int32)
        d.num_materials = 1
        d.materials = C.cast(self.mats, C.POINTER(wf.WfMaterial))
        d.environment.width, d.environment.height = W, H
        d.environment.rgb = wf.ptr(self.env)
        d.environment.intensity_scale = 1.0
        d.environment.tint[:] = (1.0, 1.0, 1.0)
        self.desc = d
        e = (0.5 - np.arange(H + 1) / H) * np.pi
        hi, lo = np.maximum(e[:-1], 0.0), np.maximum(e[1:], 0.0)
        row = (np.sin(hi) ** 2 - np.sin(lo) ** 2) / 2.0 * (2.0 * np.pi / W)
        self.expected = 0.5 / np.pi * (self.env.astype(np.float64) * row[:, None, None]).sum(axis=(0, 1))

    def camera(self, wf, w, h):
        return wf.camera_make([0, 1, 0], [0, 0, 0.001], [0, 0, -1], 30.0, w, h)
