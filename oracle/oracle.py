"""ctypes bindings of the CPU oracle — TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline legs use this
module, and only as the checker or as the timed CPU baseline.  The product
(libwfgpu.so) never calls it.

  Port       build/liboracle.so  — C++ restatement of the reference loop
                                    (wf_oracle.cpp), built by `make port`.
  Reference  _ref/libwfref.so     — the reference's own sources compiled in
                                    place with shims (`make ref`); exists only
                                    where the reference checkout is present.
"""
from __future__ import annotations

import ctypes as C
import importlib.util
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent
PORT_LIB = HERE / "build" / "liboracle.so"
REF_LIB = HERE / "_ref" / "libwfref.so"
# The reference checkout: WF_REFERENCE_DIR, else a `reference` directory
# beside this repository.  Only the development machine has one.
REF_SRC = Path(os.environ.get("WF_REFERENCE_DIR", str(ROOT.parent / "reference")))


def _abi():
    """include/wf_abi.py: the ABI's ctypes structs, shared with the product's
    binding.  It is pure Python: importing it loads no library."""
    import sys

    if "wf_abi" in sys.modules:
        return sys.modules["wf_abi"]
    spec = importlib.util.spec_from_file_location("wf_abi", ROOT / "include" / "wf_abi.py")
    m = importlib.util.module_from_spec(spec)
    sys.modules["wf_abi"] = m
    spec.loader.exec_module(m)
    return m


wf = _abi()
f32p, i32p, u8p, f64p, i64p, u64p = wf.f32p, wf.i32p, wf.u8p, wf.f64p, wf.i64p, wf.u64p
ptr = wf.ptr
render_params = wf.render_params


def build_port() -> Path:
    subprocess.run(["make", "-s", "-C", str(HERE), "port"], check=True)
    return PORT_LIB


def build_ref() -> Path | None:
    if not (REF_SRC / "src" / "render" / "WavefrontRenderer.cpp").exists():
        return None
    subprocess.run(["make", "-s", "-C", str(HERE), "ref", f"REF={REF_SRC.resolve()}"], check=True)
    return REF_LIB


class OrcCounters(C.Structure):
    _fields_ = [("closest_rays", C.c_uint64), ("shadow_rays", C.c_uint64), ("shaded_hits", C.c_uint64),
                ("misses", C.c_uint64)]


_port = None


def port_lib() -> C.CDLL:
    global _port
    if _port is not None:
        return _port
    sources = [HERE / "wf_oracle.cpp", ROOT / "wavefront-renderer_gb300" / "csrc" / "wf_scenes.cpp"]
    if not PORT_LIB.exists() or PORT_LIB.stat().st_mtime < max(p.stat().st_mtime for p in sources):
        build_port()
    lib = C.CDLL(str(PORT_LIB))
    V = C.c_void_p
    sig = {
        "orc_scene_create": ([C.POINTER(wf.WfSceneDesc)], V),
        "orc_scene_destroy": ([V], None),
        "orc_scene_bounds": ([V, f32p, f32p], None),
        "orc_scene_total_emissive_area": ([V], C.c_float),
        "orc_philox4x32_10": ([C.POINTER(C.c_uint32), C.POINTER(C.c_uint32), C.POINTER(C.c_uint32)], None),
        "orc_camera_get_ray": ([C.POINTER(wf.WfCamera), C.c_float, C.c_float, f32p, f32p], None),
        "orc_generate_primary": ([C.POINTER(wf.WfCamera), C.c_int32, C.c_int32, C.c_uint32, C.c_uint32,
                                  C.c_int32, C.c_int32] + [f32p] * 6 + [i32p, i32p], None),
        "orc_trace_closest": ([V, C.c_int64] + [f32p] * 6 + [C.c_float, C.c_float, C.POINTER(wf.WfHitColumns)], None),
        "orc_trace_closest_brute": ([V, C.c_int64] + [f32p] * 6 + [C.c_float, C.c_float, C.POINTER(wf.WfHitColumns)], None),
        "orc_trace_occluded": ([V, C.c_int64] + [f32p] * 7 + [u8p], None),
        "orc_ray_sort_keys": ([C.c_int64] + [f32p] * 6 + [f32p, f32p, u64p], None),
        "orc_ray_schedule": ([C.c_int64] + [f32p] * 6 + [f32p, f32p, i32p], None),
        "orc_shading_schedule": ([C.c_int32, C.c_int64, i32p, i32p] + [f32p] * 6 +
                                 [C.c_int32, C.POINTER(wf.WfMaterial), C.c_int32, i64p, f64p, f64p, i32p], None),
        "orc_render_window": ([V, C.POINTER(wf.WfRenderParams), C.c_int32, C.c_int32, C.c_int32, C.c_int32,
                               C.c_int32, f32p, C.POINTER(OrcCounters)], None),
        "orc_render_window_counts": ([V, C.POINTER(wf.WfRenderParams), C.c_int32, C.c_int32, C.c_int32,
                                      C.c_int32, C.c_int32, f32p, i32p, C.POINTER(OrcCounters)], None),
        "orc_cost_tracker_relative": ([C.c_int32, C.c_int64, i32p, f64p, f64p], None),
        "wf_camera_make": ([f32p, f32p, f32p, C.c_float, C.c_int32, C.c_int32, C.POINTER(wf.WfCamera)], C.c_int),
        "wf_host_scene_generate": ([C.c_int32, C.c_uint64, C.POINTER(V)], C.c_int),
        "wf_host_scene_describe": ([V, C.POINTER(wf.WfSceneDesc)], C.c_int),
        "wf_host_scene_camera": ([V, C.c_int32, C.c_int32, C.POINTER(wf.WfCamera)], C.c_int),
        "wf_host_scene_free": ([V], C.c_int),
    }
    for name, (args, res) in sig.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = res
    _port = lib
    return lib


class HostScene:
    """A procedural workload built by the generator compiled into
    liboracle.so (the same source as the GPU library's wf_host_scene_*):
    0 Cornell box, 1 icosphere scene, 2 lattice, 3 Cornell variants, 100/102
    small variants, 104 Cornell box under a directional light."""

    def __init__(self, config: int, seed: int = 1):
        lib = port_lib()
        self._lib = lib
        self._h = C.c_void_p()
        if lib.wf_host_scene_generate(config, seed, C.byref(self._h)) != 0:
            raise RuntimeError(f"scene generator: config {config} failed")
        self.desc = wf.WfSceneDesc()
        lib.wf_host_scene_describe(self._h, C.byref(self.desc))
        self.config = config

    def camera(self, width: int, height: int):
        cam = wf.WfCamera()
        if self._lib.wf_host_scene_camera(self._h, width, height, C.byref(cam)) != 0:
            raise RuntimeError("scene camera failed")
        return cam

    def __del__(self):
        if getattr(self, "_h", None):
            self._lib.wf_host_scene_free(self._h)
            self._h = None


def camera_make(look_from, look_at, up, vfov, width, height):
    """Camera::Camera (include/core/Camera.h:13-33) as the oracle restates it."""
    cam = wf.WfCamera()
    a = [np.asarray(v, dtype=np.float32) for v in (look_from, look_at, up)]
    if port_lib().wf_camera_make(ptr(a[0]), ptr(a[1]), ptr(a[2]), vfov, width, height, C.byref(cam)) != 0:
        raise RuntimeError("camera_make failed")
    return cam


def _cols(a: np.ndarray) -> list:
    a = np.ascontiguousarray(a, dtype=np.float32)
    return [np.ascontiguousarray(a[:, k]) for k in range(3)]


class Port:
    """The oracle restatement over one scene."""

    def __init__(self, desc):
        self.lib = port_lib()
        self.h = self.lib.orc_scene_create(C.byref(desc))

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.orc_scene_destroy(self.h)
            self.h = None

    def bounds(self):
        bmin = np.zeros(3, np.float32)
        bmax = np.zeros(3, np.float32)
        self.lib.orc_scene_bounds(self.h, ptr(bmin), ptr(bmax))
        return bmin, bmax

    def total_emissive_area(self) -> float:
        return float(self.lib.orc_scene_total_emissive_area(self.h))

    def trace_closest(self, o, d, tmin=0.001, tmax=1e9, brute=False) -> dict:
        n = o.shape[0]
        cols, hc = wf.make_hit_columns(n)
        fn = self.lib.orc_trace_closest_brute if brute else self.lib.orc_trace_closest
        fn(self.h, n, *[ptr(x) for x in _cols(o) + _cols(d)], tmin, tmax, C.byref(hc))
        return cols

    def trace_occluded(self, o, d, maxd) -> np.ndarray:
        n = o.shape[0]
        out = np.zeros(n, np.uint8)
        maxd = np.ascontiguousarray(maxd, dtype=np.float32)
        self.lib.orc_trace_occluded(self.h, n, *[ptr(x) for x in _cols(o) + _cols(d)], ptr(maxd),
                                    ptr(out, C.c_uint8))
        return out

    def render_window(self, params, x0, y0, w, h, threads=0, counts=False):
        """Per-pixel sums of the window; with counts=True also each pixel's
        sample count (adaptive sampling stops pixels early)."""
        acc = np.zeros(w * h * 3, np.float32)
        cnt = OrcCounters()
        if counts:
            n = np.zeros(w * h, np.int32)
            self.lib.orc_render_window_counts(self.h, C.byref(params), x0, y0, w, h, threads, ptr(acc),
                                              ptr(n, C.c_int32), C.byref(cnt))
            return acc.reshape(h, w, 3), {k: getattr(cnt, k) for k, _ in OrcCounters._fields_}, n.reshape(h, w)
        self.lib.orc_render_window(self.h, C.byref(params), x0, y0, w, h, threads, ptr(acc), C.byref(cnt))
        return acc.reshape(h, w, 3), {k: getattr(cnt, k) for k, _ in OrcCounters._fields_}


def philox(ctr, key) -> np.ndarray:
    c = (C.c_uint32 * 4)(*ctr)
    k = (C.c_uint32 * 2)(*key)
    o = (C.c_uint32 * 4)()
    port_lib().orc_philox4x32_10(c, k, o)
    return np.array(list(o), dtype=np.uint32)


def camera_get_ray(cam, u, v):
    o = np.zeros(3, np.float32)
    d = np.zeros(3, np.float32)
    port_lib().orc_camera_get_ray(C.byref(cam), u, v, ptr(o), ptr(d))
    return o, d


def generate_primary(cam, w, h, seed, first_sample, nspp) -> dict:
    n = w * h * nspp
    cols = {k: np.zeros(n, np.float32) for k in ("ox", "oy", "oz", "dx", "dy", "dz")}
    pix = np.zeros(n, np.int32)
    smp = np.zeros(n, np.int32)
    port_lib().orc_generate_primary(C.byref(cam), w, h, seed & 0xFFFFFFFF, (seed >> 32) & 0xFFFFFFFF,
                                    first_sample, nspp, *[ptr(cols[k]) for k in ("ox", "oy", "oz", "dx", "dy", "dz")],
                                    ptr(pix, C.c_int32), ptr(smp, C.c_int32))
    cols["pixel"], cols["sample"] = pix, smp
    return cols


def ray_sort_keys(o, d, bmin, bmax) -> np.ndarray:
    n = o.shape[0]
    keys = np.zeros(n, np.uint64)
    port_lib().orc_ray_sort_keys(n, *[ptr(x) for x in _cols(o) + _cols(d)], ptr(np.asarray(bmin, np.float32)),
                                 ptr(np.asarray(bmax, np.float32)), ptr(keys, C.c_uint64))
    return keys


def ray_schedule(o, d, bmin, bmax) -> np.ndarray:
    n = o.shape[0]
    out = np.zeros(n, np.int32)
    port_lib().orc_ray_schedule(n, *[ptr(x) for x in _cols(o) + _cols(d)], ptr(np.asarray(bmin, np.float32)),
                                ptr(np.asarray(bmax, np.float32)), ptr(out, C.c_int32))
    return out


def shading_schedule(policy, mat_ids, tex_ids, thr, pts, materials, texture_bytes,
                     rel_cost_material=None, rel_cost_texture=None) -> np.ndarray:
    mat_ids = np.ascontiguousarray(mat_ids, np.int32)
    tex_ids = np.ascontiguousarray(tex_ids, np.int32)
    n = mat_ids.shape[0]
    out = np.zeros(n, np.int32)
    marr = (wf.WfMaterial * len(materials))(*materials)
    tb = np.ascontiguousarray(texture_bytes, np.int64)
    rcm = None if rel_cost_material is None else np.ascontiguousarray(rel_cost_material, np.float64)
    rct = None if rel_cost_texture is None else np.ascontiguousarray(rel_cost_texture, np.float64)
    port_lib().orc_shading_schedule(policy, n, ptr(mat_ids, C.c_int32), ptr(tex_ids, C.c_int32),
                                    *[ptr(x) for x in _cols(thr) + _cols(pts)], len(materials), marr, len(tb),
                                    ptr(tb, C.c_int64) if len(tb) else None, ptr(rcm, C.c_double),
                                    ptr(rct, C.c_double), ptr(out, C.c_int32))
    return out


def cost_tracker_relative(items, ids, costs, ref=False) -> np.ndarray:
    ids = np.ascontiguousarray(ids, np.int32)
    costs = np.ascontiguousarray(costs, np.float64)
    out = np.zeros(items, np.float64)
    if ref:
        ref_lib().ref_cost_tracker_relative(items, len(ids), ptr(ids, C.c_int32), ptr(costs, C.c_double),
                                            ptr(out, C.c_double))
    else:
        port_lib().orc_cost_tracker_relative(items, len(ids), ptr(ids, C.c_int32), ptr(costs, C.c_double),
                                             ptr(out, C.c_double))
    return out


# --------------------------------------------------------------------------
# The reference compiled in place (only where its checkout exists).
# --------------------------------------------------------------------------
_ref = None


def ref_available() -> bool:
    try:
        ref_lib()
        return True
    except RuntimeError:
        return False


def ref_lib() -> C.CDLL:
    global _ref
    if _ref is not None:
        return _ref
    if not REF_LIB.exists():
        if build_ref() is None:
            raise RuntimeError("reference sources not present; oracle/_ref cannot be built here")
    lib = C.CDLL(str(REF_LIB))
    V = C.c_void_p
    sig = {
        "ref_set_seed": ([C.c_ulonglong], None),
        "ref_set_threads": ([C.c_int], None),
        "ref_scene_create": ([C.POINTER(wf.WfSceneDesc), C.c_int], V),
        "ref_scene_destroy": ([V], None),
        "ref_scene_bounds": ([V, f32p, f32p], None),
        "ref_scene_total_emissive_area": ([V], C.c_float),
        "ref_camera": ([f32p, f32p, f32p, C.c_float, C.c_int, C.c_int, f32p], None),
        "ref_camera_get_ray": ([f32p, C.c_float, C.c_float, f32p, f32p], None),
        "ref_trace": ([V, C.c_int, C.c_longlong] + [f32p] * 6 + [C.c_float, C.c_float, C.POINTER(wf.WfHitColumns)], None),
        "ref_occluded": ([V, C.c_longlong] + [f32p] * 7 + [u8p], None),
        "ref_intersect_triangle": ([f32p] * 5 + [C.c_float, C.c_float, f32p], C.c_int),
        "ref_ray_schedule": ([C.c_longlong] + [f32p] * 6 + [f32p, f32p, i32p, C.POINTER(C.c_ulonglong)], None),
        "ref_cost_tracker_relative": ([C.c_int, C.c_longlong, i32p, f64p, f64p], None),
        "ref_shading_schedule": ([C.c_int, C.c_longlong, i32p, i32p] + [f32p] * 6 +
                                 [C.c_int, C.POINTER(wf.WfMaterial), C.c_int, i32p,
                                  C.c_longlong, i32p, f64p, C.c_longlong, i32p, f64p, C.c_int, i32p], None),
        "ref_render": ([V, f32p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_float, C.c_char_p, f32p],
                       None),
        "ref_render_adaptive": ([V, f32p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_float, f32p], None),
        "ref_front_face_stats": ([C.POINTER(C.c_longlong), C.POINTER(C.c_longlong)], None),
    }
    for name, (args, res) in sig.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = res
    _ref = lib
    return lib


class Ref:
    """The reference's Scene + EmbreeAccelerator stand-in over one scene."""

    def __init__(self, desc, build_accelerator=True):
        self.lib = ref_lib()
        self.h = self.lib.ref_scene_create(C.byref(desc), int(build_accelerator))

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.ref_scene_destroy(self.h)
            self.h = None

    def bounds(self):
        bmin = np.zeros(3, np.float32)
        bmax = np.zeros(3, np.float32)
        self.lib.ref_scene_bounds(self.h, ptr(bmin), ptr(bmax))
        return bmin, bmax

    def trace(self, o, d, tmin=0.001, tmax=1e9, mode=1) -> dict:
        n = o.shape[0]
        cols, hc = wf.make_hit_columns(n)
        self.lib.ref_trace(self.h, mode, n, *[ptr(x) for x in _cols(o) + _cols(d)], tmin, tmax, C.byref(hc))
        return cols

    def occluded(self, o, d, maxd) -> np.ndarray:
        n = o.shape[0]
        out = np.zeros(n, np.uint8)
        self.lib.ref_occluded(self.h, n, *[ptr(x) for x in _cols(o) + _cols(d)],
                              ptr(np.ascontiguousarray(maxd, np.float32)), ptr(out, C.c_uint8))
        return out

    def render(self, cam12, w, h, spp, max_depth, policy=0, ray_sort=False, firefly=10.0, seed=1, threads=0,
               env_path=None):
        """env_path: a PFM (write_pfm) loaded as the renderer's environment map."""
        if threads:
            self.lib.ref_set_threads(threads)
        self.lib.ref_set_seed(seed)
        img = np.zeros(w * h * 3, np.float32)
        cam12 = np.ascontiguousarray(cam12, np.float32)
        env = str(env_path).encode() if env_path else None
        self.lib.ref_render(self.h, ptr(cam12), w, h, spp, max_depth, policy, int(ray_sort), firefly, env, ptr(img))
        return img.reshape(h, w, 3)


    def render_adaptive(self, cam12, w, h, spp, max_depth, threshold=0.05, seed=1, threads=0):
        """renderScene with the reference's AdaptiveSampler on."""
        if threads:
            self.lib.ref_set_threads(threads)
        self.lib.ref_set_seed(seed)
        img = np.zeros(w * h * 3, np.float32)
        cam12 = np.ascontiguousarray(cam12, np.float32)
        self.lib.ref_render_adaptive(self.h, ptr(cam12), w, h, spp, max_depth, threshold, ptr(img))
        return img.reshape(h, w, 3)


def ref_front_face_stats() -> tuple[int, int]:
    """(unresolved, ambiguous) rebuilt-record frontFace lookups of the last
    reference render (shims/core/HitRecord.h); unresolved must be 0."""
    a, b = C.c_longlong(), C.c_longlong()
    ref_lib().ref_front_face_stats(C.byref(a), C.byref(b))
    return a.value, b.value


def write_pfm(path, rgb: np.ndarray) -> None:
    """Writes an (h, w, 3) float image, top row first in memory, as a
    little-endian PFM (rows stored bottom to top)."""
    rgb = np.ascontiguousarray(rgb, np.float32)
    h, w, _ = rgb.shape
    with open(path, "wb") as f:
        f.write(f"PF\n{w} {h}\n-1.0\n".encode())
        f.write(rgb[::-1].astype("<f4").tobytes())


def scene_environment(desc) -> np.ndarray | None:
    """The (h, w, 3) environment map of a wf_scene_desc, or None."""
    e = desc.environment
    if e.width <= 0 or not e.rgb:
        return None
    return np.ctypeslib.as_array(e.rgb, shape=(e.height * e.width * 3,)).reshape(e.height, e.width, 3).copy()


def ref_camera(look_from, look_at, up, vfov, w, h) -> np.ndarray:
    out = np.zeros(12, np.float32)
    a = [np.asarray(v, np.float32) for v in (look_from, look_at, up)]
    ref_lib().ref_camera(ptr(a[0]), ptr(a[1]), ptr(a[2]), vfov, w, h, ptr(out))
    return out


def ref_camera_get_ray(cam12, u, v):
    o = np.zeros(3, np.float32)
    d = np.zeros(3, np.float32)
    ref_lib().ref_camera_get_ray(ptr(np.ascontiguousarray(cam12, np.float32)), u, v, ptr(o), ptr(d))
    return o, d


def ref_ray_schedule(o, d, bmin, bmax):
    n = o.shape[0]
    out = np.zeros(n, np.int32)
    keys = np.zeros(n, np.uint64)
    ref_lib().ref_ray_schedule(n, *[ptr(x) for x in _cols(o) + _cols(d)], ptr(np.asarray(bmin, np.float32)),
                               ptr(np.asarray(bmax, np.float32)), ptr(out, C.c_int32), ptr(keys, C.c_ulonglong))
    return out, keys


def ref_shading_schedule(policy, mat_ids, tex_ids, thr, pts, materials, tex_wh, mat_samples=None,
                         tex_samples=None, use_trackers=True) -> np.ndarray:
    mat_ids = np.ascontiguousarray(mat_ids, np.int32)
    tex_ids = np.ascontiguousarray(tex_ids, np.int32)
    n = mat_ids.shape[0]
    out = np.zeros(n, np.int32)
    marr = (wf.WfMaterial * len(materials))(*materials)
    wh = np.ascontiguousarray(np.asarray(tex_wh, np.int32).reshape(-1))
    ms_ids, ms_ns = mat_samples if mat_samples is not None else (np.zeros(0, np.int32), np.zeros(0))
    ts_ids, ts_ns = tex_samples if tex_samples is not None else (np.zeros(0, np.int32), np.zeros(0))
    ms_ids = np.ascontiguousarray(ms_ids, np.int32)
    ms_ns = np.ascontiguousarray(ms_ns, np.float64)
    ts_ids = np.ascontiguousarray(ts_ids, np.int32)
    ts_ns = np.ascontiguousarray(ts_ns, np.float64)
    ref_lib().ref_shading_schedule(policy, n, ptr(mat_ids, C.c_int32), ptr(tex_ids, C.c_int32),
                                   *[ptr(x) for x in _cols(thr) + _cols(pts)], len(materials), marr,
                                   len(wh) // 2, ptr(wh, C.c_int32) if len(wh) else None,
                                   len(ms_ids), ptr(ms_ids, C.c_int32), ptr(ms_ns, C.c_double),
                                   len(ts_ids), ptr(ts_ids, C.c_int32), ptr(ts_ns, C.c_double),
                                   int(use_trackers), ptr(out, C.c_int32))
    return out


def ref_intersect_triangle(o, d, v0, v1, v2, tmin, tmax):
    out = np.zeros(3, np.float32)
    a = [np.asarray(x, np.float32) for x in (o, d, v0, v1, v2)]
    hit = ref_lib().ref_intersect_triangle(*[ptr(x) for x in a], tmin, tmax, ptr(out))
    return bool(hit), out
