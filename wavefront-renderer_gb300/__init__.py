"""Python bindings of libwfgpu.so (the C ABI in include/wf_api.h).

The GB300 wavefront path tracer is a C ABI shared library; this module only
loads it with ctypes and wraps the entry points with numpy-friendly calls.
There is no Python or CPU fallback: if the library is missing or no CUDA
device is visible, the calls raise.

Import it by path (the directory name is not a Python identifier):

    import importlib.util, pathlib
    spec = importlib.util.spec_from_file_location(
        "wavefront_gb300", pathlib.Path("wavefront-renderer_gb300/__init__.py"))
"""
from __future__ import annotations

import ctypes as C
import os
import weakref
from pathlib import Path

import numpy as np

PKG_DIR = Path(__file__).resolve().parent
LIB_PATH = PKG_DIR / "lib" / "libwfgpu.so"
HEADER = PKG_DIR.parent / "include" / "wf_api.h"

_ABI_PATH = PKG_DIR.parent / "include" / "wf_abi.py"


def _load_abi():
    import importlib.util
    import sys

    if "wf_abi" in sys.modules:
        return sys.modules["wf_abi"]
    spec = importlib.util.spec_from_file_location("wf_abi", _ABI_PATH)
    mod = importlib.util.module_from_spec(spec)
    sys.modules["wf_abi"] = mod
    spec.loader.exec_module(mod)
    return mod


abi = _load_abi()
globals().update({k: v for k, v in vars(abi).items() if not k.startswith("__") and k not in ("C", "np")})

_lib = None


def load_library(path: str | os.PathLike | None = None) -> C.CDLL:
    """Loads libwfgpu.so; raises if it has not been built."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise RuntimeError(f"{p} not built: run __graft_entry__.build() (nvcc, sm_103a)")
    lib = C.CDLL(str(p))
    _declare(lib)
    if path is None:
        _lib = lib
    return lib


def _declare(lib: C.CDLL) -> None:
    V = C.c_void_p
    sig = {
        "wf_version": ([], C.c_int),
        "wf_create": ([C.POINTER(WfConfig), C.POINTER(V)], C.c_int),
        "wf_destroy": ([V], C.c_int),
        "wf_last_error": ([V], C.c_char_p),
        "wf_camera_make": ([f32p, f32p, f32p, C.c_float, C.c_int32, C.c_int32, C.POINTER(WfCamera)], C.c_int),
        "wf_scene_upload": ([V, C.POINTER(WfSceneDesc)], C.c_int),
        "wf_scene_get_info": ([V, C.POINTER(WfSceneInfo)], C.c_int),
        "wf_trace_closest_host": ([V, C.c_int64] + [f32p] * 6 + [C.c_float, C.c_float, C.POINTER(WfHitColumns)], C.c_int),
        "wf_trace_occluded_host": ([V, C.c_int64] + [f32p] * 7 + [u8p], C.c_int),
        "wf_generate_primary_host": ([V, C.POINTER(WfCamera), C.c_int32, C.c_int32, C.c_uint32, C.c_uint32,
                                      C.c_int32, C.c_int32] + [f32p] * 6 + [i32p, i32p], C.c_int),
        "wf_ray_schedule_static": ([V, C.c_int64] + [C.c_void_p] * 6 + [f32p, f32p, C.c_void_p, C.c_void_p], C.c_int),
        "wf_ray_schedule_host": ([V, C.c_int64] + [f32p] * 6 + [f32p, f32p, i32p, u64p], C.c_int),
        "wf_shading_schedule_host": ([V, C.c_int32, C.c_int64, i32p, i32p] + [f32p] * 6 +
                                     [C.c_int32, C.POINTER(WfMaterial), C.c_int32, i64p, f64p, f64p, i32p], C.c_int),
        "wf_render": ([V, C.POINTER(WfRenderParams), f32p, C.POINTER(WfRenderStats)], C.c_int),
        "wf_render_accumulate": ([V, C.POINTER(WfRenderParams), f32p, C.POINTER(WfRenderStats)], C.c_int),
        "wf_render_device": ([V, C.POINTER(WfRenderParams), C.POINTER(WfRenderStats)], C.c_int),
        "wf_image_download": ([V, f32p, C.c_int64], C.c_int),
        "wf_host_alloc": ([C.c_size_t, C.POINTER(V)], C.c_int),
        "wf_host_free": ([V], C.c_int),
        "wf_adaptive_sample_counts": ([V, i32p, C.c_int64], C.c_int),
        "wf_autotune": ([V, C.POINTER(WfRenderParams), C.POINTER(WfTuning), C.POINTER(C.c_double)], C.c_int),
        "wf_scene_save": ([C.c_char_p, C.POINTER(WfSceneDesc), f32p, f32p, f32p, C.c_float], C.c_int),
        "wf_scene_load": ([C.c_char_p, C.POINTER(V)], C.c_int),
        "wf_image_write_pfm": ([C.c_char_p, f32p, C.c_int32, C.c_int32], C.c_int),
        "wf_cost_tracker_state": ([V, f64p, C.c_int32, f64p, C.c_int32], C.c_int),
        "wf_cost_tracker_replay": ([V, C.c_int32, C.c_int32, C.POINTER(C.c_uint64), C.POINTER(C.c_uint32), f64p],
                                   C.c_int),
        "wf_get_stream": ([V, C.POINTER(V)], C.c_int),
        "wf_timer_begin": ([V], C.c_int),
        "wf_set_tuning": ([V, C.POINTER(WfTuning)], C.c_int),
        "wf_scene_add": ([V, C.POINTER(WfSceneDesc), C.POINTER(C.c_int32)], C.c_int),
        "wf_scene_remove": ([V, C.c_int32], C.c_int),
        "wf_scene_get_info_id": ([V, C.c_int32, C.POINTER(WfSceneInfo)], C.c_int),
        "wf_render_batch": ([V, C.POINTER(WfJob), C.c_int32, C.POINTER(f32p), C.POINTER(WfRenderStats)], C.c_int),
        "wf_server_create": ([V, C.POINTER(WfServerConfig), C.POINTER(V)], C.c_int),
        "wf_server_destroy": ([V], C.c_int),
        "wf_server_submit": ([V, C.POINTER(WfJob), C.POINTER(C.c_int64)], C.c_int),
        "wf_server_step": ([V, C.POINTER(WfServerStepInfo)], C.c_int),
        "wf_server_status": ([V, C.c_int64, C.POINTER(WfJobStatus)], C.c_int),
        "wf_server_image": ([V, C.c_int64, f32p, C.c_int64], C.c_int),
        "wf_server_cancel": ([V, C.c_int64], C.c_int),
        "wf_server_clock": ([V], C.c_double),
        "wf_get_tuning": ([V, C.POINTER(WfTuning)], C.c_int),
        "wf_timer_end": ([V, f64p], C.c_int),
        "wf_host_scene_generate": ([C.c_int32, C.c_uint64, C.POINTER(V)], C.c_int),
        "wf_host_scene_describe": ([V, C.POINTER(WfSceneDesc)], C.c_int),
        "wf_host_scene_camera": ([V, C.c_int32, C.c_int32, C.POINTER(WfCamera)], C.c_int),
        "wf_host_scene_free": ([V], C.c_int),
        "wf_ray_queue_alloc": ([V, C.c_int64, C.POINTER(V)], C.c_int),
        "wf_ray_queue_free": ([V], C.c_int),
        "wf_shading_queue_alloc": ([V, C.c_int64, C.POINTER(V)], C.c_int),
        "wf_shading_queue_free": ([V], C.c_int),
        "wf_shadow_queue_alloc": ([V, C.c_int64, C.POINTER(V)], C.c_int),
        "wf_shadow_queue_free": ([V], C.c_int),
        "wf_ray_queue_size": ([V, C.POINTER(C.c_int64)], C.c_int),
        "wf_shading_queue_size": ([V, C.POINTER(C.c_int64)], C.c_int),
        "wf_shadow_queue_size": ([V, C.POINTER(C.c_int64)], C.c_int),
        "wf_ray_queue_upload": ([V, C.POINTER(WfRayColumns), C.c_int64], C.c_int),
        "wf_ray_queue_download": ([V, C.POINTER(WfRayColumns), C.c_int64, C.POINTER(C.c_int64)], C.c_int),
        "wf_shading_queue_download": ([V, C.POINTER(WfHitColumns), C.POINTER(WfRayColumns), C.c_int64,
                                       C.POINTER(C.c_int64)], C.c_int),
        "wf_stage_begin": ([V, C.POINTER(WfRenderParams)], C.c_int),
        "wf_generate_primary": ([V, C.c_int32, C.c_int32, V], C.c_int),
        "wf_ray_queue_schedule": ([V, f32p, f32p, i32p], C.c_int),
        "wf_ray_queue_materialize": ([V], C.c_int),
        "wf_intersect": ([V, V, V, V], C.c_int),
        "wf_shading_queue_schedule": ([V, C.c_int32, f64p, f64p, i32p], C.c_int),
        "wf_shading_queue_materialize": ([V], C.c_int),
        "wf_shade": ([V, V, V, V], C.c_int),
        "wf_trace_occluded": ([V, V], C.c_int),
        "wf_miss": ([V, V], C.c_int),
        "wf_stage_image": ([V, f32p, C.c_int64], C.c_int),
    }
    for name, (args, res) in sig.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = res


def header_symbols() -> list[str]:
    """Every function the C header declares."""
    import re
    text = HEADER.read_text()
    return sorted(set(re.findall(r"^(?:int|const char\*|void|double)\s+(wf_\w+)\s*\(", text, re.M)))


class WfError(RuntimeError):
    pass


def host_array(count: int, dtype=np.float32) -> np.ndarray:
    """A 1-D numpy array of `count` elements in page-locked host memory
    (wf_host_alloc); the memory is released when the array is collected."""
    import weakref

    dt = np.dtype(dtype)
    p = C.c_void_p()
    _check(load_library().wf_host_alloc(C.c_size_t(count * dt.itemsize), C.byref(p)), "wf_host_alloc")
    raw = (C.c_uint8 * (count * dt.itemsize)).from_address(p.value)
    weakref.finalize(raw, load_library().wf_host_free, C.c_void_p(p.value))
    return np.frombuffer(raw, dtype=dt, count=count)


def _check(rc: int, what: str, ctx=None) -> None:
    if rc != WF_OK:
        msg = ""
        if ctx is not None and ctx._h:
            msg = (load_library().wf_last_error(ctx._h) or b"").decode()
        raise WfError(f"{what} failed: {ERRORS.get(rc, rc)} {msg}")


def save_scene(path, desc: WfSceneDesc, look_from, look_at, up, vfov: float) -> None:
    """Writes a scene description and its default camera (wf_scene_save)."""
    v = [(C.c_float * 3)(*map(float, x)) for x in (look_from, look_at, up)]
    _check(load_library().wf_scene_save(str(path).encode(), C.byref(desc), v[0], v[1], v[2], float(vfov)),
           "wf_scene_save")


def write_pfm(path, image: np.ndarray) -> None:
    """An (h, w, 3) float image, top row first, as a PFM (wf_image_write_pfm)."""
    img = np.ascontiguousarray(image, np.float32)
    h, w, _ = img.shape
    _check(load_library().wf_image_write_pfm(str(path).encode(), ptr(img), w, h), "wf_image_write_pfm")


class HostScene:
    """A procedural workload (wf_host_scene_*): 0 Cornell box, 1 icosphere
    scene (1.31 M triangles), 100 the icosphere scene at subdivision 4."""

    def __init__(self, config: int, seed: int = 1, *, _handle: C.c_void_p | None = None):
        lib = load_library()
        if _handle is None:
            self._h = C.c_void_p()
            _check(lib.wf_host_scene_generate(config, seed, C.byref(self._h)), "wf_host_scene_generate")
        else:
            self._h = _handle
        self.desc = WfSceneDesc()
        _check(lib.wf_host_scene_describe(self._h, C.byref(self.desc)), "wf_host_scene_describe")
        self.config = config

    @classmethod
    def load(cls, path) -> "HostScene":
        """A scene file written by save_scene (wf_scene_load)."""
        h = C.c_void_p()
        _check(load_library().wf_scene_load(str(path).encode(), C.byref(h)), "wf_scene_load")
        return cls(-1, _handle=h)

    def save(self, path, look_from, look_at, up, vfov) -> None:
        save_scene(path, self.desc, look_from, look_at, up, vfov)

    def camera(self, width: int, height: int) -> WfCamera:
        cam = WfCamera()
        _check(load_library().wf_host_scene_camera(self._h, width, height, C.byref(cam)), "camera")
        return cam

    def arrays(self) -> dict:
        d = self.desc
        nv, ni, nm = d.num_vertices, d.num_indices, d.num_meshes
        return {
            "px": np.ctypeslib.as_array(d.positions_x, (nv,)).copy(),
            "py": np.ctypeslib.as_array(d.positions_y, (nv,)).copy(),
            "pz": np.ctypeslib.as_array(d.positions_z, (nv,)).copy(),
            "indices": np.ctypeslib.as_array(d.indices, (ni,)).copy(),
            "mesh_offsets": np.ctypeslib.as_array(d.mesh_index_offsets, (nm,)).copy(),
            "mesh_counts": np.ctypeslib.as_array(d.mesh_index_counts, (nm,)).copy(),
            "mesh_materials": np.ctypeslib.as_array(d.mesh_material_ids, (nm,)).copy(),
            "materials": [d.materials[i] for i in range(d.num_materials)],
        }

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.wf_host_scene_free(self._h)
            self._h = None


def camera_make(look_from, look_at, up, vfov, width, height) -> WfCamera:
    cam = WfCamera()
    a = [np.asarray(v, dtype=np.float32) for v in (look_from, look_at, up)]
    _check(load_library().wf_camera_make(ptr(a[0]), ptr(a[1]), ptr(a[2]), vfov, width, height, C.byref(cam)),
           "wf_camera_make")
    return cam


class Server:
    """The serving loop (wf_server_*): admission by HBM budget, a streaming
    wave (a fixed-capacity ray queue refilled with new camera rays as paths
    end, 8 bounce iterations per step), progressive frames every frame_spp
    samples."""

    def __init__(self, ctx: "Context", hbm_budget_bytes: int, frame_spp: int = 8, max_paths_per_wave: int = 0):
        self.ctx = ctx
        self._h = C.c_void_p()
        cfg = WfServerConfig(hbm_budget_bytes, max_paths_per_wave, frame_spp)
        _check(load_library().wf_server_create(ctx._h, C.byref(cfg), C.byref(self._h)), "wf_server_create", ctx)
        ctx._children.add(self)

    def close(self):
        if self._h:
            load_library().wf_server_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def submit(self, job: WfJob) -> int:
        jid = C.c_int64()
        _check(load_library().wf_server_submit(self._h, C.byref(job), C.byref(jid)), "wf_server_submit", self.ctx)
        return jid.value

    def step(self) -> dict:
        info = WfServerStepInfo()
        _check(load_library().wf_server_step(self._h, C.byref(info)), "wf_server_step", self.ctx)
        return info.as_dict()

    def status(self, jid: int) -> dict:
        st = WfJobStatus()
        _check(load_library().wf_server_status(self._h, jid, C.byref(st)), "wf_server_status", self.ctx)
        return st.as_dict()

    def image(self, jid: int, width: int, height: int) -> np.ndarray:
        img = np.zeros(width * height * 3, np.float32)
        _check(load_library().wf_server_image(self._h, jid, ptr(img), img.size), "wf_server_image", self.ctx)
        return img.reshape(height, width, 3)

    def cancel(self, jid: int) -> None:
        _check(load_library().wf_server_cancel(self._h, jid), "wf_server_cancel", self.ctx)

    def clock(self) -> float:
        return load_library().wf_server_clock(self._h)


class _DeviceQueue:
    """A queue in device memory (wf_*_queue_alloc); freed by close()."""

    _kind = ""

    def __init__(self, ctx: "Context", capacity: int):
        self.ctx = ctx
        self.capacity = int(capacity)
        self._h = C.c_void_p()
        _check(getattr(load_library(), f"wf_{self._kind}_queue_alloc")(ctx._h, self.capacity, C.byref(self._h)),
               f"wf_{self._kind}_queue_alloc", ctx)
        ctx._children.add(self)

    def close(self):
        if self._h:
            getattr(load_library(), f"wf_{self._kind}_queue_free")(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def size(self) -> int:
        n = C.c_int64()
        _check(getattr(load_library(), f"wf_{self._kind}_queue_size")(self._h, C.byref(n)),
               f"wf_{self._kind}_queue_size", self.ctx)
        return n.value


class RayQueue(_DeviceQueue):
    """A RayQueue in device memory (RayQueue.h:63-245)."""

    _kind = "ray"

    def upload(self, cols: dict) -> None:
        """cols: RAY_FIELDS arrays (origins, directions and pixel indices
        required; the others default as RayQueue::addPrimary sets them)."""
        n = len(cols["origins_x"])
        keep, rc = make_ray_columns(n, cols)
        _check(load_library().wf_ray_queue_upload(self._h, C.byref(rc), n), "wf_ray_queue_upload", self.ctx)

    def download(self) -> dict:
        n = self.size()
        cols, rc = make_ray_columns(n)
        got = C.c_int64()
        _check(load_library().wf_ray_queue_download(self._h, C.byref(rc), n, C.byref(got)), "wf_ray_queue_download",
               self.ctx)
        return {k: v[:got.value] for k, v in cols.items()}

    def schedule(self, bounds_min, bounds_max) -> np.ndarray:
        """RayQueue::schedule: the permutation (sortedIndices), also kept in
        the queue for materialize()."""
        n = self.size()
        perm = np.zeros(max(n, 1), np.int32)
        bmin = np.ascontiguousarray(bounds_min, np.float32)
        bmax = np.ascontiguousarray(bounds_max, np.float32)
        _check(load_library().wf_ray_queue_schedule(self._h, ptr(bmin), ptr(bmax), ptr(perm, C.c_int32)),
               "wf_ray_queue_schedule", self.ctx)
        return perm[:n]

    def materialize(self) -> None:
        _check(load_library().wf_ray_queue_materialize(self._h), "wf_ray_queue_materialize", self.ctx)


class ShadingQueue(_DeviceQueue):
    """A ShadingQueue in device memory (ShadingQueue.h:27-551)."""

    _kind = "shading"

    def download(self) -> tuple[dict, dict]:
        """The queue's hit columns (HIT_FIELDS) and its rays' columns
        (RAY_FIELDS), in queue order."""
        n = self.size()
        hits, hc = make_hit_columns(n)
        rays, rc = make_ray_columns(n)
        got = C.c_int64()
        _check(load_library().wf_shading_queue_download(self._h, C.byref(hc), C.byref(rc), n, C.byref(got)),
               "wf_shading_queue_download", self.ctx)
        return hits, rays

    def schedule(self, policy: int, rel_cost_material=None, rel_cost_texture=None) -> np.ndarray:
        n = self.size()
        perm = np.zeros(max(n, 1), np.int32)
        rcm = None if rel_cost_material is None else np.ascontiguousarray(rel_cost_material, np.float64)
        rct = None if rel_cost_texture is None else np.ascontiguousarray(rel_cost_texture, np.float64)
        _check(load_library().wf_shading_queue_schedule(self._h, policy, ptr(rcm, C.c_double), ptr(rct, C.c_double),
                                                        ptr(perm, C.c_int32)), "wf_shading_queue_schedule", self.ctx)
        return perm[:n]

    def materialize(self) -> None:
        _check(load_library().wf_shading_queue_materialize(self._h), "wf_shading_queue_materialize", self.ctx)


class ShadowQueue(_DeviceQueue):
    """The shadow rays of one bounce, in device memory."""

    _kind = "shadow"


class Context:
    """A device context (wf_create): one CUDA stream, a resident scene."""

    def __init__(self, device: int = 0, max_paths_per_wave: int = 0):
        lib = load_library()
        self._h = C.c_void_p()
        # servers and device queues made on this context: closed before it,
        # whatever still refers to them (the C API wants them destroyed first)
        self._children = weakref.WeakSet()
        cfg = WfConfig(device, max_paths_per_wave)
        rc = lib.wf_create(C.byref(cfg), C.byref(self._h))
        _check(rc, "wf_create")

    def close(self):
        if self._h:
            for child in list(self._children):
                child.close()
            load_library().wf_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def upload(self, desc: WfSceneDesc) -> WfSceneInfo:
        lib = load_library()
        _check(lib.wf_scene_upload(self._h, C.byref(desc)), "wf_scene_upload", self)
        info = WfSceneInfo()
        _check(lib.wf_scene_get_info(self._h, C.byref(info)), "wf_scene_get_info", self)
        return info

    def trace_closest(self, o: np.ndarray, d: np.ndarray, tmin=0.001, tmax=1e9) -> dict:
        o = np.ascontiguousarray(o, dtype=np.float32)
        d = np.ascontiguousarray(d, dtype=np.float32)
        n = o.shape[0]
        cols, hc = make_hit_columns(n)
        oc = [np.ascontiguousarray(o[:, k]) for k in range(3)]
        dc = [np.ascontiguousarray(d[:, k]) for k in range(3)]
        _check(load_library().wf_trace_closest_host(self._h, n, *[ptr(x) for x in oc + dc], tmin, tmax,
                                                    C.byref(hc)), "wf_trace_closest_host", self)
        return cols

    def trace_occluded(self, o: np.ndarray, d: np.ndarray, maxd: np.ndarray) -> np.ndarray:
        o = np.ascontiguousarray(o, dtype=np.float32)
        d = np.ascontiguousarray(d, dtype=np.float32)
        maxd = np.ascontiguousarray(maxd, dtype=np.float32)
        n = o.shape[0]
        out = np.zeros(n, dtype=np.uint8)
        oc = [np.ascontiguousarray(o[:, k]) for k in range(3)]
        dc = [np.ascontiguousarray(d[:, k]) for k in range(3)]
        _check(load_library().wf_trace_occluded_host(self._h, n, *[ptr(x) for x in oc + dc], ptr(maxd),
                                                     ptr(out, C.c_uint8)), "wf_trace_occluded_host", self)
        return out

    def generate_primary(self, cam: WfCamera, w: int, h: int, seed: int, first_sample: int, nspp: int) -> dict:
        n = w * h * nspp
        cols = {k: np.zeros(n, dtype=np.float32) for k in ("ox", "oy", "oz", "dx", "dy", "dz")}
        pix = np.zeros(n, dtype=np.int32)
        smp = np.zeros(n, dtype=np.int32)
        _check(load_library().wf_generate_primary_host(
            self._h, C.byref(cam), w, h, seed & 0xFFFFFFFF, (seed >> 32) & 0xFFFFFFFF, first_sample, nspp,
            *[ptr(cols[k]) for k in ("ox", "oy", "oz", "dx", "dy", "dz")], ptr(pix, C.c_int32),
            ptr(smp, C.c_int32)), "wf_generate_primary_host", self)
        cols["pixel"], cols["sample"] = pix, smp
        return cols

    def ray_schedule(self, o, d, bmin, bmax):
        o = np.ascontiguousarray(o, dtype=np.float32)
        d = np.ascontiguousarray(d, dtype=np.float32)
        n = o.shape[0]
        out = np.zeros(n, dtype=np.int32)
        keys = np.zeros(n, dtype=np.uint64)
        bmin = np.asarray(bmin, dtype=np.float32)
        bmax = np.asarray(bmax, dtype=np.float32)
        oc = [np.ascontiguousarray(o[:, k]) for k in range(3)]
        dc = [np.ascontiguousarray(d[:, k]) for k in range(3)]
        _check(load_library().wf_ray_schedule_host(self._h, n, *[ptr(x) for x in oc + dc], ptr(bmin), ptr(bmax),
                                                   ptr(out, C.c_int32), ptr(keys, C.c_uint64)),
               "wf_ray_schedule_host", self)
        return out, keys

    def shading_schedule(self, policy, mat_ids, tex_ids, thr, pts, materials, texture_bytes,
                         rel_cost_material=None, rel_cost_texture=None) -> np.ndarray:
        mat_ids = np.ascontiguousarray(mat_ids, dtype=np.int32)
        tex_ids = np.ascontiguousarray(tex_ids, dtype=np.int32)
        thr = np.ascontiguousarray(thr, dtype=np.float32)
        pts = np.ascontiguousarray(pts, dtype=np.float32)
        n = mat_ids.shape[0]
        out = np.zeros(n, dtype=np.int32)
        marr = (WfMaterial * len(materials))(*materials)
        tb = np.ascontiguousarray(texture_bytes, dtype=np.int64)
        cols = [np.ascontiguousarray(thr[:, k]) for k in range(3)] + [np.ascontiguousarray(pts[:, k]) for k in range(3)]
        rcm = None if rel_cost_material is None else np.ascontiguousarray(rel_cost_material, dtype=np.float64)
        rct = None if rel_cost_texture is None else np.ascontiguousarray(rel_cost_texture, dtype=np.float64)
        _check(load_library().wf_shading_schedule_host(
            self._h, policy, n, ptr(mat_ids, C.c_int32), ptr(tex_ids, C.c_int32), *[ptr(c) for c in cols],
            len(materials), marr, len(tb), ptr(tb, C.c_int64) if len(tb) else None,
            ptr(rcm, C.c_double), ptr(rct, C.c_double), ptr(out, C.c_int32)), "wf_shading_schedule_host", self)
        return out

    def render_device(self, params: WfRenderParams) -> dict:
        st = WfRenderStats()
        _check(load_library().wf_render_device(self._h, C.byref(params), C.byref(st)), "wf_render_device", self)
        return st.as_dict()

    def image_download(self, width: int, height: int, out: np.ndarray | None = None) -> np.ndarray:
        img = out if out is not None else np.zeros(width * height * 3, dtype=np.float32)
        _check(load_library().wf_image_download(self._h, ptr(img), img.size), "wf_image_download", self)
        return img.reshape(height, width, 3)

    def sample_counts(self, width: int, height: int) -> np.ndarray:
        """Per-pixel sample counts of the last render (adaptive sampling)."""
        n = np.zeros(width * height, dtype=np.int32)
        _check(load_library().wf_adaptive_sample_counts(self._h, ptr(n, C.c_int32), n.size),
               "wf_adaptive_sample_counts", self)
        return n.reshape(height, width)

    def cost_tracker_state(self, num_materials: int, num_textures: int) -> tuple[np.ndarray, np.ndarray]:
        """relativeCost per material and per texture of the live trackers."""
        m = np.zeros(max(num_materials, 1), np.float64)
        t = np.zeros(max(num_textures, 1), np.float64)
        _check(load_library().wf_cost_tracker_state(self._h, ptr(m, C.c_double), num_materials,
                                                    ptr(t, C.c_double) if num_textures else None, num_textures),
               "wf_cost_tracker_state", self)
        return m[:num_materials], t[:num_textures]

    def cost_tracker_replay(self, sums: np.ndarray, counts: np.ndarray) -> np.ndarray:
        """Feeds (steps, items) cycle sums and counts through the device
        CostTracker; returns relativeCost per item."""
        sums = np.ascontiguousarray(sums, np.uint64)
        counts = np.ascontiguousarray(counts, np.uint32)
        steps, items = sums.shape
        out = np.zeros(items, np.float64)
        _check(load_library().wf_cost_tracker_replay(self._h, items, steps, ptr(sums, C.c_uint64),
                                                     ptr(counts, C.c_uint32), ptr(out, C.c_double)),
               "wf_cost_tracker_replay", self)
        return out

    def set_tuning(self, trace_variant: int = 0, persistent_blocks_per_sm: int = 0, graph_mode: int = 0,
                   bvh_builder: int = 0, sort_min_queue: int = 0, ray_sort_bits: int = 0) -> None:
        t = WfTuning(trace_variant, persistent_blocks_per_sm, graph_mode, bvh_builder, sort_min_queue, 0, 0,
                     ray_sort_bits)
        _check(load_library().wf_set_tuning(self._h, C.byref(t)), "wf_set_tuning", self)

    def autotune(self, params: WfRenderParams) -> tuple[dict, float]:
        """wf_autotune: the fastest launch tuning for one wave of params
        (kept on the context) and its device time per wave in ms."""
        t = WfTuning()
        ms = C.c_double()
        _check(load_library().wf_autotune(self._h, C.byref(params), C.byref(t), C.byref(ms)), "wf_autotune", self)
        return self.get_tuning(), ms.value

    def get_tuning(self) -> dict:
        t = WfTuning()
        _check(load_library().wf_get_tuning(self._h, C.byref(t)), "wf_get_tuning", self)
        return {"trace_variant": t.trace_variant, "persistent_blocks_per_sm": t.persistent_blocks_per_sm,
                "graph_mode": t.graph_mode, "bvh_builder": t.bvh_builder, "sort_min_queue": t.sort_min_queue,
                "ray_sort_bits": t.ray_sort_bits}

    def add_scene(self, desc: WfSceneDesc) -> int:
        sid = C.c_int32()
        _check(load_library().wf_scene_add(self._h, C.byref(desc), C.byref(sid)), "wf_scene_add", self)
        return sid.value

    def remove_scene(self, sid: int) -> None:
        _check(load_library().wf_scene_remove(self._h, sid), "wf_scene_remove", self)

    def render_batch(self, jobs: list, want_images: bool = True):
        n = len(jobs)
        arr = (WfJob * n)(*jobs)
        imgs = [np.zeros(j.width * j.height * 3, np.float32) for j in jobs] if want_images else []
        ptrs = (f32p * n)(*[ptr(a) for a in imgs]) if want_images else None
        st = WfRenderStats()
        _check(load_library().wf_render_batch(self._h, arr, n, ptrs, C.byref(st)), "wf_render_batch", self)
        out = [a.reshape(j.height, j.width, 3) for a, j in zip(imgs, jobs)]
        return out, st.as_dict()

    def timer_begin(self) -> None:
        _check(load_library().wf_timer_begin(self._h), "wf_timer_begin", self)

    def timer_end(self) -> float:
        ms = C.c_double()
        _check(load_library().wf_timer_end(self._h, C.byref(ms)), "wf_timer_end", self)
        return ms.value

    def stream(self) -> int:
        s = C.c_void_p()
        _check(load_library().wf_get_stream(self._h, C.byref(s)), "wf_get_stream", self)
        return s.value or 0

    # ---- per-bounce stages on device-resident queues ----
    def stage_begin(self, params: WfRenderParams) -> None:
        self._stage = params
        _check(load_library().wf_stage_begin(self._h, C.byref(params)), "wf_stage_begin", self)

    def stage_generate_primary(self, first_sample: int, nspp: int, out: RayQueue) -> None:
        _check(load_library().wf_generate_primary(self._h, first_sample, nspp, out._h), "wf_generate_primary", self)

    def intersect(self, rays: RayQueue, hits: ShadingQueue, misses: RayQueue | None = None) -> None:
        _check(load_library().wf_intersect(self._h, rays._h, hits._h, misses._h if misses else None),
               "wf_intersect", self)

    def shade(self, hits: ShadingQueue, next_rays: RayQueue, shadows: ShadowQueue) -> None:
        _check(load_library().wf_shade(self._h, hits._h, next_rays._h, shadows._h), "wf_shade", self)

    def occluded(self, shadows: ShadowQueue) -> None:
        _check(load_library().wf_trace_occluded(self._h, shadows._h), "wf_trace_occluded", self)

    def miss(self, misses: RayQueue) -> None:
        _check(load_library().wf_miss(self._h, misses._h), "wf_miss", self)

    def stage_image(self) -> np.ndarray:
        p = self._stage
        img = np.zeros(p.width * p.height * 3, np.float32)
        _check(load_library().wf_stage_image(self._h, ptr(img), img.size), "wf_stage_image", self)
        return img.reshape(p.height, p.width, 3)

    def render(self, params: WfRenderParams, accumulate: bool = False, out: np.ndarray | None = None):
        """wf_render (or wf_render_accumulate) into `out` when given — a
        contiguous float32 array of width*height*3 values, e.g. a host_array
        in page-locked memory — else into a new array."""
        nf = params.width * params.height * 3
        if out is None:
            img = np.zeros(nf, dtype=np.float32)
        else:
            if out.dtype != np.float32 or out.size != nf or not out.flags.c_contiguous:
                raise ValueError("out must be a contiguous float32 array of width*height*3 values")
            img = out.reshape(-1)
        st = WfRenderStats()
        fn = load_library().wf_render_accumulate if accumulate else load_library().wf_render
        _check(fn(self._h, C.byref(params), ptr(img), C.byref(st)), "wf_render", self)
        return img.reshape(params.height, params.width, 3), st.as_dict()
