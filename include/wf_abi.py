"""Python mirror of the C ABI's types (include/wf_api.h): constants, structs,
and helpers that only build structs.  Pure ctypes + numpy: importing it loads
no library.  The binding of libwfgpu.so (wavefront-renderer_gb300/__init__.py)
and the CPU oracle's binding (oracle/oracle.py) both use it, so a scene
description or a render-parameter block built for one is valid for the other.

Every struct here must match its C declaration field for field; the CPU
tests check the sizes against the header.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

WF_OK = 0
ERRORS = {
    -1: "WF_ERR_INVALID_ARGUMENT",
    -2: "WF_ERR_CUDA",
    -3: "WF_ERR_OUT_OF_MEMORY",
    -4: "WF_ERR_STATE",
    -5: "WF_ERR_DEVICE_CHECK",
    -6: "WF_ERR_NO_DEVICE",
    -7: "WF_ERR_CAPACITY",
}

MATERIAL_DIFFUSE, MATERIAL_METAL, MATERIAL_EMISSIVE, MATERIAL_SPOTLIGHT, MATERIAL_GLASS, MATERIAL_PLASTIC = range(6)
POLICY_NONE, POLICY_MATERIAL, POLICY_TEXTURE, POLICY_COST_BENEFIT = range(4)
POLICIES = {"none": 0, "material": 1, "texture": 2, "costBenefit": 3}
TEXEL_RGB32F, TEXEL_RGBA8_SRGB = 0, 1

STATIC_SCHEDULE_MAX_RAYS = 1 << 20  # WF_STATIC_SCHEDULE_MAX_RAYS
f32p = C.POINTER(C.c_float)
i32p = C.POINTER(C.c_int32)
u8p = C.POINTER(C.c_uint8)
f64p = C.POINTER(C.c_double)
i64p = C.POINTER(C.c_int64)
u64p = C.POINTER(C.c_uint64)


class WfMaterial(C.Structure):
    _fields_ = [("type", C.c_int32), ("albedo", C.c_float * 3), ("roughness", C.c_float),
                ("emission", C.c_float), ("texture_id", C.c_int32), ("ior", C.c_float),
                ("spot_outer_deg", C.c_float), ("spot_falloff_deg", C.c_float),
                ("use_spatial_checker", C.c_int32), ("checker_cell_size", C.c_float)]


class WfTexture(C.Structure):
    _fields_ = [("width", C.c_int32), ("height", C.c_int32), ("format", C.c_int32), ("data", C.c_void_p)]


class WfEnvironment(C.Structure):
    _fields_ = [("width", C.c_int32), ("height", C.c_int32), ("rgb", f32p),
                ("intensity_scale", C.c_float), ("tint", C.c_float * 3)]


class WfDirectional(C.Structure):
    _fields_ = [("direction", C.c_float * 3), ("color", C.c_float * 3), ("intensity", C.c_float)]


class WfSceneDesc(C.Structure):
    _fields_ = [("num_vertices", C.c_int32), ("positions_x", f32p), ("positions_y", f32p),
                ("positions_z", f32p), ("num_indices", C.c_int32), ("indices", i32p),
                ("num_meshes", C.c_int32), ("mesh_index_offsets", i32p), ("mesh_index_counts", i32p),
                ("mesh_material_ids", i32p), ("corner_u", f32p), ("corner_v", f32p),
                ("mesh_has_uv", u8p), ("num_materials", C.c_int32), ("materials", C.POINTER(WfMaterial)),
                ("num_textures", C.c_int32), ("textures", C.POINTER(WfTexture)),
                ("environment", WfEnvironment), ("directional", WfDirectional)]


class WfCamera(C.Structure):
    _fields_ = [("origin", C.c_float * 3), ("top_left", C.c_float * 3), ("horizontal", C.c_float * 3),
                ("vertical", C.c_float * 3)]

    def as_array(self) -> np.ndarray:
        return np.array([*self.origin, *self.top_left, *self.horizontal, *self.vertical], dtype=np.float32)


class WfRenderParams(C.Structure):
    _fields_ = [("width", C.c_int32), ("height", C.c_int32), ("samples_per_pixel", C.c_int32),
                ("max_depth", C.c_int32), ("rr_min_depth", C.c_int32), ("policy", C.c_int32),
                ("enable_ray_sort", C.c_int32), ("enable_cost_aware_rr", C.c_int32),
                ("firefly_threshold", C.c_float), ("seed_lo", C.c_uint32), ("seed_hi", C.c_uint32),
                ("first_sample", C.c_int32), ("spp_per_wave", C.c_int32), ("enable_env_nee", C.c_int32),
                ("enable_adaptive_sampling", C.c_int32), ("adaptive_threshold", C.c_float),
                ("enable_cost_tracking", C.c_int32), ("reserved0", C.c_int32),
                ("rel_cost_material", f64p), ("rel_cost_texture", f64p), ("camera", WfCamera)]


class WfRenderStats(C.Structure):
    _fields_ = [("closest_rays", C.c_uint64), ("shadow_rays", C.c_uint64), ("shaded_hits", C.c_uint64),
                ("misses", C.c_uint64), ("sorted_elements", C.c_uint64), ("ms_total", C.c_double),
                ("ms_ray_sort", C.c_double), ("ms_intersect", C.c_double), ("ms_shade", C.c_double),
                ("ms_schedule", C.c_double), ("waves", C.c_int32), ("bounces", C.c_int32),
                ("kernel_launches", C.c_int64), ("samples_run", C.c_int32), ("active_pixels", C.c_int32)]

    def as_dict(self) -> dict:
        return {name: getattr(self, name) for name, _ in self._fields_}


class WfConfig(C.Structure):
    _fields_ = [("device", C.c_int32), ("max_paths_per_wave", C.c_int64)]


class WfSceneInfo(C.Structure):
    _fields_ = [("bounds_min", C.c_float * 3), ("bounds_max", C.c_float * 3),
                ("total_emissive_area", C.c_float), ("num_triangles", C.c_int32),
                ("num_meshes", C.c_int32), ("num_emissive_meshes", C.c_int32), ("bvh_nodes", C.c_int32),
                ("bvh_build_ms", C.c_double), ("device_bytes", C.c_int64), ("bvh_builder", C.c_int32),
                ("bvh_depth", C.c_int32)]


class WfTuning(C.Structure):
    _fields_ = [("trace_variant", C.c_int32), ("persistent_blocks_per_sm", C.c_int32), ("graph_mode", C.c_int32),
                ("bvh_builder", C.c_int32), ("sort_min_queue", C.c_int32), ("reserved2", C.c_int32),
                ("reserved", C.c_int32), ("ray_sort_bits", C.c_int32)]


class WfJob(C.Structure):
    _fields_ = [("scene_id", C.c_int32), ("width", C.c_int32), ("height", C.c_int32),
                ("samples_per_pixel", C.c_int32), ("max_depth", C.c_int32), ("rr_min_depth", C.c_int32),
                ("enable_cost_aware_rr", C.c_int32), ("firefly_threshold", C.c_float), ("seed_lo", C.c_uint32),
                ("seed_hi", C.c_uint32), ("first_sample", C.c_int32), ("enable_env_nee", C.c_int32),
                ("rel_cost_material", f64p), ("camera", WfCamera)]


class WfServerConfig(C.Structure):
    _fields_ = [("hbm_budget_bytes", C.c_int64), ("max_paths_per_wave", C.c_int64), ("frame_spp", C.c_int32),
                ("reserved", C.c_int32 * 7)]


class WfJobStatus(C.Structure):
    _fields_ = [("state", C.c_int32), ("samples_done", C.c_int32), ("frames", C.c_int32), ("reserved", C.c_int32),
                ("t_submit", C.c_double), ("t_admit", C.c_double), ("t_first_frame", C.c_double),
                ("t_done", C.c_double)]

    def as_dict(self) -> dict:
        return {name: getattr(self, name) for name, _ in self._fields_ if name != "reserved"}


class WfServerStepInfo(C.Structure):
    _fields_ = [("queued", C.c_int32), ("running", C.c_int32), ("completed_this_step", C.c_int32),
                ("jobs_in_wave", C.c_int32), ("paths_in_wave", C.c_int64), ("rays_traced", C.c_uint64),
                ("step_ms", C.c_double), ("budget_used_bytes", C.c_int64)]

    def as_dict(self) -> dict:
        return {name: getattr(self, name) for name, _ in self._fields_}


JOB_QUEUED, JOB_RUNNING, JOB_DONE, JOB_CANCELLED, JOB_REJECTED = range(5)


class WfHitColumns(C.Structure):
    _fields_ = [("geom_id", i32p), ("prim_id", i32p), ("distance", f32p), ("bary_u", f32p),
                ("bary_v", f32p), ("point_x", f32p), ("point_y", f32p), ("point_z", f32p),
                ("normal_x", f32p), ("normal_y", f32p), ("normal_z", f32p), ("front_face", u8p),
                ("u", f32p), ("v", f32p), ("material_id", i32p), ("texture_id", i32p)]


class WfRayColumns(C.Structure):
    _fields_ = [("origins_x", f32p), ("origins_y", f32p), ("origins_z", f32p), ("dirs_x", f32p), ("dirs_y", f32p),
                ("dirs_z", f32p), ("throughputs_r", f32p), ("throughputs_g", f32p), ("throughputs_b", f32p),
                ("pdfs", f32p), ("pixel_indices", i32p), ("depths", i32p), ("sample_indices", i32p)]


RAY_FIELDS = {"origins_x": np.float32, "origins_y": np.float32, "origins_z": np.float32, "dirs_x": np.float32,
              "dirs_y": np.float32, "dirs_z": np.float32, "throughputs_r": np.float32, "throughputs_g": np.float32,
              "throughputs_b": np.float32, "pdfs": np.float32, "pixel_indices": np.int32, "depths": np.int32,
              "sample_indices": np.int32}


def make_ray_columns(n: int, given: dict | None = None):
    """Host columns of n rays (RAY_FIELDS) and the WfRayColumns pointing at
    them; `given` supplies arrays for some columns (others are zero), or,
    with given is not None, only those columns are pointed at."""
    cols = {}
    for k, t in RAY_FIELDS.items():
        if given is None:
            cols[k] = np.zeros(n, dtype=t)
        elif k in given:
            cols[k] = np.ascontiguousarray(given[k], dtype=t)
    ct = {np.int32: C.c_int32, np.float32: C.c_float}
    rc = WfRayColumns(**{k: ptr(v, ct[RAY_FIELDS[k]]) for k, v in cols.items()})
    return cols, rc


HIT_FIELDS = {"geom_id": np.int32, "prim_id": np.int32, "distance": np.float32, "bary_u": np.float32,
              "bary_v": np.float32, "point_x": np.float32, "point_y": np.float32, "point_z": np.float32,
              "normal_x": np.float32, "normal_y": np.float32, "normal_z": np.float32,
              "front_face": np.uint8, "u": np.float32, "v": np.float32, "material_id": np.int32,
              "texture_id": np.int32}


def ptr(a: np.ndarray | None, ctype=C.c_float):
    if a is None:
        return None
    assert a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(C.POINTER(ctype))


def make_hit_columns(n: int):
    cols = {k: np.zeros(n, dtype=t) for k, t in HIT_FIELDS.items()}
    ct = {np.int32: C.c_int32, np.float32: C.c_float, np.uint8: C.c_uint8}
    hc = WfHitColumns(**{k: ptr(v, ct[HIT_FIELDS[k]]) for k, v in cols.items()})
    return cols, hc


def make_job(scene_id, width, height, spp, max_depth, camera: WfCamera, *, seed=1, rr_min_depth=3, firefly=10.0,
             first_sample=0, env_nee=False) -> WfJob:
    j = WfJob()
    j.scene_id, j.width, j.height, j.samples_per_pixel, j.max_depth = scene_id, width, height, spp, max_depth
    j.rr_min_depth, j.firefly_threshold, j.first_sample = rr_min_depth, firefly, first_sample
    j.seed_lo, j.seed_hi = seed & 0xFFFFFFFF, (seed >> 32) & 0xFFFFFFFF
    j.enable_env_nee = int(bool(env_nee))
    j.camera = camera
    return j


def render_params(width, height, spp, max_depth, camera: WfCamera, *, policy=0, ray_sort=False,
                  rr_min_depth=3, firefly=10.0, seed=1, first_sample=0, spp_per_wave=0,
                  cost_aware_rr=False, rel_cost_material=None, rel_cost_texture=None,
                  env_nee=False, adaptive=False, adaptive_threshold=0.05, cost_tracking=False) -> WfRenderParams:
    p = WfRenderParams()
    p.width, p.height, p.samples_per_pixel, p.max_depth = width, height, spp, max_depth
    p.rr_min_depth, p.policy, p.enable_ray_sort = rr_min_depth, policy, int(bool(ray_sort))
    p.enable_cost_aware_rr = int(bool(cost_aware_rr))
    p.firefly_threshold = firefly
    p.seed_lo, p.seed_hi = seed & 0xFFFFFFFF, (seed >> 32) & 0xFFFFFFFF
    p.first_sample, p.spp_per_wave = first_sample, spp_per_wave
    p.enable_env_nee = int(bool(env_nee))
    p.enable_adaptive_sampling = int(bool(adaptive))
    p.adaptive_threshold = adaptive_threshold
    p.enable_cost_tracking = int(bool(cost_tracking))
    p._keep = []
    if rel_cost_material is not None:
        a = np.ascontiguousarray(rel_cost_material, dtype=np.float64)
        p._keep.append(a)
        p.rel_cost_material = ptr(a, C.c_double)
    if rel_cost_texture is not None:
        a = np.ascontiguousarray(rel_cost_texture, dtype=np.float64)
        p._keep.append(a)
        p.rel_cost_texture = ptr(a, C.c_double)
    p.camera = camera
    return p
