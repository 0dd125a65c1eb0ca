"""The C ABI library (no GPU needed): it loads, exports every entry point the
header declares, and its host-only parts (procedural scenes, camera) work."""
from __future__ import annotations

import ctypes as C
import subprocess

import numpy as np
import pytest


def test_library_exports_every_header_symbol(wf):
    lib = wf.load_library()
    declared = wf.header_symbols()
    assert len(declared) >= 20
    missing = [s for s in declared if not hasattr(lib, s)]
    assert not missing, missing
    out = subprocess.run(["nm", "-D", "--defined-only", str(wf.LIB_PATH)], capture_output=True, text=True).stdout
    exported = {ln.split()[-1] for ln in out.splitlines() if " T " in ln}
    assert set(declared) <= exported
    assert lib.wf_version() == 1


def test_build_targets_sm_103a_only():
    """build.py compiles one -gencode, sm_103a, with no fused multiply-add."""
    import importlib.util
    from conftest import ROOT
    spec = importlib.util.spec_from_file_location("wf_build_flags", ROOT / "wavefront-renderer_gb300" / "build.py")
    b = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(b)
    assert b.ARCH == ["-gencode", "arch=compute_103a,code=sm_103a"]
    assert "-fmad=false" in b.NVCC_FLAGS and "--use_fast_math" not in b.NVCC_FLAGS


def test_host_scene_config0(wf):
    s = wf.HostScene(0)
    a = s.arrays()
    assert s.desc.num_indices == 36 * 3 and s.desc.num_meshes == 18
    assert len(a["materials"]) == 6
    # the light quad's geometric normal points down (one-sided NEE)
    light = [m for m in range(18) if a["mesh_materials"][m] == 3][0]
    i = a["indices"][a["mesh_offsets"][light]:a["mesh_offsets"][light] + 3]
    v = np.stack([a["px"][i], a["py"][i], a["pz"][i]], 1)
    assert np.cross(v[1] - v[0], v[2] - v[0])[1] < 0


def test_host_scene_config1_is_deterministic(wf):
    a = wf.HostScene(100, seed=3).arrays()
    b = wf.HostScene(100, seed=3).arrays()
    c = wf.HostScene(100, seed=4).arrays()
    assert np.array_equal(a["px"], b["px"]) and np.array_equal(a["indices"], b["indices"])
    assert not np.array_equal(a["px"], c["px"])
    assert len(a["indices"]) // 3 == 12 + 20 * 4 ** 4


def test_camera_make_matches_reference_constructor(wf, orc):
    cam = wf.camera_make([0, 0.275, 0.8], [0, 0.275, 0], [0, 1, 0], 40.0, 256, 256)
    if orc.ref_available():
        assert np.array_equal(cam.as_array(), orc.ref_camera([0, 0.275, 0.8], [0, 0.275, 0], [0, 1, 0], 40.0, 256, 256))
    assert abs(np.linalg.norm(cam.as_array()[6:9]) / np.linalg.norm(cam.as_array()[9:12]) - 1.0) < 1e-6


def test_invalid_arguments_are_rejected_without_a_device(wf):
    lib = wf.load_library()
    assert lib.wf_camera_make(None, None, None, 40.0, 8, 8, None) == -1
    assert lib.wf_host_scene_generate(99, 1, C.byref(C.c_void_p())) == -1
    assert lib.wf_create(None, None) == -1


# ------------------------------------------------ scene files, PFM ---------

def test_scene_file_round_trip(wf, orc, tmp_path):
    """A textured scene with UVs and an HDRI survives wf_scene_save /
    wf_scene_load array for array, and the port renders both the same."""
    hs = wf.HostScene(102)
    path = tmp_path / "lattice.wfscene"
    hs.save(path, [8, 4.5, 18], [8, 0, 6], [0, 1, 0], 50.0)
    back = wf.HostScene.load(path)
    a, b = hs.arrays(), back.arrays()
    for k in ("px", "py", "pz", "indices", "mesh_offsets", "mesh_counts", "mesh_materials"):
        assert np.array_equal(a[k], b[k]), k
    d0, d1 = hs.desc, back.desc
    assert d0.num_materials == d1.num_materials and d0.num_textures == d1.num_textures == 64
    assert all(bytes(d0.materials[i]) == bytes(d1.materials[i]) for i in range(d0.num_materials))
    n = d0.num_indices
    for k in ("corner_u", "corner_v"):
        assert np.array_equal(np.ctypeslib.as_array(getattr(d0, k), (n,)), np.ctypeslib.as_array(getattr(d1, k), (n,)))
    t0, t1 = d0.textures[5], d1.textures[5]
    assert (t0.width, t0.height, t0.format) == (t1.width, t1.height, t1.format)
    assert C.string_at(t0.data, t0.width * t0.height * 4) == C.string_at(t1.data, t1.width * t1.height * 4)
    assert np.array_equal(orc.scene_environment(d0), orc.scene_environment(d1))
    cam = back.camera(24, 16)
    assert np.allclose(cam.as_array(), wf.camera_make([8, 4.5, 18], [8, 0, 6], [0, 1, 0], 50.0, 24, 16).as_array())
    p = wf.render_params(24, 16, 2, 4, cam, seed=3)
    r0, _ = orc.Port(d0).render_window(p, 0, 0, 24, 16)
    r1, _ = orc.Port(d1).render_window(p, 0, 0, 24, 16)
    assert np.array_equal(r0, r1)


def test_scene_file_rejects_damage(wf, tmp_path):
    hs = wf.HostScene(0)
    path = tmp_path / "box.wfscene"
    hs.save(path, [0, 0.275, 0.8], [0, 0.275, 0], [0, 1, 0], 40.0)
    raw = path.read_bytes()
    for bad in (raw[:-3], raw + b"x", b"WFSCENE2" + raw[8:], raw[:40]):
        path.write_bytes(bad)
        with pytest.raises(RuntimeError):
            wf.HostScene.load(path)
    with pytest.raises(RuntimeError):
        wf.HostScene.load(tmp_path / "missing.wfscene")


def test_pfm_writer(wf, orc, tmp_path):
    img = np.random.default_rng(1).random((5, 7, 3)).astype(np.float32)
    path = tmp_path / "img.pfm"
    wf.write_pfm(path, img)
    raw = path.read_bytes()
    header = b"PF\n7 5\n-1.0\n"
    assert raw.startswith(header)
    rows = np.frombuffer(raw[len(header):], "<f4").reshape(5, 7, 3)
    assert np.array_equal(rows[::-1], img)
    orc.write_pfm(tmp_path / "ref.pfm", img)  # the checker's writer: same bytes
    assert (tmp_path / "ref.pfm").read_bytes() == raw
