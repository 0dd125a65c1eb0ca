// wf_scene_io.cpp — scene files and float images (host only).
//
// The reference reads scenes through OpenUSD (src/scene/UsdSceneLoader.cpp)
// and writes images through OpenImageIO (src/core/Image.cpp); neither
// library is part of this build.  What the render path consumes is the flat
// scene of Scene/SceneGeometry (include/core/Scene.h:14-107) — vertex and
// index arrays, per-mesh ranges and material ids, materials, textures, an
// environment map and a directional light — so the scene file stores exactly
// that, and wf_scene_load hands back the same wf_host_scene the procedural
// generators produce.
//
// File layout (little-endian, no padding):
//   "WFSCENE1"                       8 bytes
//   u32 version (1), u32 0x01020304  byte-order check
//   i32 num_vertices, num_indices, num_meshes, num_materials, num_textures,
//       has_uv (0/1)
//   f32 look_from[3], look_at[3], up[3], vfov
//   f32 px[nv], py[nv], pz[nv]; i32 indices[ni]
//   i32 mesh_offsets[nm], mesh_counts[nm], mesh_materials[nm]
//   has_uv: f32 corner_u[ni], corner_v[ni]; u8 mesh_has_uv[nm]
//   materials: 12 four-byte fields each, in wf_material order
//   textures: i32 width, height, format, then width*height texels
//             (RGB32F: 12 bytes, RGBA8_SRGB: 4 bytes)
//   environment: i32 width, height; f32 intensity, tint[3]; f32 rgb[w*h*3]
//   directional: f32 direction[3], color[3], intensity
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/wf_api.h"
#include "wf_host_scene.h"

namespace {

constexpr char kMagic[8] = {'W', 'F', 'S', 'C', 'E', 'N', 'E', '1'};
constexpr uint32_t kVersion = 1;
constexpr uint32_t kOrder = 0x01020304u;

struct Writer {
    FILE* f;
    bool ok = true;
    void bytes(const void* p, size_t n)
    {
        if (ok && n > 0 && std::fwrite(p, 1, n, f) != n) ok = false;
    }
    template <class T>
    void value(T v)
    {
        bytes(&v, sizeof(T));
    }
    template <class T>
    void array(const T* p, size_t n)
    {
        if (n > 0 && !p) {
            ok = false;
            return;
        }
        bytes(p, sizeof(T) * n);
    }
};

struct Reader {
    FILE* f;
    int64_t left;  // bytes not yet read
    bool ok = true;
    void bytes(void* p, size_t n)
    {
        if (!ok) return;
        if ((int64_t)n > left || (n > 0 && std::fread(p, 1, n, f) != n)) {
            ok = false;
            return;
        }
        left -= (int64_t)n;
    }
    template <class T>
    T value()
    {
        T v{};
        bytes(&v, sizeof(T));
        return v;
    }
    // n elements of T, refused when the file cannot hold them
    template <class T>
    bool array(std::vector<T>& out, int64_t n)
    {
        if (!ok || n < 0 || n * (int64_t)sizeof(T) > left) {
            ok = false;
            return false;
        }
        out.resize((size_t)n);
        bytes(out.data(), sizeof(T) * (size_t)n);
        return ok;
    }
};

int64_t texel_bytes(int32_t format) { return format == WF_TEXEL_RGB32F ? 12 : 4; }

}  // namespace

extern "C" {

int wf_scene_save(const char* path, const wf_scene_desc* d, const float look_from[3], const float look_at[3],
                  const float up[3], float vfov)
{
    if (!path || !d || !look_from || !look_at || !up) return WF_ERR_INVALID_ARGUMENT;
    if (d->num_vertices < 0 || d->num_indices < 0 || d->num_meshes < 0 || d->num_materials < 0 ||
        d->num_textures < 0 || (d->num_textures > 0 && !d->textures))
        return WF_ERR_INVALID_ARGUMENT;
    FILE* f = std::fopen(path, "wb");
    if (!f) return WF_ERR_INVALID_ARGUMENT;
    Writer w{f};
    const int32_t has_uv = (d->corner_u && d->corner_v && d->mesh_has_uv) ? 1 : 0;
    w.bytes(kMagic, sizeof(kMagic));
    w.value(kVersion);
    w.value(kOrder);
    w.value(d->num_vertices);
    w.value(d->num_indices);
    w.value(d->num_meshes);
    w.value(d->num_materials);
    w.value(d->num_textures);
    w.value(has_uv);
    w.array(look_from, 3);
    w.array(look_at, 3);
    w.array(up, 3);
    w.value(vfov);
    w.array(d->positions_x, (size_t)d->num_vertices);
    w.array(d->positions_y, (size_t)d->num_vertices);
    w.array(d->positions_z, (size_t)d->num_vertices);
    w.array(d->indices, (size_t)d->num_indices);
    w.array(d->mesh_index_offsets, (size_t)d->num_meshes);
    w.array(d->mesh_index_counts, (size_t)d->num_meshes);
    w.array(d->mesh_material_ids, (size_t)d->num_meshes);
    if (has_uv) {
        w.array(d->corner_u, (size_t)d->num_indices);
        w.array(d->corner_v, (size_t)d->num_indices);
        w.array(d->mesh_has_uv, (size_t)d->num_meshes);
    }
    for (int32_t m = 0; m < d->num_materials; ++m) {
        const wf_material& x = d->materials[m];
        w.value(x.type);
        w.array(x.albedo, 3);
        w.value(x.roughness);
        w.value(x.emission);
        w.value(x.texture_id);
        w.value(x.ior);
        w.value(x.spot_outer_deg);
        w.value(x.spot_falloff_deg);
        w.value(x.use_spatial_checker);
        w.value(x.checker_cell_size);
    }
    for (int32_t t = 0; t < d->num_textures; ++t) {
        const wf_texture& x = d->textures[t];
        if (x.width < 0 || x.height < 0 || (x.format != WF_TEXEL_RGB32F && x.format != WF_TEXEL_RGBA8_SRGB)) {
            w.ok = false;
            break;
        }
        w.value(x.width);
        w.value(x.height);
        w.value(x.format);
        w.array((const uint8_t*)x.data, (size_t)((int64_t)x.width * x.height * texel_bytes(x.format)));
    }
    const wf_environment& e = d->environment;
    const int32_t ew = (e.width > 0 && e.rgb) ? e.width : 0, eh = ew > 0 ? e.height : 0;
    w.value(ew);
    w.value(eh);
    w.value(e.intensity_scale);
    w.array(e.tint, 3);
    w.array(e.rgb, (size_t)ew * (size_t)eh * 3);
    w.array(d->directional.direction, 3);
    w.array(d->directional.color, 3);
    w.value(d->directional.intensity);
    const bool ok = w.ok && std::fclose(f) == 0;
    if (!w.ok) std::fclose(f);
    return ok ? WF_OK : WF_ERR_INVALID_ARGUMENT;
}

int wf_scene_load(const char* path, wf_host_scene** out)
{
    if (!path || !out) return WF_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    FILE* f = std::fopen(path, "rb");
    if (!f) return WF_ERR_INVALID_ARGUMENT;
    std::fseek(f, 0, SEEK_END);
    const long size = std::ftell(f);
    std::fseek(f, 0, SEEK_SET);
    Reader r{f, (int64_t)(size > 0 ? size : 0)};
    auto* s = new wf_host_scene();
    s->config = -1;
    char magic[8];
    r.bytes(magic, sizeof(magic));
    const uint32_t version = r.value<uint32_t>(), order = r.value<uint32_t>();
    if (!r.ok || std::memcmp(magic, kMagic, sizeof(kMagic)) != 0 || version != kVersion || order != kOrder)
        r.ok = false;
    const int32_t nv = r.value<int32_t>(), ni = r.value<int32_t>(), nm = r.value<int32_t>();
    const int32_t nmat = r.value<int32_t>(), ntex = r.value<int32_t>(), has_uv = r.value<int32_t>();
    for (int k = 0; k < 3; ++k) s->look_from[k] = r.value<float>();
    for (int k = 0; k < 3; ++k) s->look_at[k] = r.value<float>();
    for (int k = 0; k < 3; ++k) s->up[k] = r.value<float>();
    s->vfov = r.value<float>();
    if (nv < 0 || ni < 0 || nm < 0 || nmat < 0 || ntex < 0 || (has_uv != 0 && has_uv != 1)) r.ok = false;
    r.array(s->px, nv);
    r.array(s->py, nv);
    r.array(s->pz, nv);
    r.array(s->idx, ni);
    r.array(s->mesh_off, nm);
    r.array(s->mesh_cnt, nm);
    r.array(s->mesh_mat, nm);
    if (has_uv) {
        r.array(s->cu, ni);
        r.array(s->cv, ni);
        r.array(s->has_uv, nm);
    }
    if (r.ok && (int64_t)nmat * 48 <= r.left) {
        s->mats.resize((size_t)nmat);
        for (int32_t m = 0; m < nmat && r.ok; ++m) {
            wf_material& x = s->mats[m];
            x.type = r.value<int32_t>();
            for (int k = 0; k < 3; ++k) x.albedo[k] = r.value<float>();
            x.roughness = r.value<float>();
            x.emission = r.value<float>();
            x.texture_id = r.value<int32_t>();
            x.ior = r.value<float>();
            x.spot_outer_deg = r.value<float>();
            x.spot_falloff_deg = r.value<float>();
            x.use_spatial_checker = r.value<int32_t>();
            x.checker_cell_size = r.value<float>();
        }
    } else {
        r.ok = false;
    }
    for (int32_t t = 0; t < ntex && r.ok; ++t) {
        wf_texture x{};
        x.width = r.value<int32_t>();
        x.height = r.value<int32_t>();
        x.format = r.value<int32_t>();
        if (x.width < 0 || x.height < 0 || (x.format != WF_TEXEL_RGB32F && x.format != WF_TEXEL_RGBA8_SRGB)) {
            r.ok = false;
            break;
        }
        std::vector<uint8_t> raw;
        r.array(raw, (int64_t)x.width * x.height * texel_bytes(x.format));
        s->tex_data.push_back(std::move(raw));
        s->textures.push_back(x);
    }
    s->env_w = r.value<int32_t>();
    s->env_h = r.value<int32_t>();
    s->env_scale = r.value<float>();
    for (int k = 0; k < 3; ++k) s->env_tint[k] = r.value<float>();
    if (s->env_w < 0 || s->env_h < 0) r.ok = false;
    r.array(s->env, (int64_t)s->env_w * s->env_h * 3);
    for (int k = 0; k < 3; ++k) s->dir.direction[k] = r.value<float>();
    for (int k = 0; k < 3; ++k) s->dir.color[k] = r.value<float>();
    s->dir.intensity = r.value<float>();
    std::fclose(f);
    if (!r.ok || r.left != 0) {
        delete s;
        return WF_ERR_INVALID_ARGUMENT;
    }
    *out = s;
    return WF_OK;
}

int wf_image_write_pfm(const char* path, const float* rgb, int32_t width, int32_t height)
{
    if (!path || !rgb || width <= 0 || height <= 0) return WF_ERR_INVALID_ARGUMENT;
    FILE* f = std::fopen(path, "wb");
    if (!f) return WF_ERR_INVALID_ARGUMENT;
    // Portable float map, little-endian (negative scale); rows bottom to top.
    const std::string header = "PF\n" + std::to_string(width) + " " + std::to_string(height) + "\n-1.0\n";
    bool ok = std::fwrite(header.data(), 1, header.size(), f) == header.size();
    for (int32_t y = height - 1; y >= 0 && ok; --y)
        ok = std::fwrite(rgb + (size_t)y * width * 3, sizeof(float), (size_t)width * 3, f) == (size_t)width * 3;
    ok = (std::fclose(f) == 0) && ok;
    return ok ? WF_OK : WF_ERR_INVALID_ARGUMENT;
}

}  // extern "C"
