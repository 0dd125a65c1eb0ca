// wf_scenes.cpp — procedural workloads standing in for the reference's stress
// scenes (which are not in its checkout).  Host code; only IEEE basic
// arithmetic (no libm transcendental in the geometry), so the same seed gives
// the same vertices on x86 and Arm when built with -ffp-contract=off.
//
// Meshes follow the reference's own convention for quads
// (src/scene/CornellBox.cpp:28-45: vertices bl, br, tr, tl; triangles
// (0,1,2), (0,2,3)) and make every quad its own mesh, as CornellBox::build and
// addRotatedBox do.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <unordered_map>
#include <vector>

#include "../../include/wf_api.h"

struct wf_host_scene {
    int32_t config = 0;
    std::vector<float> px, py, pz;
    std::vector<int32_t> idx;
    std::vector<int32_t> mesh_off, mesh_cnt, mesh_mat;
    std::vector<wf_material> mats;
    float look_from[3], look_at[3], up[3];
    float vfov = 40.0f;
};

namespace {

struct P3 {
    float x, y, z;
};

wf_material make_material(int type, float r, float g, float b)
{
    wf_material m;
    std::memset(&m, 0, sizeof(m));
    m.type = type;
    m.albedo[0] = r;
    m.albedo[1] = g;
    m.albedo[2] = b;
    m.roughness = 0.0f;
    m.emission = 0.0f;
    m.texture_id = -1;
    m.ior = 1.5f;
    m.spot_outer_deg = 0.0f;
    m.spot_falloff_deg = 0.0f;
    m.use_spatial_checker = 0;
    m.checker_cell_size = 1.0f;
    return m;
}

// Material::makeDiffuse / makeMetal / makeEmissive / makeGlass
// (src/shading/Material.cpp:67-129) field values.
wf_material diffuse(float r, float g, float b)
{
    wf_material m = make_material(WF_MATERIAL_DIFFUSE, r, g, b);
    m.roughness = 1.0f;
    return m;
}
wf_material metal(float r, float g, float b, float rough)
{
    wf_material m = make_material(WF_MATERIAL_METAL, r, g, b);
    m.roughness = rough;
    return m;
}
wf_material emissive(float r, float g, float b, float strength)
{
    wf_material m = make_material(WF_MATERIAL_EMISSIVE, r, g, b);
    m.emission = strength;
    return m;
}
wf_material glass(float ior)
{
    wf_material m = make_material(WF_MATERIAL_GLASS, 1.0f, 1.0f, 1.0f);
    m.ior = ior;
    return m;
}

void begin_mesh(wf_host_scene& s, int material)
{
    s.mesh_off.push_back((int32_t)s.idx.size());
    s.mesh_cnt.push_back(0);
    s.mesh_mat.push_back(material);
}
void end_mesh(wf_host_scene& s) { s.mesh_cnt.back() = (int32_t)s.idx.size() - s.mesh_off.back(); }

int add_vertex(wf_host_scene& s, P3 p)
{
    s.px.push_back(p.x);
    s.py.push_back(p.y);
    s.pz.push_back(p.z);
    return (int)s.px.size() - 1;
}

// One quad = one mesh of two triangles.
void add_quad(wf_host_scene& s, int material, P3 bl, P3 br, P3 tr, P3 tl)
{
    begin_mesh(s, material);
    int a = add_vertex(s, bl), b = add_vertex(s, br), c = add_vertex(s, tr), d = add_vertex(s, tl);
    int tri[6] = {a, b, c, a, c, d};
    s.idx.insert(s.idx.end(), tri, tri + 6);
    end_mesh(s);
}

// Box of 6 quads rotated about the vertical axis through its base centre.
// cos/sin of the angle are given as exact constants by the caller.
void add_box(wf_host_scene& s, int material, P3 lo, P3 hi, float cosa, float sina)
{
    const float cx = 0.5f * (lo.x + hi.x), cz = 0.5f * (lo.z + hi.z);
    auto rot = [&](float x, float y, float z) {
        float lx = x - cx, lz = z - cz;
        return P3{cosa * lx - sina * lz + cx, y, sina * lx + cosa * lz + cz};
    };
    P3 c[8] = {rot(lo.x, lo.y, lo.z), rot(hi.x, lo.y, lo.z), rot(hi.x, lo.y, hi.z), rot(lo.x, lo.y, hi.z),
               rot(lo.x, hi.y, lo.z), rot(hi.x, hi.y, lo.z), rot(hi.x, hi.y, hi.z), rot(lo.x, hi.y, hi.z)};
    add_quad(s, material, c[0], c[1], c[2], c[3]);  // bottom
    add_quad(s, material, c[7], c[6], c[5], c[4]);  // top
    add_quad(s, material, c[3], c[2], c[6], c[7]);  // front
    add_quad(s, material, c[1], c[0], c[4], c[5]);  // back
    add_quad(s, material, c[0], c[3], c[7], c[4]);  // left
    add_quad(s, material, c[2], c[1], c[5], c[6]);  // right
}

// The 0.55 m room: floor, ceiling, back wall (white), left (red), right
// (green), open towards the camera at z = 0, and the ceiling light whose
// geometric normal points down (the reference's NEE is one-sided,
// WavefrontRenderer.cpp:673-676).  Materials 0..3.
void add_room(wf_host_scene& s)
{
    s.mats.push_back(diffuse(0.73f, 0.73f, 0.73f));   // 0 white
    s.mats.push_back(diffuse(0.65f, 0.05f, 0.05f));   // 1 red
    s.mats.push_back(diffuse(0.12f, 0.45f, 0.15f));   // 2 green
    s.mats.push_back(emissive(17.0f, 12.0f, 4.0f, 1.0f));  // 3 light
    const float X = 0.275f, Y = 0.55f, Z = -0.55f;
    add_quad(s, 0, {-X, 0, 0}, {X, 0, 0}, {X, 0, Z}, {-X, 0, Z});    // floor
    add_quad(s, 0, {-X, Y, Z}, {X, Y, Z}, {X, Y, 0}, {-X, Y, 0});    // ceiling
    add_quad(s, 0, {-X, 0, Z}, {X, 0, Z}, {X, Y, Z}, {-X, Y, Z});    // back
    add_quad(s, 1, {-X, 0, 0}, {-X, 0, Z}, {-X, Y, Z}, {-X, Y, 0});  // left, red
    add_quad(s, 2, {X, 0, Z}, {X, 0, 0}, {X, Y, 0}, {X, Y, Z});      // right, green
    const float ly = Y - 0.001f;
    add_quad(s, 3, {-0.065f, ly, -0.33f}, {0.065f, ly, -0.33f}, {0.065f, ly, -0.22f},
             {-0.065f, ly, -0.22f});  // light, normal -y
}

void set_camera(wf_host_scene& s)
{
    const float f[3] = {0.0f, 0.275f, 0.8f}, a[3] = {0.0f, 0.275f, 0.0f}, u[3] = {0.0f, 1.0f, 0.0f};
    std::memcpy(s.look_from, f, sizeof(f));
    std::memcpy(s.look_at, a, sizeof(a));
    std::memcpy(s.up, u, sizeof(u));
    s.vfov = 40.0f;
}

// Config 0: room + a metal box (roughness 0.3, the reference's fuzzy metal)
// rotated 15 degrees and a white Lambert box rotated -18 degrees.  18 meshes,
// 36 triangles.  cos/sin(15 deg) and cos/sin(-18 deg) as float constants.
void build_config0(wf_host_scene& s)
{
    add_room(s);
    s.mats.push_back(metal(0.8f, 0.8f, 0.8f, 0.3f));  // 4 tall box, metal
    s.mats.push_back(diffuse(0.73f, 0.73f, 0.73f));   // 5 short box, white
    add_box(s, 4, {-0.19f, 0.0f, -0.42f}, {-0.025f, 0.33f, -0.255f}, 0.96592583f, 0.25881905f);
    add_box(s, 5, {0.0325f, 0.0f, -0.2225f}, {0.1975f, 0.165f, -0.0575f}, 0.95105652f, -0.30901699f);
    set_camera(s);
}

// --- seeded value noise / FBM (only +, -, *, floor) -----------------------
uint32_t hash3(int x, int y, int z, uint32_t seed)
{
    uint32_t h = seed ^ 0x9E3779B9u;
    h ^= (uint32_t)x * 0x8DA6B343u;
    h ^= (uint32_t)y * 0xD8163841u;
    h ^= (uint32_t)z * 0xCB1AB31Fu;
    h ^= h >> 16;
    h *= 0x7FEB352Du;
    h ^= h >> 15;
    h *= 0x846CA68Bu;
    h ^= h >> 16;
    return h;
}
float lattice(int x, int y, int z, uint32_t seed)
{
    return (float)(hash3(x, y, z, seed) >> 8) * (2.0f / 16777216.0f) - 1.0f;
}
float value_noise(float x, float y, float z, uint32_t seed)
{
    float fx = std::floor(x), fy = std::floor(y), fz = std::floor(z);
    int ix = (int)fx, iy = (int)fy, iz = (int)fz;
    float tx = x - fx, ty = y - fy, tz = z - fz;
    float wx = tx * tx * (3.0f - 2.0f * tx), wy = ty * ty * (3.0f - 2.0f * ty), wz = tz * tz * (3.0f - 2.0f * tz);
    float c[2][2][2];
    for (int a = 0; a < 2; ++a)
        for (int b = 0; b < 2; ++b)
            for (int d = 0; d < 2; ++d) c[a][b][d] = lattice(ix + a, iy + b, iz + d, seed);
    float x00 = c[0][0][0] + (c[1][0][0] - c[0][0][0]) * wx;
    float x10 = c[0][1][0] + (c[1][1][0] - c[0][1][0]) * wx;
    float x01 = c[0][0][1] + (c[1][0][1] - c[0][0][1]) * wx;
    float x11 = c[0][1][1] + (c[1][1][1] - c[0][1][1]) * wx;
    float y0 = x00 + (x10 - x00) * wy;
    float y1 = x01 + (x11 - x01) * wy;
    return y0 + (y1 - y0) * wz;
}
float fbm(float x, float y, float z, uint32_t seed)
{
    float sum = 0.0f, amp = 1.0f, norm = 0.0f, f = 1.0f;
    for (int o = 0; o < 5; ++o) {
        sum += amp * value_noise(x * f, y * f, z * f, seed + (uint32_t)o * 1013u);
        norm += amp;
        amp *= 0.5f;
        f *= 2.0f;
    }
    return sum / norm;
}

uint64_t splitmix64(uint64_t& s)
{
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
float uniform01(uint64_t& s) { return (float)(splitmix64(s) >> 40) * (1.0f / 16777216.0f); }

// Config 1: the config-0 room plus a displaced icosphere (20 * 4^8 =
// 1,310,720 triangles), radius 0.16 m at (0, 0.22, -0.28), radial FBM
// displacement of amplitude 0.05 (relative).  Base face f goes to material
// region f % 3: Lambert (4), metal with roughness U[0.05, 0.6] (5), glass
// IOR 1.5 (6).  One mesh per region.
void build_config1(wf_host_scene& s, uint64_t seed, int subdiv)
{
    add_room(s);
    uint64_t rs = seed;
    float rough = 0.05f + 0.55f * uniform01(rs);
    s.mats.push_back(diffuse(0.75f, 0.6f, 0.45f));     // 4
    s.mats.push_back(metal(0.9f, 0.85f, 0.8f, rough)); // 5
    s.mats.push_back(glass(1.5f));                     // 6
    // Icosahedron: golden-ratio rectangles.
    const float t = 1.61803399f;
    std::vector<P3> v = {{-1, t, 0}, {1, t, 0}, {-1, -t, 0}, {1, -t, 0}, {0, -1, t}, {0, 1, t},
                         {0, -1, -t}, {0, 1, -t}, {t, 0, -1}, {t, 0, 1}, {-t, 0, -1}, {-t, 0, 1}};
    for (P3& p : v) {
        float l = std::sqrt(p.x * p.x + p.y * p.y + p.z * p.z);
        p = {p.x / l, p.y / l, p.z / l};
    }
    const int base[20][3] = {{0, 11, 5}, {0, 5, 1},  {0, 1, 7},   {0, 7, 10}, {0, 10, 11},
                             {1, 5, 9},  {5, 11, 4}, {11, 10, 2}, {10, 7, 6}, {7, 1, 8},
                             {3, 9, 4},  {3, 4, 2},  {3, 2, 6},   {3, 6, 8},  {3, 8, 9},
                             {4, 9, 5},  {2, 4, 11}, {6, 2, 10},  {8, 6, 7},  {9, 8, 1}};
    struct Tri {
        int a, b, c, face;
    };
    std::vector<Tri> tris;
    for (int f = 0; f < 20; ++f) tris.push_back({base[f][0], base[f][1], base[f][2], f});
    for (int level = 0; level < subdiv; ++level) {
        std::unordered_map<uint64_t, int> mid;
        mid.reserve(tris.size() * 2);
        auto midpoint = [&](int a, int b) {
            uint64_t key = a < b ? ((uint64_t)a << 32 | (uint32_t)b) : ((uint64_t)b << 32 | (uint32_t)a);
            auto it = mid.find(key);
            if (it != mid.end()) return it->second;
            P3 m = {(v[a].x + v[b].x) * 0.5f, (v[a].y + v[b].y) * 0.5f, (v[a].z + v[b].z) * 0.5f};
            float l = std::sqrt(m.x * m.x + m.y * m.y + m.z * m.z);
            v.push_back({m.x / l, m.y / l, m.z / l});
            int id = (int)v.size() - 1;
            mid.emplace(key, id);
            return id;
        };
        std::vector<Tri> next;
        next.reserve(tris.size() * 4);
        for (const Tri& tr : tris) {
            int ab = midpoint(tr.a, tr.b), bc = midpoint(tr.b, tr.c), ca = midpoint(tr.c, tr.a);
            next.push_back({tr.a, ab, ca, tr.face});
            next.push_back({tr.b, bc, ab, tr.face});
            next.push_back({tr.c, ca, bc, tr.face});
            next.push_back({ab, bc, ca, tr.face});
        }
        tris.swap(next);
    }
    const float R = 0.16f, A = 0.05f, cx = 0.0f, cy = 0.22f, cz = -0.28f;
    const uint32_t nseed = (uint32_t)(seed ^ (seed >> 32));
    const int vbase = (int)s.px.size();
    for (const P3& p : v) {
        float n = fbm(p.x * 4.0f + 11.0f, p.y * 4.0f + 23.0f, p.z * 4.0f + 37.0f, nseed);
        float r = R * (1.0f + A * n);
        add_vertex(s, {cx + p.x * r, cy + p.y * r, cz + p.z * r});
    }
    for (int region = 0; region < 3; ++region) {
        begin_mesh(s, 4 + region);
        for (const Tri& tr : tris) {
            if (tr.face % 3 != region) continue;
            // keep the winding outward (glass reads frontFace)
            const P3 &a = v[tr.a], &b = v[tr.b], &c = v[tr.c];
            P3 e1 = {b.x - a.x, b.y - a.y, b.z - a.z}, e2 = {c.x - a.x, c.y - a.y, c.z - a.z};
            P3 n = {e1.y * e2.z - e1.z * e2.y, e1.z * e2.x - e1.x * e2.z, e1.x * e2.y - e1.y * e2.x};
            bool outward = n.x * (a.x + b.x + c.x) + n.y * (a.y + b.y + c.y) + n.z * (a.z + b.z + c.z) > 0.0f;
            s.idx.push_back(vbase + tr.a);
            s.idx.push_back(vbase + (outward ? tr.b : tr.c));
            s.idx.push_back(vbase + (outward ? tr.c : tr.b));
        }
        end_mesh(s);
    }
    set_camera(s);
}

// Config 3 job scenes: seeded variants of config 0 — wall, box and metal
// albedos, metal roughness, the light quad's position on the ceiling and a
// jitter of the camera position.
void build_config3(wf_host_scene& s, uint64_t seed)
{
    uint64_t rs = seed * 0x9E3779B97F4A7C15ull + 12345u;
    auto u = [&](float lo, float hi) { return lo + (hi - lo) * uniform01(rs); };
    const float g = u(0.5f, 0.85f);
    s.mats.push_back(diffuse(g, g, g));                                  // 0 white
    s.mats.push_back(diffuse(u(0.5f, 0.8f), u(0.02f, 0.1f), u(0.02f, 0.1f)));  // 1 red
    s.mats.push_back(diffuse(u(0.05f, 0.2f), u(0.3f, 0.6f), u(0.05f, 0.2f)));  // 2 green
    s.mats.push_back(emissive(17.0f, 12.0f, 4.0f, 1.0f));               // 3 light
    s.mats.push_back(metal(u(0.6f, 0.95f), u(0.6f, 0.95f), u(0.6f, 0.95f), u(0.1f, 0.5f)));  // 4 metal box
    const float b = u(0.4f, 0.9f);
    s.mats.push_back(diffuse(b, b, b));                                  // 5 short box
    const float X = 0.275f, Y = 0.55f, Z = -0.55f;
    add_quad(s, 0, {-X, 0, 0}, {X, 0, 0}, {X, 0, Z}, {-X, 0, Z});
    add_quad(s, 0, {-X, Y, Z}, {X, Y, Z}, {X, Y, 0}, {-X, Y, 0});
    add_quad(s, 0, {-X, 0, Z}, {X, 0, Z}, {X, Y, Z}, {-X, Y, Z});
    add_quad(s, 1, {-X, 0, 0}, {-X, 0, Z}, {-X, Y, Z}, {-X, Y, 0});
    add_quad(s, 2, {X, 0, Z}, {X, 0, 0}, {X, Y, 0}, {X, Y, Z});
    const float cx = u(-0.12f, 0.12f), cz = u(-0.42f, -0.13f), ly = Y - 0.001f;
    add_quad(s, 3, {cx - 0.065f, ly, cz - 0.055f}, {cx + 0.065f, ly, cz - 0.055f}, {cx + 0.065f, ly, cz + 0.055f},
             {cx - 0.065f, ly, cz + 0.055f});
    add_box(s, 4, {-0.19f, 0.0f, -0.42f}, {-0.025f, 0.33f, -0.255f}, 0.96592583f, 0.25881905f);
    add_box(s, 5, {0.0325f, 0.0f, -0.2225f}, {0.1975f, 0.165f, -0.0575f}, 0.95105652f, -0.30901699f);
    set_camera(s);
    s.look_from[0] += u(-0.03f, 0.03f);
    s.look_from[1] += u(-0.03f, 0.03f);
}

}  // namespace

extern "C" {

int wf_host_scene_generate(int32_t config, uint64_t seed, wf_host_scene** out)
{
    if (!out) return WF_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    wf_host_scene* s = new wf_host_scene();
    s->config = config;
    switch (config) {
    case 0:
        build_config0(*s);
        break;
    case 1:
        build_config1(*s, seed, 8);
        break;
    case 3:  // a job scene of the batched workload: variant `seed` of config 0
        build_config3(*s, seed);
        break;
    case 100:  // small variant of config 1 (subdivision 4) for fast tests
        build_config1(*s, seed, 4);
        break;
    default:
        delete s;
        return WF_ERR_INVALID_ARGUMENT;
    }
    *out = s;
    return WF_OK;
}

int wf_host_scene_describe(const wf_host_scene* s, wf_scene_desc* d)
{
    if (!s || !d) return WF_ERR_INVALID_ARGUMENT;
    std::memset(d, 0, sizeof(*d));
    d->num_vertices = (int32_t)s->px.size();
    d->positions_x = s->px.data();
    d->positions_y = s->py.data();
    d->positions_z = s->pz.data();
    d->num_indices = (int32_t)s->idx.size();
    d->indices = s->idx.data();
    d->num_meshes = (int32_t)s->mesh_off.size();
    d->mesh_index_offsets = s->mesh_off.data();
    d->mesh_index_counts = s->mesh_cnt.data();
    d->mesh_material_ids = s->mesh_mat.data();
    d->num_materials = (int32_t)s->mats.size();
    d->materials = s->mats.data();
    d->environment.intensity_scale = 1.0f;
    d->environment.tint[0] = d->environment.tint[1] = d->environment.tint[2] = 1.0f;
    d->directional.color[0] = d->directional.color[1] = d->directional.color[2] = 1.0f;
    return WF_OK;
}

int wf_host_scene_camera(const wf_host_scene* s, int32_t w, int32_t h, wf_camera* out)
{
    if (!s || !out) return WF_ERR_INVALID_ARGUMENT;
    return wf_camera_make(s->look_from, s->look_at, s->up, s->vfov, w, h, out);
}

int wf_host_scene_free(wf_host_scene* s)
{
    delete s;
    return WF_OK;
}

}  // extern "C"
