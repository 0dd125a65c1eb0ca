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

#include "wf_host_scene.h"

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

// Config 104: config 0 lit also by a directional light (the reference's
// DirectionalLight, include/core/Scene.h:57-62), with the short box made of
// glass, so the directional NEE of WavefrontRenderer.cpp:712-737 runs on
// Lambert, metal and glass hits.  The light comes in through the room's open
// front, from above and in front of the camera: direction normalize(0.35,
// -0.6, -1), warm white (1, 0.9, 0.75), intensity 1.5.
void build_config104(wf_host_scene& s)
{
    add_room(s);
    s.mats.push_back(metal(0.8f, 0.8f, 0.8f, 0.3f));  // 4 tall box, metal
    s.mats.push_back(glass(1.5f));                     // 5 short box, glass
    add_box(s, 4, {-0.19f, 0.0f, -0.42f}, {-0.025f, 0.33f, -0.255f}, 0.96592583f, 0.25881905f);
    add_box(s, 5, {0.0325f, 0.0f, -0.2225f}, {0.1975f, 0.165f, -0.0575f}, 0.95105652f, -0.30901699f);
    s.dir = wf_directional_light{{0.28745555f, -0.49278094f, -0.82130156f}, {1.0f, 0.9f, 0.75f}, 1.5f};
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

// --- config 2: the shading-divergence stress scene ------------------------

struct LocalMesh {
    std::vector<P3> v;
    std::vector<int> t;  // 3 per triangle
};

LocalMesh icosphere_local(int subdiv)
{
    const float tt = 1.61803399f;
    LocalMesh m;
    m.v = {{-1, tt, 0}, {1, tt, 0}, {-1, -tt, 0}, {1, -tt, 0}, {0, -1, tt}, {0, 1, tt},
           {0, -1, -tt}, {0, 1, -tt}, {tt, 0, -1}, {tt, 0, 1}, {-tt, 0, -1}, {-tt, 0, 1}};
    for (P3& p : m.v) {
        float l = std::sqrt(p.x * p.x + p.y * p.y + p.z * p.z);
        p = {p.x / l, p.y / l, p.z / l};
    }
    m.t = {0, 11, 5, 0, 5, 1, 0, 1, 7, 0, 7, 10, 0, 10, 11, 1, 5, 9, 5, 11, 4, 11, 10, 2, 10, 7, 6, 7, 1, 8,
           3, 9, 4, 3, 4, 2, 3, 2, 6, 3, 6, 8, 3, 8, 9, 4, 9, 5, 2, 4, 11, 6, 2, 10, 8, 6, 7, 9, 8, 1};
    for (int level = 0; level < subdiv; ++level) {
        std::unordered_map<uint64_t, int> mid;
        auto midpoint = [&](int a, int b) {
            uint64_t key = a < b ? ((uint64_t)a << 32 | (uint32_t)b) : ((uint64_t)b << 32 | (uint32_t)a);
            auto it = mid.find(key);
            if (it != mid.end()) return it->second;
            P3 q = {(m.v[a].x + m.v[b].x) * 0.5f, (m.v[a].y + m.v[b].y) * 0.5f, (m.v[a].z + m.v[b].z) * 0.5f};
            float l = std::sqrt(q.x * q.x + q.y * q.y + q.z * q.z);
            m.v.push_back({q.x / l, q.y / l, q.z / l});
            mid.emplace(key, (int)m.v.size() - 1);
            return (int)m.v.size() - 1;
        };
        std::vector<int> next;
        for (size_t i = 0; i < m.t.size(); i += 3) {
            int a = m.t[i], b = m.t[i + 1], c = m.t[i + 2];
            int ab = midpoint(a, b), bc = midpoint(b, c), ca = midpoint(c, a);
            int tri[12] = {a, ab, ca, b, bc, ab, c, ca, bc, ab, bc, ca};
            next.insert(next.end(), tri, tri + 12);
        }
        m.t.swap(next);
    }
    return m;
}

// Torus around the y axis; angles from double-precision cos/sin rounded to
// float (the only libm use in the generators).
LocalMesh torus_local(int nu, int nv, float R, float r)
{
    LocalMesh m;
    for (int i = 0; i < nu; ++i) {
        const double a = 2.0 * 3.14159265358979323846 * i / nu;
        const float ca = (float)std::cos(a), sa = (float)std::sin(a);
        for (int j = 0; j < nv; ++j) {
            const double b = 2.0 * 3.14159265358979323846 * j / nv;
            const float cb = (float)std::cos(b), sb = (float)std::sin(b);
            m.v.push_back({(R + r * cb) * ca, r * sb, (R + r * cb) * sa});
        }
    }
    for (int i = 0; i < nu; ++i)
        for (int j = 0; j < nv; ++j) {
            int a = i * nv + j, b = ((i + 1) % nu) * nv + j, c = ((i + 1) % nu) * nv + (j + 1) % nv,
                d = i * nv + (j + 1) % nv;
            int tri[6] = {a, b, c, a, c, d};
            m.t.insert(m.t.end(), tri, tri + 6);
        }
    return m;
}

// Cube [-1,1]^3 with every face split into n x n quads.
LocalMesh cube_local(int n)
{
    LocalMesh m;
    const int axes[6][3] = {{0, 1, 2}, {0, 1, 2}, {1, 2, 0}, {1, 2, 0}, {2, 0, 1}, {2, 0, 1}};
    for (int f = 0; f < 6; ++f) {
        const float sgn = (f % 2) ? -1.0f : 1.0f;
        const int base = (int)m.v.size();
        for (int i = 0; i <= n; ++i)
            for (int j = 0; j <= n; ++j) {
                float c[3];
                c[axes[f][0]] = -1.0f + 2.0f * i / n;
                c[axes[f][1]] = -1.0f + 2.0f * j / n;
                c[axes[f][2]] = sgn;
                m.v.push_back({c[0], c[1], c[2]});
            }
        for (int i = 0; i < n; ++i)
            for (int j = 0; j < n; ++j) {
                int a = base + i * (n + 1) + j, b = a + n + 1, c = b + 1, d = a + 1;
                if (sgn > 0) {
                    int tri[6] = {a, b, c, a, c, d};
                    m.t.insert(m.t.end(), tri, tri + 6);
                } else {
                    int tri[6] = {a, c, b, a, d, c};
                    m.t.insert(m.t.end(), tri, tri + 6);
                }
            }
    }
    return m;
}

// 512x512 RGBA8 texture: a checker (even ids) or value noise (odd ids).
std::vector<uint32_t> make_texture(int id, int size, uint64_t seed)
{
    std::vector<uint32_t> px((size_t)size * size);
    uint64_t rs = seed * 977u + (uint64_t)id * 0x9E3779B97F4A7C15ull;
    uint8_t ca[3], cb[3];
    for (int k = 0; k < 3; ++k) {
        ca[k] = (uint8_t)(40 + (splitmix64(rs) % 200));
        cb[k] = (uint8_t)(40 + (splitmix64(rs) % 200));
    }
    const int cell = 8 + (int)(splitmix64(rs) % 56);
    const uint32_t nseed = (uint32_t)splitmix64(rs);
    for (int y = 0; y < size; ++y)
        for (int x = 0; x < size; ++x) {
            uint8_t c[3];
            if (id % 2 == 0) {
                const bool odd = ((x / cell) + (y / cell)) % 2;
                for (int k = 0; k < 3; ++k) c[k] = odd ? ca[k] : cb[k];
            } else {
                float nz = 0.5f + 0.5f * fbm(x * 0.02f, y * 0.02f, 0.5f, nseed);
                nz = std::fmin(1.0f, std::fmax(0.0f, nz));
                for (int k = 0; k < 3; ++k) c[k] = (uint8_t)(ca[k] * nz + cb[k] * (1.0f - nz));
            }
            px[(size_t)y * size + x] = (uint32_t)c[0] | ((uint32_t)c[1] << 8) | ((uint32_t)c[2] << 16) | 0xFF000000u;
        }
    return px;
}

// Equirect HDRI in the mapping of EnvironmentMap::sample (u = 0.5 +
// atan2(z,x)/2pi, v = 0.5 - asin(y)/pi): a sky gradient, a dim ground and a
// sun lobe `sun` times brighter than the sky around it.
void make_hdri(wf_host_scene& s, int w, int h, float sun)
{
    s.env_w = w;
    s.env_h = h;
    s.env.assign((size_t)w * h * 3, 0.0f);
    const double pi = 3.14159265358979323846;
    const double se = 35.0 * pi / 180.0, sp = 40.0 * pi / 180.0;
    const double sx = std::cos(se) * std::cos(sp), sy = std::sin(se), sz = std::cos(se) * std::sin(sp);
    const double cos_r = std::cos(1.5 * pi / 180.0);
    for (int y = 0; y < h; ++y) {
        const double elev = (0.5 - (y + 0.5) / h) * pi;
        const double dyv = std::sin(elev), ce = std::cos(elev);
        for (int x = 0; x < w; ++x) {
            const double phi = ((x + 0.5) / w - 0.5) * 2.0 * pi;
            const double dx = ce * std::cos(phi), dz = ce * std::sin(phi);
            double r, g, b;
            if (dyv >= 0.0) {
                const double t = std::pow(dyv, 0.5);
                r = 0.9 * (1 - t) + 0.25 * t;
                g = 0.85 * (1 - t) + 0.45 * t;
                b = 0.8 * (1 - t) + 0.9 * t;
            } else {
                r = 0.18;
                g = 0.17;
                b = 0.16;
            }
            const double cd = dx * sx + dyv * sy + dz * sz;
            if (cd > cos_r) {
                const double f = (cd - cos_r) / (1.0 - cos_r);
                const double k = 1.0 + (sun - 1.0) * std::sqrt(f);
                r *= k;
                g *= k * 0.95;
                b *= k * 0.85;
            }
            float* o = &s.env[((size_t)y * w + x) * 3];
            o[0] = (float)r;
            o[1] = (float)g;
            o[2] = (float)b;
        }
    }
}

// Config 2: a grid x grid lattice of meshes (icospheres, tori, subdivided
// cubes of ~1.3k-20k triangles) resting on a ground quad, 256 materials
// spread evenly over Diffuse / Metal / Glass, the first 64 non-glass ones
// textured (512^2 RGBA8 checker or noise, planar UVs), lit by an HDRI with a
// sun lobe of 1e4.
void build_config2(wf_host_scene& s, uint64_t seed, int grid, int tex_size, int env_w, int env_h)
{
    uint64_t rs = seed * 0xD1B54A32D192ED03ull + 77u;
    auto u = [&](float lo, float hi) { return lo + (hi - lo) * uniform01(rs); };
    const int nmat = 256, ntex = 64;
    int textured = 0;
    for (int m = 0; m < nmat; ++m) {
        const int type = m % 3;
        wf_material mt;
        if (type == 0)
            mt = diffuse(u(0.2f, 0.9f), u(0.2f, 0.9f), u(0.2f, 0.9f));
        else if (type == 1)
            mt = metal(u(0.5f, 0.95f), u(0.5f, 0.95f), u(0.5f, 0.95f), u(0.05f, 0.5f));
        else
            mt = glass(1.5f);
        if (type != 2 && textured < ntex) mt.texture_id = textured++;
        s.mats.push_back(mt);
    }
    const int ground_mat = (int)s.mats.size();
    s.mats.push_back(diffuse(0.45f, 0.45f, 0.42f));
    for (int t = 0; t < ntex; ++t) {
        const std::vector<uint32_t> px = make_texture(t, tex_size, seed);
        std::vector<uint8_t> raw(px.size() * 4);
        std::memcpy(raw.data(), px.data(), raw.size());
        s.tex_data.push_back(std::move(raw));
        s.textures.push_back(wf_texture{tex_size, tex_size, WF_TEXEL_RGBA8_SRGB, nullptr});
    }
    // ground
    const float G = (float)grid;
    begin_mesh(s, ground_mat);
    {
        int a = add_vertex(s, {-1, 0, -1}), b = add_vertex(s, {G + 1, 0, -1}), c = add_vertex(s, {G + 1, 0, G + 1}),
            d = add_vertex(s, {-1, 0, G + 1});
        int tri[6] = {a, b, c, a, c, d};
        s.idx.insert(s.idx.end(), tri, tri + 6);
        for (int k = 0; k < 6; ++k) {
            s.cu.push_back(0.0f);
            s.cv.push_back(0.0f);
        }
    }
    end_mesh(s);
    s.has_uv.push_back(0);
    const LocalMesh shapes[9] = {icosphere_local(3), icosphere_local(4), icosphere_local(5),
                                 torus_local(40, 26, 1.0f, 0.35f), torus_local(80, 64, 1.0f, 0.35f),
                                 torus_local(128, 80, 1.0f, 0.35f), cube_local(10), cube_local(20), cube_local(40)};
    for (int gz = 0; gz < grid; ++gz)
        for (int gx = 0; gx < grid; ++gx) {
            const float pick = uniform01(rs);
            const int size_class = pick < 0.72f ? 0 : (pick < 0.95f ? 1 : 2);
            const int kind = (int)(splitmix64(rs) % 3);
            const LocalMesh& L = shapes[kind * 3 + size_class];
            const int mat = (int)(splitmix64(rs) % nmat);
            const float scale = u(0.28f, 0.42f);
            const float t = u(-1.0f, 1.0f);  // rotation about y: cos/sin from tan(angle/2) = t
            const float ca = (1.0f - t * t) / (1.0f + t * t), sa = 2.0f * t / (1.0f + t * t);
            const float cx = gx + 0.5f + u(-0.08f, 0.08f), cz = gz + 0.5f + u(-0.08f, 0.08f);
            const float lift = kind == 1 ? 0.35f : 1.0f;  // the torus is 0.35 tall
            const float cy = scale * lift;
            begin_mesh(s, mat);
            const int base = (int)s.px.size();
            for (const P3& p : L.v) {
                const float x = p.x * scale, y = p.y * scale, z = p.z * scale;
                add_vertex(s, {ca * x - sa * z + cx, y + cy, sa * x + ca * z + cz});
            }
            for (size_t i = 0; i < L.t.size(); ++i) {
                s.idx.push_back(base + L.t[i]);
                const P3& p = L.v[L.t[i]];
                s.cu.push_back(0.5f + 0.5f * p.x);
                s.cv.push_back(0.5f + 0.5f * p.y);
            }
            end_mesh(s);
            s.has_uv.push_back(s.mats[mat].texture_id >= 0 ? 1 : 0);
        }
    make_hdri(s, env_w, env_h, 1.0e4f);
    const float f[3] = {G * 0.5f, G * 0.28f, G * 1.12f}, a[3] = {G * 0.5f, 0.0f, G * 0.38f}, up[3] = {0, 1, 0};
    std::memcpy(s.look_from, f, sizeof(f));
    std::memcpy(s.look_at, a, sizeof(a));
    std::memcpy(s.up, up, sizeof(up));
    s.vfov = 50.0f;
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
    case 2:
        build_config2(*s, seed, 64, 512, 2048, 1024);
        break;
    case 102:  // small variant of config 2 (16 x 16 meshes, 128^2 textures, 256x128 HDRI)
        build_config2(*s, seed, 16, 128, 256, 128);
        break;
    case 100:  // small variant of config 1 (subdivision 4) for fast tests
        build_config1(*s, seed, 4);
        break;
    case 104:  // config 0 with a directional light and a glass box
        build_config104(*s);
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
    if (!s->cu.empty()) {
        d->corner_u = s->cu.data();
        d->corner_v = s->cv.data();
        d->mesh_has_uv = s->has_uv.data();
    }
    if (!s->textures.empty()) {
        auto* tex = const_cast<wf_host_scene*>(s);
        for (size_t t = 0; t < tex->textures.size(); ++t) tex->textures[t].data = tex->tex_data[t].data();
        d->num_textures = (int32_t)s->textures.size();
        d->textures = s->textures.data();
    }
    if (s->env_w > 0) {
        d->environment.width = s->env_w;
        d->environment.height = s->env_h;
        d->environment.rgb = s->env.data();
    }
    d->environment.intensity_scale = s->env_scale;
    for (int k = 0; k < 3; ++k) d->environment.tint[k] = s->env_tint[k];
    d->directional = s->dir;
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
