// wf_oracle.cpp — CPU restatement of the reference's per-bounce loop.
// TEST INFRASTRUCTURE ONLY (see wf_oracle.h).  Every function names the
// reference file:line it restates (fhidargue/wavefront-renderer).
// Build: -O2 -std=c++17 -ffp-contract=off (no fused multiply-add).

#include "wf_oracle.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <limits>
#include <numeric>
#include <thread>
#include <unordered_map>
#include <vector>

namespace {

// ---------------------------------------------------------------------------
// Vector arithmetic with the reference's operation order
// (include/math/Vec3.h:8-77): component-wise ops, dot = (x*x' + y*y') + z*z',
// normalized = v / length().
// ---------------------------------------------------------------------------
struct V3 {
    float x, y, z;
};
inline V3 operator+(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V3 operator-(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 operator*(V3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
inline V3 operator/(V3 a, float s) { return {a.x / s, a.y / s, a.z / s}; }
inline V3 operator*(V3 a, V3 b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
inline float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline V3 cross(V3 a, V3 b)
{
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
inline float length(V3 a) { return std::sqrt(a.x * a.x + a.y * a.y + a.z * a.z); }
inline V3 normalized(V3 a) { return a / length(a); }

constexpr float kPi = 3.14159265f;  // WavefrontRenderer.h:22, Material.cpp:8

// ---------------------------------------------------------------------------
// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as easy
// as 1, 2, 3", SC'11): 10 rounds of two 32x32->64 multiplies, key bumped by
// the Weyl constants between rounds.
// ---------------------------------------------------------------------------
inline void philox10(const uint32_t in[4], const uint32_t key[2], uint32_t out[4])
{
    uint32_t c0 = in[0], c1 = in[1], c2 = in[2], c3 = in[3];
    uint32_t k0 = key[0], k1 = key[1];
    for (int r = 0; r < 10; ++r) {
        if (r > 0) {
            k0 += 0x9E3779B9u;
            k1 += 0xBB67AE85u;
        }
        uint64_t p0 = (uint64_t)0xD2511F53u * c0;
        uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
        uint32_t n0 = (uint32_t)(p1 >> 32) ^ c1 ^ k0;
        uint32_t n1 = (uint32_t)p1;
        uint32_t n2 = (uint32_t)(p0 >> 32) ^ c3 ^ k1;
        uint32_t n3 = (uint32_t)p0;
        c0 = n0;
        c1 = n1;
        c2 = n2;
        c3 = n3;
    }
    out[0] = c0;
    out[1] = c1;
    out[2] = c2;
    out[3] = c3;
}

// Random-number purposes.  Each (purpose, depth) of a path is its own stream,
// so the numbers a path sees do not depend on queue order or batching.
enum : uint32_t { kPurposeCamera = 1, kPurposeLight = 2, kPurposeScatter = 3, kPurposeRoulette = 4, kPurposeEnvironment = 5 };

// A sequential stream of floats in [0, 1) with 24 random bits each.
struct Stream {
    uint32_t key[2];
    uint32_t ctr[4];
    uint32_t buf[4];
    int used = 4;
    Stream(uint32_t seed_lo, uint32_t seed_hi, uint32_t purpose, uint32_t depth, uint32_t pixel,
           uint32_t sample)
    {
        key[0] = seed_lo;
        key[1] = seed_hi;
        ctr[0] = 0;
        ctr[1] = (purpose << 16) | (depth & 0xFFFFu);
        ctr[2] = pixel;
        ctr[3] = sample;
    }
    float next()
    {
        if (used == 4) {
            philox10(ctr, key, buf);
            ctr[0] += 1;
            used = 0;
        }
        uint32_t x = buf[used++];
        return (float)(x >> 8) * (1.0f / 16777216.0f);
    }
};

// ---------------------------------------------------------------------------
// Scene
// ---------------------------------------------------------------------------
struct Tex {
    int w = 0, h = 0;
    std::vector<float> rgb;  // linear float RGB, Texture::pixels
};

struct BNode {
    float lo[3], hi[3];
    int left = -1, right = -1;  // children (internal)
    int first = 0, count = 0;   // leaf range in bvh_tris (count > 0)
};

}  // namespace

struct orc_scene {
    std::vector<float> px, py, pz;
    std::vector<int> idx;
    std::vector<int> mesh_off, mesh_cnt, mesh_mat;
    std::vector<float> cu, cv;
    std::vector<uint8_t> has_uv;
    std::vector<wf_material> mats;
    std::vector<Tex> texs;
    int env_w = 0, env_h = 0;
    std::vector<float> env_rgb;
    float env_scale = 1.0f;
    float env_tint[3] = {1, 1, 1};
    // environment importance sampler (no reference counterpart)
    std::vector<float> env_prob, env_pdf;
    std::vector<int> env_alias;
    wf_directional_light dir{};
    // derived
    std::vector<int> tri_mesh;        // global triangle -> mesh (geomID)
    std::vector<int> mesh_first_tri;  // mesh -> first global triangle
    std::vector<int> emissive_meshes; // Scene::emissiveMeshIndices
    float total_emissive_area = 0.0f;
    float bmin[3], bmax[3];
    std::vector<BNode> nodes;
    std::vector<int> bvh_tris;  // global triangle ids in leaf order

    int num_tris() const { return (int)(idx.size() / 3); }
    V3 vert(int gi) const { return {px[gi], py[gi], pz[gi]}; }
    void tri_verts(int t, V3& a, V3& b, V3& c) const
    {
        a = vert(idx[3 * t + 0]);
        b = vert(idx[3 * t + 1]);
        c = vert(idx[3 * t + 2]);
    }
};

namespace {

// srgbToLinear, reference src/shading/Texture.cpp:20-27; 8-bit sources are
// first scaled to [0,1] by /255 (the image loader's float conversion).
float srgb_to_linear(float s)
{
    if (s <= 0.04045f) return s / 12.92f;
    return std::pow((s + 0.055f) / 1.055f, 2.4f);
}

// Moller-Trumbore, reference include/geometry/Triangle.h:6-43, operation for
// operation.
inline bool intersect_triangle(V3 o, V3 d, V3 v0, V3 v1, V3 v2, float tmin, float tmax,
                               float& t_out, float& u_out, float& v_out)
{
    const float eps = 0.0000001f;
    V3 e1 = v1 - v0;
    V3 e2 = v2 - v0;
    V3 p = cross(d, e2);
    float det = dot(e1, p);
    if (det > -eps && det < eps) return false;
    float inv = 1.0f / det;
    V3 s = o - v0;
    float u = inv * dot(s, p);
    if (u < 0.0f || u > 1.0f) return false;
    V3 q = cross(s, e1);
    float v = inv * dot(d, q);
    if (v < 0.0f || u + v > 1.0f) return false;
    float t = inv * dot(e2, q);
    if (t < tmin || t > tmax) return false;
    t_out = t;
    u_out = u;
    v_out = v;
    return true;
}

// --- CPU BVH: median split on the widest centroid axis, leaves <= 4 ------
// Boxes are padded by a small relative margin so that a triangle accepted by
// Moller-Trumbore can never sit in a box the slab test rejects.
void build_bvh(orc_scene& S)
{
    const int n = S.num_tris();
    S.bvh_tris.resize(n);
    std::iota(S.bvh_tris.begin(), S.bvh_tris.end(), 0);
    S.nodes.clear();
    if (n == 0) return;
    std::vector<float> cx(n), cy(n), cz(n), lo(3 * (size_t)n), hi(3 * (size_t)n);
    for (int t = 0; t < n; ++t) {
        V3 a, b, c;
        S.tri_verts(t, a, b, c);
        float l[3] = {std::min({a.x, b.x, c.x}), std::min({a.y, b.y, c.y}), std::min({a.z, b.z, c.z})};
        float h[3] = {std::max({a.x, b.x, c.x}), std::max({a.y, b.y, c.y}), std::max({a.z, b.z, c.z})};
        for (int k = 0; k < 3; ++k) {
            lo[3 * (size_t)t + k] = l[k];
            hi[3 * (size_t)t + k] = h[k];
        }
        cx[t] = 0.5f * (l[0] + h[0]);
        cy[t] = 0.5f * (l[1] + h[1]);
        cz[t] = 0.5f * (l[2] + h[2]);
    }
    S.nodes.reserve(2 * (size_t)n / 2 + 16);
    struct Job {
        int node, first, count;
    };
    std::vector<Job> stack;
    S.nodes.push_back(BNode{});
    stack.push_back({0, 0, n});
    while (!stack.empty()) {
        Job j = stack.back();
        stack.pop_back();
        float bl[3] = {INFINITY, INFINITY, INFINITY}, bh[3] = {-INFINITY, -INFINITY, -INFINITY};
        float cl[3] = {INFINITY, INFINITY, INFINITY}, ch[3] = {-INFINITY, -INFINITY, -INFINITY};
        for (int i = j.first; i < j.first + j.count; ++i) {
            int t = S.bvh_tris[i];
            for (int k = 0; k < 3; ++k) {
                bl[k] = std::min(bl[k], lo[3 * (size_t)t + k]);
                bh[k] = std::max(bh[k], hi[3 * (size_t)t + k]);
            }
            float c3[3] = {cx[t], cy[t], cz[t]};
            for (int k = 0; k < 3; ++k) {
                cl[k] = std::min(cl[k], c3[k]);
                ch[k] = std::max(ch[k], c3[k]);
            }
        }
        BNode& nd = S.nodes[j.node];
        for (int k = 0; k < 3; ++k) {
            float mag = std::max(std::fabs(bl[k]), std::fabs(bh[k]));
            float pad = mag * 1e-5f + 1e-6f;
            nd.lo[k] = bl[k] - pad;
            nd.hi[k] = bh[k] + pad;
        }
        if (j.count <= 4) {
            nd.first = j.first;
            nd.count = j.count;
            continue;
        }
        int axis = 0;
        float ext[3] = {ch[0] - cl[0], ch[1] - cl[1], ch[2] - cl[2]};
        if (ext[1] > ext[axis]) axis = 1;
        if (ext[2] > ext[axis]) axis = 2;
        const std::vector<float>& key = axis == 0 ? cx : (axis == 1 ? cy : cz);
        int mid = j.first + j.count / 2;
        std::nth_element(S.bvh_tris.begin() + j.first, S.bvh_tris.begin() + mid,
                         S.bvh_tris.begin() + j.first + j.count,
                         [&](int a, int b) { return key[a] < key[b] || (key[a] == key[b] && a < b); });
        int left = (int)S.nodes.size();
        S.nodes.push_back(BNode{});
        S.nodes.push_back(BNode{});
        S.nodes[j.node].left = left;
        S.nodes[j.node].right = left + 1;
        stack.push_back({left, j.first, mid - j.first});
        stack.push_back({left + 1, mid, j.first + j.count - mid});
    }
}

inline bool slab(const BNode& nd, V3 o, V3 inv, float tmin, float tmax, float& tnear)
{
    float t0x = (nd.lo[0] - o.x) * inv.x, t1x = (nd.hi[0] - o.x) * inv.x;
    float t0y = (nd.lo[1] - o.y) * inv.y, t1y = (nd.hi[1] - o.y) * inv.y;
    float t0z = (nd.lo[2] - o.z) * inv.z, t1z = (nd.hi[2] - o.z) * inv.z;
    float a = std::max({std::min(t0x, t1x), std::min(t0y, t1y), std::min(t0z, t1z), tmin});
    float b = std::min({std::max(t0x, t1x), std::max(t0y, t1y), std::max(t0z, t1z), tmax});
    tnear = a;
    return a <= b;
}

inline float safe_inv(float d)
{
    if (std::fabs(d) < 1e-20f) d = std::copysign(1e-20f, d);
    return 1.0f / d;
}

struct Closest {
    int tri = -1;
    float t, bu, bv;
};

// Closest hit with brute-force tie semantics: smallest t, then the larger
// global triangle index (the later mesh / triangle wins on equal t, as in
// Scene::hit and Mesh::hit where intersectTriangle accepts t == maxDistance).
Closest closest_bvh(const orc_scene& S, V3 o, V3 d, float tmin, float tmax)
{
    Closest best;
    if (S.nodes.empty()) return best;
    float best_t = tmax;
    V3 inv = {safe_inv(d.x), safe_inv(d.y), safe_inv(d.z)};
    int stack[128];
    int sp = 0;
    stack[sp++] = 0;
    while (sp) {
        const BNode& nd = S.nodes[stack[--sp]];
        float tn;
        if (!slab(nd, o, inv, tmin, best_t, tn)) continue;
        if (nd.count > 0) {
            for (int i = nd.first; i < nd.first + nd.count; ++i) {
                int t = S.bvh_tris[i];
                V3 a, b, c;
                S.tri_verts(t, a, b, c);
                float th, uh, vh;
                if (intersect_triangle(o, d, a, b, c, tmin, best_t, th, uh, vh)) {
                    if (th < best_t || best.tri < 0 || t > best.tri) {
                        best.tri = t;
                        best.t = th;
                        best.bu = uh;
                        best.bv = vh;
                        best_t = th;
                    }
                }
            }
        } else {
            float tl, tr;
            bool hl = slab(S.nodes[nd.left], o, inv, tmin, best_t, tl);
            bool hr = slab(S.nodes[nd.right], o, inv, tmin, best_t, tr);
            if (hl && hr) {
                if (tl <= tr) {
                    stack[sp++] = nd.right;
                    stack[sp++] = nd.left;
                } else {
                    stack[sp++] = nd.left;
                    stack[sp++] = nd.right;
                }
            } else if (hl) {
                stack[sp++] = nd.left;
            } else if (hr) {
                stack[sp++] = nd.right;
            }
        }
    }
    return best;
}

bool occluded_bvh(const orc_scene& S, V3 o, V3 d, float max_distance)
{
    if (S.nodes.empty()) return false;
    const float tmin = 0.001f, tmax = max_distance - 0.001f;  // Embree.cpp:268-269
    V3 inv = {safe_inv(d.x), safe_inv(d.y), safe_inv(d.z)};
    int stack[128];
    int sp = 0;
    stack[sp++] = 0;
    while (sp) {
        const BNode& nd = S.nodes[stack[--sp]];
        float tn;
        if (!slab(nd, o, inv, tmin, tmax, tn)) continue;
        if (nd.count > 0) {
            for (int i = nd.first; i < nd.first + nd.count; ++i) {
                V3 a, b, c;
                S.tri_verts(S.bvh_tris[i], a, b, c);
                float th, uh, vh;
                if (intersect_triangle(o, d, a, b, c, tmin, tmax, th, uh, vh)) return true;
            }
        } else {
            stack[sp++] = nd.left;
            stack[sp++] = nd.right;
        }
    }
    return false;
}

// HitRecord as EmbreeAccelerator::intersect4 fills it (Embree.cpp:224-252).
struct Hit {
    int geom, prim, mat, tex;
    float t, bu, bv, u, v;
    V3 p, n;
    bool front;
};

// Mesh::interpolateUV, reference src/geometry/Mesh.cpp:46-63.
void interpolate_uv(const orc_scene& S, int mesh, int tri, float bu, float bv, float& u, float& v)
{
    if (S.has_uv.empty() || !S.has_uv[mesh] || S.cu.empty()) {
        u = bu;
        v = bv;
        return;
    }
    size_t c = 3 * (size_t)tri;
    float w0 = 1.0f - bu - bv;
    u = w0 * S.cu[c + 0] + bu * S.cu[c + 1] + bv * S.cu[c + 2];
    v = w0 * S.cv[c + 0] + bu * S.cv[c + 1] + bv * S.cv[c + 2];
}

void make_hit(const orc_scene& S, V3 o, V3 d, const Closest& c, Hit& h)
{
    int mesh = S.tri_mesh[c.tri];
    h.geom = mesh;
    h.prim = c.tri - S.mesh_first_tri[mesh];
    h.t = c.t;
    h.bu = c.bu;
    h.bv = c.bv;
    h.p = o + d * c.t;                       // Ray::at, include/core/Ray.h:21-24
    h.mat = S.mesh_mat[mesh];
    h.tex = S.mats[h.mat].texture_id;        // Embree.cpp:244 (intersect4 only)
    interpolate_uv(S, mesh, c.tri, c.bu, c.bv, h.u, h.v);
    V3 a, b, cc;
    S.tri_verts(c.tri, a, b, cc);
    V3 outward = normalized(cross(b - a, cc - a));
    h.front = dot(d, outward) < 0.0f;        // HitRecord::setFaceNormal, HitRecord.h:17-21
    h.n = h.front ? outward : outward * -1.0f;
}

void write_hit(wf_hit_columns* out, int64_t i, const Hit* h)
{
    if (!out) return;
    if (out->geom_id) out->geom_id[i] = h ? h->geom : -1;
    if (out->prim_id) out->prim_id[i] = h ? h->prim : -1;
    if (out->distance) out->distance[i] = h ? h->t : 0.0f;
    if (out->bary_u) out->bary_u[i] = h ? h->bu : 0.0f;
    if (out->bary_v) out->bary_v[i] = h ? h->bv : 0.0f;
    if (out->point_x) out->point_x[i] = h ? h->p.x : 0.0f;
    if (out->point_y) out->point_y[i] = h ? h->p.y : 0.0f;
    if (out->point_z) out->point_z[i] = h ? h->p.z : 0.0f;
    if (out->normal_x) out->normal_x[i] = h ? h->n.x : 0.0f;
    if (out->normal_y) out->normal_y[i] = h ? h->n.y : 0.0f;
    if (out->normal_z) out->normal_z[i] = h ? h->n.z : 0.0f;
    if (out->front_face) out->front_face[i] = h ? (uint8_t)h->front : 0;
    if (out->u) out->u[i] = h ? h->u : 0.0f;
    if (out->v) out->v[i] = h ? h->v : 0.0f;
    if (out->material_id) out->material_id[i] = h ? h->mat : -1;
    if (out->texture_id) out->texture_id[i] = h ? h->tex : -1;
}

// Texture::sample, include/shading/Texture.h:34-46.
V3 texture_sample(const Tex& t, float u, float v)
{
    u = u - std::floor(u);
    v = v - std::floor(v);
    int x = (int)(u * t.w);
    int y = (int)(v * t.h);
    x = std::max(0, std::min(x, t.w - 1));
    y = std::max(0, std::min(y, t.h - 1));
    size_t k = 3 * ((size_t)y * t.w + x);
    return {t.rgb[k], t.rgb[k + 1], t.rgb[k + 2]};
}

// hashGridCell / hashToUV, include/math/SpatialHash.h:18-45 (Teschner et al.
// spatial hash primes, Knuth multiplicative constant).
inline uint32_t hash_grid_cell(int x, int y, int z)
{
    uint32_t h = (uint32_t)x * 73856093u ^ (uint32_t)y * 19349663u ^ (uint32_t)z * 83492791u;
    return h * 2654435761u;
}

// Material::getSurfaceColor, src/shading/Material.cpp:143-163.
V3 surface_color(const orc_scene& S, const wf_material& m, const Hit& h)
{
    int tid = m.texture_id;
    bool valid = tid >= 0 && tid < (int)S.texs.size();
    if (m.use_spatial_checker && valid) {
        int cx = (int)std::floor(h.p.x / m.checker_cell_size);
        int cy = (int)std::floor(h.p.y / m.checker_cell_size);
        int cz = (int)std::floor(h.p.z / m.checker_cell_size);
        uint32_t hh = hash_grid_cell(cx, cy, cz);
        float pu = ((hh >> 16) & 0xFFFFu) / 65535.0f;
        float pv = (hh & 0xFFFFu) / 65535.0f;
        return texture_sample(S.texs[tid], pu, pv);
    }
    if (valid) return texture_sample(S.texs[tid], h.u, h.v);
    return {m.albedo[0], m.albedo[1], m.albedo[2]};
}

// Material::emitted, src/shading/Material.cpp:268-296.
V3 emitted(const wf_material& m, V3 light_normal, V3 dir_from_light)
{
    V3 alb = {m.albedo[0], m.albedo[1], m.albedo[2]};
    if (m.type == WF_MATERIAL_EMISSIVE) return alb * m.emission;
    if (m.type == WF_MATERIAL_SPOTLIGHT) {
        V3 radiance = alb * m.emission;
        float c = dot(light_normal, dir_from_light);
        float ang = std::acos(std::max(-1.0f, std::min(1.0f, c))) * (180.0f / kPi);
        if (ang >= m.spot_outer_deg) return {0, 0, 0};
        if (ang > m.spot_falloff_deg) {
            float t = (ang - m.spot_falloff_deg) / (m.spot_outer_deg - m.spot_falloff_deg);
            float f = 1.0f - t;
            f = f * f * (3.0f - 2.0f * f);
            radiance = radiance * f;
        }
        return radiance;
    }
    return {0, 0, 0};
}

// randomInUnitSphere (Material.cpp:10-19): rejection sampling; the stream
// gives up after 64 rejections (probability ~1e-21) and returns the origin.
V3 random_in_unit_sphere(Stream& rng)
{
    for (int k = 0; k < 64; ++k) {
        V3 c;
        c.x = rng.next() * 2.0f - 1.0f;
        c.y = rng.next() * 2.0f - 1.0f;
        c.z = rng.next() * 2.0f - 1.0f;
        if (dot(c, c) < 1.0f) return c;
    }
    return {0, 0, 0};
}

inline V3 reflect(V3 in, V3 n) { return in - n * 2.0f * dot(in, n); }  // Material.cpp:21-24

V3 refract(V3 in, V3 n, float eta)  // Material.cpp:26-37
{
    float c = std::min(1.0f, dot(in * -1.0f, n));
    V3 perp = (in + n * c) * eta;
    V3 par = n * -std::sqrt(std::fabs(1.0f - dot(perp, perp)));
    return perp + par;
}

float schlick(float c, float eta)  // Material.cpp:39-46
{
    float r0 = (1.0f - eta) / (1.0f + eta);
    r0 = r0 * r0;
    return r0 + (1.0f - r0) * std::pow((1.0f - c), 5.0f);
}

V3 cosine_sample_hemisphere(V3 n, Stream& rng)  // Material.cpp:48-65
{
    float r = std::sqrt(rng.next());
    float a = 2.0f * kPi * rng.next();
    float x = r * std::cos(a);
    float z = r * std::sin(a);
    float y = std::sqrt(std::max(0.0f, 1.0f - r * r));
    V3 up = std::fabs(n.x) > 0.9f ? V3{0, 1, 0} : V3{1, 0, 0};
    V3 tangent = normalized(cross(n, up));
    V3 bitangent = cross(n, tangent);
    return normalized(tangent * x + n * y + bitangent * z);
}

// Material::scatter, src/shading/Material.cpp:165-266.
bool scatter(const orc_scene& S, const wf_material& m, V3 in_dir, const Hit& h, Stream& rng,
             V3& att, V3& out_dir, float& pdf)
{
    V3 surf = surface_color(S, m, h);
    switch (m.type) {
    case WF_MATERIAL_DIFFUSE: {
        V3 d = cosine_sample_hemisphere(h.n, rng);
        out_dir = d;
        att = surf;
        float c = std::max(0.0f, dot(h.n, d));
        pdf = c / kPi;
        return true;
    }
    case WF_MATERIAL_METAL: {
        V3 r = reflect(in_dir, h.n);
        V3 fuzz = random_in_unit_sphere(rng) * m.roughness;
        out_dir = normalized(r + fuzz);
        att = surf;
        pdf = -1.0f;
        return dot(out_dir, h.n) > 0.0f;
    }
    case WF_MATERIAL_EMISSIVE:
    case WF_MATERIAL_SPOTLIGHT:
        att = surf * m.emission;
        pdf = -1.0f;
        return false;
    case WF_MATERIAL_GLASS: {
        att = surf;
        pdf = -1.0f;
        float eta = h.front ? (1.0f / m.ior) : m.ior;
        V3 id = normalized(in_dir);
        float c = std::min(1.0f, dot(id * -1.0f, h.n));
        float s = std::sqrt(1.0f - c * c);
        bool tir = eta * s > 1.0f;
        if (tir || schlick(c, eta) > rng.next())
            out_dir = reflect(id, h.n);
        else
            out_dir = refract(id, h.n, eta);
        return true;
    }
    case WF_MATERIAL_PLASTIC: {
        float c = std::max(0.0f, dot(in_dir * -1.0f, h.n));
        float refl = schlick(c, 1.5f);
        if (rng.next() < refl) {
            V3 r = reflect(normalized(in_dir), h.n);
            V3 fuzz = random_in_unit_sphere(rng) * m.roughness;
            out_dir = normalized(r + fuzz);
            att = {1.0f, 1.0f, 1.0f};
            pdf = -1.0f;
        } else {
            V3 d = cosine_sample_hemisphere(h.n, rng);
            out_dir = d;
            att = surf;
            float cc = std::max(0.0f, dot(h.n, d));
            pdf = cc / kPi;
        }
        return true;
    }
    default:
        pdf = -1.0f;
        return false;
    }
}

// MIS helpers, include/shading/MIS.h:6-32.
inline float area_to_angle(float area, float dist, float cosine)
{
    float sc = std::max(std::fabs(cosine), 1e-4f);
    return area * (dist * dist) / sc;
}
inline float mis_balance(float a, float b)
{
    float den = a + b;
    if (den <= 0.0f) return 0.0f;
    return a / den;
}
inline float light_area_pdf(const orc_scene& S)
{
    float total = S.total_emissive_area;
    if (total <= 0.0f) return 0.0f;
    return 1.0f / total;
}

struct LightSample {
    V3 p, n, e;
    float area = 0.0f;
    bool valid = false;
};

// Scene::sampleLight, src/core/Scene.cpp:192-238.
LightSample sample_light(const orc_scene& S, V3 shading_point, Stream& rng)
{
    LightSample ls;
    if (S.emissive_meshes.empty()) return ls;
    const int ne = (int)S.emissive_meshes.size();
    int mesh = S.emissive_meshes[(int)(rng.next() * (float)ne) % ne];
    int tri_count = S.mesh_cnt[mesh] / 3;
    float xi_tri = rng.next();
    if (tri_count <= 0) return ls;
    int local = (int)(xi_tri * (float)tri_count) % tri_count;
    int g = S.mesh_first_tri[mesh] + local;
    V3 v0, v1, v2;
    S.tri_verts(g, v0, v1, v2);
    float r1 = rng.next();
    float r2 = rng.next();
    if (r1 + r2 > 1.0f) {
        r1 = 1.0f - r1;
        r2 = 1.0f - r2;
    }
    float r3 = 1.0f - r1 - r2;
    ls.p = v0 * r3 + v1 * r1 + v2 * r2;
    ls.n = normalized(cross(v1 - v0, v2 - v0));
    V3 from_light = normalized(shading_point - ls.p);
    ls.e = emitted(S.mats[S.mesh_mat[mesh]], ls.n, from_light);
    ls.area = S.total_emissive_area;
    ls.valid = true;
    return ls;
}

// EnvironmentMap::sample's texel of a normalized direction
// (src/core/EnvironmentMap.cpp:34-42).
size_t env_texel(const orc_scene& S, V3 d)
{
    float u = 0.5f + std::atan2(d.z, d.x) / (2.0f * (float)M_PI);
    float v = 0.5f - std::asin(std::max(-1.0f, std::min(1.0f, d.y))) / (float)M_PI;
    int x = std::min(S.env_w - 1, std::max(0, (int)(u * S.env_w)));
    int y = std::min(S.env_h - 1, std::max(0, (int)(v * S.env_h)));
    return (size_t)y * S.env_w + x;
}

// WavefrontRenderer::getSkyColor (.cpp:879-888) and EnvironmentMap::sample
// (src/core/EnvironmentMap.cpp:30-49).
V3 sky_color(const orc_scene& S, V3 dir)
{
    if (S.env_w > 0) {
        size_t k = env_texel(S, normalized(dir)) * 3;
        V3 raw = {S.env_rgb[k], S.env_rgb[k + 1], S.env_rgb[k + 2]};
        return raw * S.env_scale * V3{S.env_tint[0], S.env_tint[1], S.env_tint[2]};
    }
    float b = 0.5f * (normalized(dir).y + 1.0f);
    V3 dark = {0.02f, 0.02f, 0.05f};
    V3 horizon = {0.05f, 0.04f, 0.03f};
    return horizon * (1.0f - b) + dark * b;
}

inline V3 vmin(V3 a, float c) { return {std::min(a.x, c), std::min(a.y, c), std::min(a.z, c)}; }

// --- environment NEE (an addition of the GPU path, restated here so the
// GPU's paths can be checked one by one; the reference has only the miss
// term).  Texel weights f = luminance(rgb * scale * tint) * cos(elevation of
// the texel row's centre); p_i = N f_i / sum f; Walker alias table by Vose's
// method with index-ordered stacks of p < 1 and p >= 1.

void build_env_sampler(orc_scene& S)
{
    const size_t W = (size_t)S.env_w, H = (size_t)S.env_h, N = W * H;
    std::vector<double> w(N);
    double total = 0.0;
    for (size_t y = 0; y < H; ++y) {
        const double row_cos = std::cos((0.5 - ((double)y + 0.5) / (double)H) * M_PI);
        for (size_t x = 0; x < W; ++x) {
            const float* t = &S.env_rgb[3 * (y * W + x)];
            double lum = 0.2126 * ((double)t[0] * S.env_scale * S.env_tint[0]) +
                         0.7152 * ((double)t[1] * S.env_scale * S.env_tint[1]) +
                         0.0722 * ((double)t[2] * S.env_scale * S.env_tint[2]);
            w[y * W + x] = std::max(0.0, lum) * row_cos;
            total += w[y * W + x];
        }
    }
    if (!(total > 0.0) || !std::isfinite(total)) return;
    S.env_prob.assign(N, 1.0f);
    S.env_pdf.resize(N);
    S.env_alias.resize(N);
    std::vector<int64_t> lo, hi;
    for (size_t i = 0; i < N; ++i) {
        w[i] = w[i] * (double)N / total;
        S.env_pdf[i] = (float)w[i];
        S.env_alias[i] = (int)i;
        if (w[i] < 1.0)
            lo.push_back((int64_t)i);
        else
            hi.push_back((int64_t)i);
    }
    while (!lo.empty() && !hi.empty()) {
        int64_t a = lo.back(), b = hi.back();
        lo.pop_back();
        hi.pop_back();
        S.env_prob[a] = (float)w[a];
        S.env_alias[a] = (int)b;
        w[b] = (w[b] + w[a]) - 1.0;
        if (w[b] < 1.0)
            lo.push_back(b);
        else
            hi.push_back(b);
    }
}

// Solid-angle density of env_sample at a normalized direction:
// p W H / (2 pi^2 cos(elevation)).
float env_pdf(const orc_scene& S, V3 d)
{
    float c = std::sqrt(std::max(0.0f, 1.0f - d.y * d.y));
    if (!(c > 0.0f)) return 0.0f;
    return S.env_pdf[env_texel(S, d)] / (2.0f * kPi * kPi * c);
}

V3 env_sample(const orc_scene& S, float x1, float x2, float x3, float x4)
{
    const int64_t n = (int64_t)S.env_w * S.env_h;
    int64_t i = std::min(n - 1, (int64_t)(x1 * (float)n));
    if (!(x2 < S.env_prob[i])) i = S.env_alias[i];
    int y = (int)(i / S.env_w), x = (int)(i - (int64_t)y * S.env_w);
    float u = ((float)x + x3) / (float)S.env_w;
    float v = ((float)y + x4) / (float)S.env_h;
    float phi = (u - 0.5f) * (2.0f * kPi);
    float el = (0.5f - v) * kPi;
    float ce = std::cos(el), se = std::sin(el);
    return {ce * std::cos(phi), se, ce * std::sin(phi)};
}

// Camera::getRay, include/core/Camera.h:35-40.
void camera_ray(const wf_camera& c, float u, float v, V3& o, V3& d)
{
    V3 org = {c.origin[0], c.origin[1], c.origin[2]};
    V3 tl = {c.top_left[0], c.top_left[1], c.top_left[2]};
    V3 hz = {c.horizontal[0], c.horizontal[1], c.horizontal[2]};
    V3 vt = {c.vertical[0], c.vertical[1], c.vertical[2]};
    V3 dir = tl + hz * u + vt * v - org;
    o = org;
    d = normalized(dir);
}

// One path of renderScene: the camera ray of (pixel, sample) and its bounce
// loop (WavefrontRenderer.cpp:141-268), shading as shadeAll's per-hit body
// (.cpp:602-797).  Contributions are added to acc in the reference's order.
void render_path(const orc_scene& S, const wf_render_params& P, int x, int y, int sample,
                 float acc[3], orc_counters& cnt)
{
    const int W = P.width, H = P.height;
    const uint32_t pixel = (uint32_t)(y * W + x);
    Stream cam(P.seed_lo, P.seed_hi, kPurposeCamera, 0, pixel, (uint32_t)sample);
    float u = ((float)x + cam.next()) / (float)(W - 1);
    float v = 1.0f - ((float)y + cam.next()) / (float)(H - 1);
    V3 o, d;
    camera_ray(P.camera, u, v, o, d);
    V3 T = {1.0f, 1.0f, 1.0f};
    float in_pdf = -1.0f;
    const float ff = P.firefly_threshold;
    auto add = [&](V3 c) {
        acc[0] = acc[0] + c.x;
        acc[1] = acc[1] + c.y;
        acc[2] = acc[2] + c.z;
    };
    for (int depth = 0; depth < P.max_depth; ++depth) {
        cnt.closest_rays++;
        Closest c = closest_bvh(S, o, d, 0.001f, 1e9f);
        if (c.tri < 0) {  // miss loop, .cpp:256-265
            cnt.misses++;
            V3 sky = T * sky_color(S, d);
            if (P.enable_env_nee && !S.env_prob.empty() && in_pdf > 0.0f)
                sky = sky * mis_balance(in_pdf, env_pdf(S, normalized(d)));
            add(sky);
            break;
        }
        cnt.shaded_hits++;
        Hit h;
        make_hit(S, o, d, c, h);
        const wf_material& m = S.mats[h.mat];
        // Emission with MIS (.cpp:629-658)
        V3 Le = emitted(m, h.n, d * -1.0f);
        if (Le.x > 0.0f || Le.y > 0.0f || Le.z > 0.0f) {
            float w = 1.0f;
            if (depth > 0 && in_pdf > 0.0f) {
                float cos_l = std::max(0.0f, dot(d * -1.0f, h.n));
                if (cos_l > 0.0f) {
                    float lp = area_to_angle(light_area_pdf(S), h.t, cos_l);
                    w = mis_balance(in_pdf, lp);
                }
            }
            Le = vmin(Le, ff);
            add(T * Le * w);
        }
        // Area-light NEE for Diffuse / Plastic (.cpp:660-710)
        if (m.type == WF_MATERIAL_DIFFUSE || m.type == WF_MATERIAL_PLASTIC) {
            Stream lrng(P.seed_lo, P.seed_hi, kPurposeLight, (uint32_t)depth, pixel, (uint32_t)sample);
            LightSample ls = sample_light(S, h.p, lrng);
            if (ls.valid) {
                V3 to = ls.p - h.p;
                float dist = length(to);
                V3 dir = to / dist;
                float cos_s = dot(h.n, dir);
                float cos_l = dot(dir * -1.0f, ls.n);
                if (cos_s > 0.0f && cos_l > 0.0f) {
                    cnt.shadow_rays++;
                    if (!occluded_bvh(S, h.p, dir, dist)) {
                        V3 surf = surface_color(S, m, h);
                        float g = (cos_s * cos_l) / (dist * dist);
                        V3 brdf = surf * (1.0f / kPi);
                        float lp = area_to_angle(light_area_pdf(S), dist, cos_l);
                        float bp = cos_s / kPi;
                        float w = mis_balance(lp, bp);
                        V3 direct = T * brdf * ls.e * g * ls.area * w;
                        add(vmin(direct, ff));
                    }
                }
            }
        }
        // Directional NEE for every type (.cpp:712-737)
        if (S.dir.intensity > 0.0f) {
            V3 to = V3{S.dir.direction[0], S.dir.direction[1], S.dir.direction[2]} * -1.0f;
            float cos_s = dot(h.n, to);
            if (cos_s > 0.0f) {
                cnt.shadow_rays++;
                if (!occluded_bvh(S, h.p, to, 1e6f)) {
                    V3 surf = surface_color(S, m, h);
                    V3 brdf = surf * (1.0f / kPi);
                    V3 col = {S.dir.color[0], S.dir.color[1], S.dir.color[2]};
                    V3 direct = T * brdf * col * S.dir.intensity * cos_s;
                    add(vmin(direct, ff));
                }
            }
        }
        // Environment NEE (GPU addition, see build_env_sampler), unclamped
        if (P.enable_env_nee && !S.env_prob.empty() && depth + 1 < P.max_depth &&
            (m.type == WF_MATERIAL_DIFFUSE || m.type == WF_MATERIAL_PLASTIC)) {
            Stream erng(P.seed_lo, P.seed_hi, kPurposeEnvironment, (uint32_t)depth, pixel, (uint32_t)sample);
            float x1 = erng.next(), x2 = erng.next(), x3 = erng.next(), x4 = erng.next();
            V3 wi = env_sample(S, x1, x2, x3, x4);
            float cos_s = dot(h.n, wi);
            float pe = env_pdf(S, wi);
            if (cos_s > 0.0f && pe > 0.0f) {
                cnt.shadow_rays++;
                if (!occluded_bvh(S, h.p, wi, 1e6f)) {
                    V3 surf = surface_color(S, m, h);
                    float kd = 1.0f;
                    if (m.type == WF_MATERIAL_PLASTIC) kd = 1.0f - schlick(std::max(0.0f, dot(d * -1.0f, h.n)), 1.5f);
                    float bp = cos_s / kPi;
                    add(T * surf * (kd / kPi) * sky_color(S, wi) * (cos_s / (pe + bp)));
                }
            }
        }
        // Scatter, Russian roulette, next ray (.cpp:739-796)
        Stream srng(P.seed_lo, P.seed_hi, kPurposeScatter, (uint32_t)depth, pixel, (uint32_t)sample);
        V3 att, nd;
        float pdf;
        if (!scatter(S, m, d, h, srng, att, nd, pdf)) break;
        V3 Tn = T * att;
        if (depth + 1 >= P.rr_min_depth) {
            float q = std::min(0.95f, std::max({Tn.x, Tn.y, Tn.z}));
            if (P.enable_cost_aware_rr) {
                float rc = P.rel_cost_material ? (float)P.rel_cost_material[h.mat] : 1.0f;
                q = std::clamp(q / rc, 0.05f, 0.95f);
            }
            Stream rr(P.seed_lo, P.seed_hi, kPurposeRoulette, (uint32_t)depth, pixel, (uint32_t)sample);
            if (rr.next() > q) break;
            Tn = Tn / q;
        }
        o = h.p;
        d = nd;
        T = Tn;
        in_pdf = pdf;
    }
}

// RayQueue::spreadBits10 / mortonEncode3 (include/scheduling/RayQueue.h:45-60):
// the standard bit-interleave masks.
inline uint32_t spread10(uint32_t v)
{
    v &= 0x3FFu;
    v = (v | (v << 16)) & 0x30000FFu;
    v = (v | (v << 8)) & 0x300F00Fu;
    v = (v | (v << 4)) & 0x30C30C3u;
    v = (v | (v << 2)) & 0x9249249u;
    return v;
}

// luminance, include/render/AdaptiveSampler.h:21-27.
inline float luminance(float r, float g, float b) { return 0.2126f * r + 0.7152f * g + 0.0722f * b; }

}  // namespace

// ===========================================================================
// C API
// ===========================================================================
extern "C" {

void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4])
{
    philox10(ctr, key, out);
}

orc_scene* orc_scene_create(const wf_scene_desc* D)
{
    orc_scene* S = new orc_scene();
    S->px.assign(D->positions_x, D->positions_x + D->num_vertices);
    S->py.assign(D->positions_y, D->positions_y + D->num_vertices);
    S->pz.assign(D->positions_z, D->positions_z + D->num_vertices);
    S->idx.assign(D->indices, D->indices + D->num_indices);
    S->mesh_off.assign(D->mesh_index_offsets, D->mesh_index_offsets + D->num_meshes);
    S->mesh_cnt.assign(D->mesh_index_counts, D->mesh_index_counts + D->num_meshes);
    S->mesh_mat.assign(D->mesh_material_ids, D->mesh_material_ids + D->num_meshes);
    if (D->corner_u && D->corner_v) {
        S->cu.assign(D->corner_u, D->corner_u + D->num_indices);
        S->cv.assign(D->corner_v, D->corner_v + D->num_indices);
    }
    if (D->mesh_has_uv) S->has_uv.assign(D->mesh_has_uv, D->mesh_has_uv + D->num_meshes);
    S->mats.assign(D->materials, D->materials + D->num_materials);
    for (int t = 0; t < D->num_textures; ++t) {
        const wf_texture& src = D->textures[t];
        Tex tx;
        tx.w = src.width;
        tx.h = src.height;
        size_t n = (size_t)src.width * src.height;
        tx.rgb.resize(3 * n);
        if (src.format == WF_TEXEL_RGB32F) {
            std::memcpy(tx.rgb.data(), src.data, 3 * n * sizeof(float));
        } else {
            const uint8_t* b = (const uint8_t*)src.data;
            for (size_t i = 0; i < n; ++i)
                for (int k = 0; k < 3; ++k) tx.rgb[3 * i + k] = srgb_to_linear((float)b[4 * i + k] / 255.0f);
        }
        S->texs.push_back(std::move(tx));
    }
    if (D->environment.width > 0 && D->environment.rgb) {
        S->env_w = D->environment.width;
        S->env_h = D->environment.height;
        S->env_rgb.assign(D->environment.rgb,
                          D->environment.rgb + 3 * (size_t)S->env_w * S->env_h);
        S->env_scale = D->environment.intensity_scale;
        for (int k = 0; k < 3; ++k) S->env_tint[k] = D->environment.tint[k];
        build_env_sampler(*S);
    }
    S->dir = D->directional;
    // Per-triangle mesh ids; meshes are contiguous in index order.
    const int nt = S->num_tris();
    S->tri_mesh.assign(nt, 0);
    S->mesh_first_tri.resize(D->num_meshes);
    for (int m = 0; m < D->num_meshes; ++m) {
        int first = S->mesh_off[m] / 3;
        S->mesh_first_tri[m] = first;
        for (int t = first; t < first + S->mesh_cnt[m] / 3; ++t) S->tri_mesh[t] = m;
    }
    // Scene::buildAccelerator: emissive meshes (Scene.cpp:82-90), area cache.
    for (int m = 0; m < D->num_meshes; ++m) {
        int ty = S->mats[S->mesh_mat[m]].type;
        if (ty == WF_MATERIAL_EMISSIVE || ty == WF_MATERIAL_SPOTLIGHT) S->emissive_meshes.push_back(m);
    }
    // Scene::totalEmissiveArea (Scene.cpp:162-190): float sum in mesh order.
    float total = 0.0f;
    for (int m : S->emissive_meshes) {
        for (int t = 0; t < S->mesh_cnt[m] / 3; ++t) {
            V3 a, b, c;
            S->tri_verts(S->mesh_first_tri[m] + t, a, b, c);
            total += length(cross(b - a, c - a)) * 0.5f;
        }
    }
    S->total_emissive_area = total;
    // Scene::computeBounds (Scene.cpp:59-77).
    for (int k = 0; k < 3; ++k) {
        S->bmin[k] = std::numeric_limits<float>::max();
        S->bmax[k] = std::numeric_limits<float>::lowest();
    }
    for (int i = 0; i < D->num_vertices; ++i) {
        float p[3] = {S->px[i], S->py[i], S->pz[i]};
        for (int k = 0; k < 3; ++k) {
            S->bmin[k] = std::min(S->bmin[k], p[k]);
            S->bmax[k] = std::max(S->bmax[k], p[k]);
        }
    }
    build_bvh(*S);
    return S;
}

void orc_scene_destroy(orc_scene* s) { delete s; }

void orc_scene_bounds(const orc_scene* s, float bmin[3], float bmax[3])
{
    for (int k = 0; k < 3; ++k) {
        bmin[k] = s->bmin[k];
        bmax[k] = s->bmax[k];
    }
}

float orc_scene_total_emissive_area(const orc_scene* s) { return s->total_emissive_area; }

// Camera::Camera, include/core/Camera.h:13-33, float arithmetic in the
// reference's order.  It carries the ABI's name because the procedural scene
// generator compiled into this library (wavefront-renderer_gb300/csrc/
// wf_scenes.cpp: the workload definition, shared so that the oracle and the
// GPU render identical scenes) calls it for a scene's default camera; the
// library is linked -Bsymbolic, so that call stays inside it.
int wf_camera_make(const float look_from[3], const float look_at[3], const float up[3], float vfov, int32_t w,
                   int32_t h, wf_camera* out)
{
    if (!look_from || !look_at || !up || !out || w <= 0 || h <= 0) return WF_ERR_INVALID_ARGUMENT;
    float aspect = static_cast<float>(w) / h;
    float theta = vfov * 3.14159265f / 180.0f;
    float view_h = 2.0f * std::tan(theta / 2.0f);
    float view_w = aspect * view_h;
    V3 from{look_from[0], look_from[1], look_from[2]};
    V3 at{look_at[0], look_at[1], look_at[2]};
    V3 upd{up[0], up[1], up[2]};
    V3 forward = normalized(from - at);
    V3 right = normalized(cross(upd, forward));
    V3 camera_up = cross(forward, right);
    V3 horizontal = right * view_w;
    V3 vertical = camera_up * view_h;
    V3 top_left = from - horizontal / 2.0f - vertical / 2.0f - forward;
    const V3 fields[4] = {from, top_left, horizontal, vertical};
    float* dst[4] = {out->origin, out->top_left, out->horizontal, out->vertical};
    for (int k = 0; k < 4; ++k) {
        dst[k][0] = fields[k].x;
        dst[k][1] = fields[k].y;
        dst[k][2] = fields[k].z;
    }
    return WF_OK;
}

void orc_camera_get_ray(const wf_camera* cam, float u, float v, float origin[3], float dir[3])
{
    V3 o, d;
    camera_ray(*cam, u, v, o, d);
    origin[0] = o.x;
    origin[1] = o.y;
    origin[2] = o.z;
    dir[0] = d.x;
    dir[1] = d.y;
    dir[2] = d.z;
}

void orc_generate_primary(const wf_camera* cam, int32_t W, int32_t H, uint32_t seed_lo,
                          uint32_t seed_hi, int32_t first_sample, int32_t nspp, float* ox,
                          float* oy, float* oz, float* dx, float* dy, float* dz, int32_t* pixel,
                          int32_t* sample)
{
    const int64_t np = (int64_t)W * H;
    for (int s = 0; s < nspp; ++s) {
        for (int y = 0; y < H; ++y) {
            for (int x = 0; x < W; ++x) {
                int64_t i = s * np + (int64_t)y * W + x;
                uint32_t p = (uint32_t)(y * W + x);
                Stream rng(seed_lo, seed_hi, kPurposeCamera, 0, p, (uint32_t)(first_sample + s));
                float u = ((float)x + rng.next()) / (float)(W - 1);
                float v = 1.0f - ((float)y + rng.next()) / (float)(H - 1);
                V3 o, d;
                camera_ray(*cam, u, v, o, d);
                ox[i] = o.x;
                oy[i] = o.y;
                oz[i] = o.z;
                dx[i] = d.x;
                dy[i] = d.y;
                dz[i] = d.z;
                if (pixel) pixel[i] = (int32_t)p;
                if (sample) sample[i] = first_sample + s;
            }
        }
    }
}

void orc_trace_closest(const orc_scene* S, int64_t n, const float* ox, const float* oy,
                       const float* oz, const float* dx, const float* dy, const float* dz,
                       float tmin, float tmax, wf_hit_columns* out)
{
    for (int64_t i = 0; i < n; ++i) {
        V3 o = {ox[i], oy[i], oz[i]}, d = {dx[i], dy[i], dz[i]};
        Closest c = closest_bvh(*S, o, d, tmin, tmax);
        if (c.tri < 0) {
            write_hit(out, i, nullptr);
            continue;
        }
        Hit h;
        make_hit(*S, o, d, c, h);
        write_hit(out, i, &h);
    }
}

void orc_trace_closest_brute(const orc_scene* S, int64_t n, const float* ox, const float* oy,
                             const float* oz, const float* dx, const float* dy, const float* dz,
                             float tmin, float tmax, wf_hit_columns* out)
{
    // Scene::hit without an accelerator (Scene.cpp:145-157) calling Mesh::hit
    // (src/geometry/Mesh.cpp:9-44) for every mesh in order.
    for (int64_t i = 0; i < n; ++i) {
        V3 o = {ox[i], oy[i], oz[i]}, d = {dx[i], dy[i], dz[i]};
        Closest best;
        float closest = tmax;
        for (int m = 0; m < (int)S->mesh_off.size(); ++m) {
            int first = S->mesh_first_tri[m];
            for (int t = first; t < first + S->mesh_cnt[m] / 3; ++t) {
                V3 a, b, c;
                S->tri_verts(t, a, b, c);
                float th, uh, vh;
                if (intersect_triangle(o, d, a, b, c, tmin, closest, th, uh, vh)) {
                    closest = th;
                    best.tri = t;
                    best.t = th;
                    best.bu = uh;
                    best.bv = vh;
                }
            }
        }
        if (best.tri < 0) {
            write_hit(out, i, nullptr);
            continue;
        }
        Hit h;
        make_hit(*S, o, d, best, h);
        // Mesh::hit keeps the raw barycentrics as (u, v) (Mesh.cpp:37-38) and
        // never sets textureID (stays -1).
        h.u = best.bu;
        h.v = best.bv;
        h.tex = -1;
        write_hit(out, i, &h);
    }
}

void orc_trace_occluded(const orc_scene* S, int64_t n, const float* ox, const float* oy,
                        const float* oz, const float* dx, const float* dy, const float* dz,
                        const float* max_distance, uint8_t* out)
{
    for (int64_t i = 0; i < n; ++i) {
        V3 o = {ox[i], oy[i], oz[i]}, d = {dx[i], dy[i], dz[i]};
        out[i] = occluded_bvh(*S, o, d, max_distance[i]) ? 1 : 0;
    }
}

void orc_ray_sort_keys(int64_t n, const float* ox, const float* oy, const float* oz,
                       const float* dx, const float* dy, const float* dz, const float bmin[3],
                       const float bmax[3], uint64_t* keys)
{
    // RayQueue::sortKey, include/scheduling/RayQueue.h:135-162.
    float ext[3];
    for (int k = 0; k < 3; ++k) ext[k] = std::max(bmax[k] - bmin[k], 1e-6f);
    auto q = [](float v, float mn, float ex) {
        float t = (v - mn) / ex;
        t = std::clamp(t, 0.0f, 1.0f);
        return (uint32_t)(t * (float)(1024u - 1));
    };
    for (int64_t i = 0; i < n; ++i) {
        uint64_t oct = (dx[i] < 0.0f ? 1u : 0u) | (dy[i] < 0.0f ? 2u : 0u) | (dz[i] < 0.0f ? 4u : 0u);
        uint32_t gx = q(ox[i], bmin[0], ext[0]);
        uint32_t gy = q(oy[i], bmin[1], ext[1]);
        uint32_t gz = q(oz[i], bmin[2], ext[2]);
        uint64_t m = spread10(gx) | (spread10(gy) << 1) | (spread10(gz) << 2);
        keys[i] = (oct << 30) | m;
    }
}

void orc_ray_schedule(int64_t n, const float* ox, const float* oy, const float* oz,
                      const float* dx, const float* dy, const float* dz, const float bmin[3],
                      const float bmax[3], int32_t* sorted)
{
    // RayQueue::schedule (RayQueue.h:165-179); tbb::parallel_sort taken as a
    // stable sort of the indices.
    std::vector<uint64_t> keys(n);
    orc_ray_sort_keys(n, ox, oy, oz, dx, dy, dz, bmin, bmax, keys.data());
    std::vector<int32_t> idx(n);
    std::iota(idx.begin(), idx.end(), 0);
    std::stable_sort(idx.begin(), idx.end(), [&](int a, int b) { return keys[a] < keys[b]; });
    std::copy(idx.begin(), idx.end(), sorted);
}

void orc_shading_schedule(int32_t policy, int64_t n, const int32_t* mat_ids,
                          const int32_t* tex_ids, const float* tr, const float* tg,
                          const float* tb, const float* px, const float* py, const float* pz,
                          int32_t num_materials, const wf_material* mats, int32_t num_textures,
                          const int64_t* tex_bytes, const double* rc_mat, const double* rc_tex,
                          int32_t* sorted)
{
    std::vector<int32_t> idx(n);
    std::iota(idx.begin(), idx.end(), 0);
    (void)num_materials;
    auto type_of = [&](int64_t i) { return mats[mat_ids[i]].type; };
    auto rel_mat = [&](int m) { return rc_mat ? rc_mat[m] : 1.0; };
    if (policy == WF_POLICY_NONE || n == 0) {  // ShadingQueue.h:96-99
        std::copy(idx.begin(), idx.end(), sorted);
        return;
    }
    if (policy == WF_POLICY_COST_BENEFIT_AWARE) {
        // scheduleCostBenefitAware, ShadingQueue.h:437-510.
        std::unordered_map<int, double> benefit;
        for (int64_t i = 0; i < n; ++i) benefit[mat_ids[i]] += luminance(tr[i], tg[i], tb[i]);
        std::unordered_map<int, double> priority;
        for (auto& kv : benefit) {
            int m = kv.first;
            double cost = rel_mat(m);
            int tid = mats[m].texture_id;
            double tcost = (rc_tex && tid >= 0) ? rc_tex[tid] : 0.0;
            priority[m] = kv.second / std::max(cost + tcost, 1e-6);
        }
        float mn[3] = {px[0], py[0], pz[0]}, mx[3] = {px[0], py[0], pz[0]};
        for (int64_t i = 0; i < n; ++i) {
            float p[3] = {px[i], py[i], pz[i]};
            for (int k = 0; k < 3; ++k) {
                mn[k] = std::min(mn[k], p[k]);
                mx[k] = std::max(mx[k], p[k]);
            }
        }
        // computeMortonCode, ShadingQueue.h:513-550.
        auto quant = [](float v, float lo, float hi) -> uint32_t {
            float t = (hi > lo) ? (v - lo) / (hi - lo) : 0.0f;
            return (uint32_t)(std::clamp(t, 0.0f, 1.0f) * 1023u);
        };
        std::vector<uint64_t> morton(n);
        for (int64_t i = 0; i < n; ++i) {
            uint64_t mx_ = spread10(quant(px[i], mn[0], mx[0]));
            uint64_t my_ = spread10(quant(py[i], mn[1], mx[1]));
            uint64_t mz_ = spread10(quant(pz[i], mn[2], mx[2]));
            morton[i] = mx_ | (my_ << 1) | (mz_ << 2);
        }
        std::stable_sort(idx.begin(), idx.end(), [&](int a, int b) {
            int ta = type_of(a), tb_ = type_of(b);
            if (ta != tb_) return ta < tb_;
            double pa = priority[mat_ids[a]], pb = priority[mat_ids[b]];
            if (pa != pb) return pa > pb;
            return morton[a] < morton[b];
        });
        std::copy(idx.begin(), idx.end(), sorted);
        return;
    }
    // computeTypeOrder (ShadingQueue.h:277-329).  The candidate list is the
    // iteration order of the reference's std::unordered_map<int,int> keyed by
    // type: with these few small keys every key has its own bucket and
    // libstdc++ links each new bucket at the front, so iteration visits the
    // types in reverse order of first appearance.  std::sort on fewer than 17
    // elements is an insertion sort, hence stable on that list.
    std::vector<int> first_seen;
    long long count_by_type[8] = {0};
    unsigned long long mem_by_type[8] = {0};
    for (int64_t i = 0; i < n; ++i) {
        int ty = type_of(i);
        if (count_by_type[ty]++ == 0) first_seen.push_back(ty);
        int tid = tex_ids[i];
        if (tid >= 0 && tid < num_textures) mem_by_type[ty] += (unsigned long long)tex_bytes[tid];
    }
    std::vector<int> order(first_seen.rbegin(), first_seen.rend());
    if (policy == WF_POLICY_MATERIAL_AWARE) {
        std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
            if (count_by_type[a] != count_by_type[b]) return count_by_type[a] > count_by_type[b];
            return a > b;
        });
    } else {
        std::stable_sort(order.begin(), order.end(),
                         [&](int a, int b) { return mem_by_type[a] > mem_by_type[b]; });
    }
    int rank[8];
    for (int k = 0; k < 8; ++k) rank[k] = 0;
    for (int r = 0; r < (int)order.size(); ++r) rank[order[r]] = r;
    auto tex_size = [&](int64_t i) -> unsigned long long {
        int tid = tex_ids[i];
        return (tid >= 0 && tid < num_textures) ? (unsigned long long)tex_bytes[tid] : 0ull;
    };
    // ShadingQueue.h:112-140 comparator; tbb::parallel_sort taken as stable.
    std::stable_sort(idx.begin(), idx.end(), [&](int a, int b) {
        int ra = rank[type_of(a)], rb = rank[type_of(b)];
        if (ra != rb) return ra < rb;
        if (policy == WF_POLICY_TEXTURE_AWARE) return tex_size(a) > tex_size(b);
        return rel_mat(mat_ids[a]) > rel_mat(mat_ids[b]);
    });
    std::copy(idx.begin(), idx.end(), sorted);
}

void orc_render_window(const orc_scene* S, const wf_render_params* P, int32_t x0, int32_t y0,
                       int32_t w, int32_t h, int32_t threads, float* accum, orc_counters* counters)
{
    orc_render_window_counts(S, P, x0, y0, w, h, threads, accum, nullptr, counters);
}

// renderScene's AdaptiveSampler per pixel (AdaptiveSampler.h:41-78 and
// WavefrontRenderer.cpp:270-294): a pixel's samples run in order; after each
// one luminance(sum after - sum before) feeds Welford's update, and after
// every 16th sample, from 32 on, the pixel stops once the standard error of
// its mean is below threshold * (mean + 0.01).  Pixels are independent (the
// reference's early exit only fires when every pixel has stopped), so the
// port runs the rule pixel by pixel.
void orc_render_window_counts(const orc_scene* S, const wf_render_params* P, int32_t x0, int32_t y0,
                              int32_t w, int32_t h, int32_t threads, float* accum, int32_t* counts,
                              orc_counters* counters)
{
    if (threads <= 0) threads = (int)std::max(1u, std::thread::hardware_concurrency());
    std::atomic<int> next_row{0};
    std::vector<orc_counters> per(threads);
    for (auto& c : per) c = orc_counters{0, 0, 0, 0};
    auto worker = [&](int tid) {
        orc_counters& cnt = per[tid];
        for (;;) {
            int r = next_row.fetch_add(1);
            if (r >= h) break;
            for (int c = 0; c < w; ++c) {
                float acc[3] = {0.0f, 0.0f, 0.0f};
                int n = 0;
                if (P->enable_adaptive_sampling) {
                    float mean = 0.0f, m2 = 0.0f;
                    for (int s = 0; s < P->samples_per_pixel; ++s) {
                        const float b0 = acc[0], b1 = acc[1], b2 = acc[2];
                        render_path(*S, *P, x0 + c, y0 + r, P->first_sample + s, acc, cnt);
                        const float lum = 0.2126f * (acc[0] - b0) + 0.7152f * (acc[1] - b1) + 0.0722f * (acc[2] - b2);
                        n += 1;
                        const float d1 = lum - mean;
                        mean += d1 / (float)n;
                        const float d2 = lum - mean;
                        m2 += d1 * d2;
                        if ((s + 1) % 16 == 0 && n >= 32) {
                            const float var = m2 / (float)(n - 1);
                            const float se = std::sqrt(var / (float)n);
                            if (se < P->adaptive_threshold * (mean + 0.01f)) break;
                        }
                    }
                } else {
                    for (int s = 0; s < P->samples_per_pixel; ++s)
                        render_path(*S, *P, x0 + c, y0 + r, P->first_sample + s, acc, cnt);
                    n = P->samples_per_pixel;
                }
                if (counts) counts[(size_t)r * w + c] = n;
                size_t k = 3 * ((size_t)r * w + c);
                accum[k + 0] = acc[0];
                accum[k + 1] = acc[1];
                accum[k + 2] = acc[2];
            }
        }
    };
    std::vector<std::thread> pool;
    for (int t = 1; t < threads; ++t) pool.emplace_back(worker, t);
    worker(0);
    for (auto& t : pool) t.join();
    if (counters) {
        *counters = orc_counters{0, 0, 0, 0};
        for (auto& c : per) {
            counters->closest_rays += c.closest_rays;
            counters->shadow_rays += c.shadow_rays;
            counters->shaded_hits += c.shaded_hits;
            counters->misses += c.misses;
        }
    }
}

void orc_cost_tracker_relative(int32_t items, int64_t n, const int32_t* ids, const double* ns,
                               double* out)
{
    // CostTracker::record / relativeCost, include/render/CostTracker.h:18-55.
    std::vector<double> avg(items, 0.0);
    std::vector<char> init(items, 0);
    std::vector<int> cnt(items, 0);
    double total = 0.0;
    int tracked = 0;
    for (int64_t i = 0; i < n; ++i) {
        int id = ids[i];
        cnt[id] += 1;
        if (!init[id]) {
            avg[id] = ns[i];
            init[id] = 1;
            tracked += 1;
            total += ns[i];
        } else {
            double old = avg[id];
            double nw = (1.0 - 0.05) * old + 0.05 * ns[i];
            avg[id] = nw;
            total += (nw - old);
        }
    }
    for (int id = 0; id < items; ++id) {
        if (cnt[id] < 50 || tracked == 0) {
            out[id] = 1.0;
            continue;
        }
        double g = total / tracked;
        out[id] = g <= 0.0 ? 1.0 : avg[id] / g;
    }
}

}  // extern "C"
