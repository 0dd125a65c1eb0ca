// wf_device.cuh — device-side data layout and shading arithmetic of the
// wavefront path tracer (sm_103a).
//
// Numerics: every translation unit is compiled with -fmad=false, so a*b+c is
// never fused and '/', sqrtf are IEEE round-to-nearest (prec-div/prec-sqrt
// stay on).  Camera rays, Moller-Trumbore hits, Morton keys and hit points
// are therefore bit-identical to the reference's float arithmetic.  Fused
// multiply-adds are used only where they cannot change a result (the
// conservative ray/box slab test), through explicit __fmaf_rn.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/wf_api.h"

namespace wf {

constexpr float kPi = 3.14159265f;  // reference WavefrontRenderer.h:22, Material.cpp:8
#ifndef WF_LEAF_MAX
#define WF_LEAF_MAX 4
#endif
constexpr int kLeafMax = WF_LEAF_MAX;  // triangles per BVH leaf (<= 8)
constexpr int kStackSize = 64;      // traversal stack entries (checked at build)
constexpr uint32_t kLeafFlag = 0x80000000u;

// ---------------------------------------------------------------------------
// Device scene
// ---------------------------------------------------------------------------

// BVH2 node holding both children's boxes (one 64-byte fetch per visited
// node).  Child encoding: >= 0 internal node index; with kLeafFlag set,
// bits 3..30 = first triangle (leaf order), bits 0..2 = count-1.  An empty
// child has an inverted box and never intersects.
struct __align__(16) BvhNode {
    float4 c0xy;  // c0.lo.x, c0.hi.x, c0.lo.y, c0.hi.y
    float4 c1xy;  // c1.lo.x, c1.hi.x, c1.lo.y, c1.hi.y
    float4 cz;    // c0.lo.z, c0.hi.z, c1.lo.z, c1.hi.z
    int4 kids;    // child0, child1, unused, unused
};

// Texture descriptor; texels live in one pool.
struct TexDesc {
    int32_t width, height, format;
    int32_t pad;
    int64_t offset;  // element offset: floats (RGB32F) or uint32 (RGBA8)
};

struct EmissiveMesh {
    int32_t first;    // first triangle in the emissive triangle array
    int32_t count;    // triangles
    int32_t material; // material id
    int32_t pad;
};

// 4-wide node: the four child boxes at full precision, one 128-byte line.
// Planes are stored per axis and side for the four children (lox.x = child
// 0's lower x plane, ...); kids holds the child words of BvhNode's encoding,
// kEmptyChild4 for an empty slot (whose box is never tested).  Interior
// children are numbered level by level, so a child's index is always larger
// than its parent's.
struct __align__(16) Bvh4Node {
    float4 lox, hix, loy, hiy, loz, hiz;
    int4 kids;
    int4 pad;
};
static_assert(sizeof(Bvh4Node) == 128, "Bvh4Node is one 128-byte line");
constexpr uint32_t kEmptyChild4 = 0xFFFFFFFFu;  // never a leaf word: scenes hold < 2^28 triangles
constexpr int kStack4 = 96;  // 4-wide traversal stack entries (checked at build: 1 + 3 x levels)

// Tree format of a resident scene; the kernels of one wave use one traversal.
enum TreeFormat : int { kTreeBinary = 0, kTreeFour = 2 };

struct DeviceScene {
    // Triangles in BVH leaf order: 3 float4 each.
    //   [0] = v0.xyz, w = global triangle index (bits)
    //   [1] = (v1 - v0).xyz, w = geomID (mesh index)
    //   [2] = (v2 - v0).xyz, w = primID (index within the mesh)
    const float4* tris;
    const BvhNode* nodes;      // binary tree, or null when nodes4 is set
    const Bvh4Node* nodes4;    // 4-wide tree, or null
    int32_t num_tris;
    int32_t num_nodes;
    int32_t root_is_empty;  // scene without triangles
    int32_t num_meshes;
    const int32_t* mesh_material;  // per mesh
    const uint8_t* mesh_has_uv;    // per mesh
    const float2* corner_uv;       // 3 per global triangle (only if any UV)
    int32_t has_any_uv;
    int32_t num_materials;
    const wf_material* materials;
    int32_t num_textures;
    const TexDesc* textures;
    const float* tex_f32;
    const uint32_t* tex_rgba8;
    const float* srgb_lut;  // 256 entries
    // Lights
    int32_t num_emissive_meshes;
    const EmissiveMesh* emissive_meshes;
    const float4* emissive_tris;  // 3 float4 each: exact v0, v1, v2
    float total_emissive_area;
    float light_area_pdf;          // 1/area or 0 (MIS.h:24-31)
    wf_directional_light directional;
    // Environment
    int32_t env_w, env_h;
    const float* env_rgb;
    float env_scale;
    float env_tint[3];
    // Environment importance sampling (device addition): an alias table over
    // the texels, weighted by luminance x cos(elevation), and each texel's
    // probability times the texel count.  Null without a map.
    const float* env_alias_prob;
    const int32_t* env_alias;
    const float* env_texel_pdf;
    // Bounds (Scene::computeBounds) for the ray sort
    float bmin[3], bmax[3];
};

__host__ __device__ __forceinline__ int tree_format(const DeviceScene& S)
{
    return S.nodes4 ? kTreeFour : kTreeBinary;
}

// ---------------------------------------------------------------------------
// Queues (device SoA).  Names follow the reference's columns
// (include/scheduling/RayQueue.h:65-90).  accumLight and alive are constant
// (0 and true) throughout the reference's loop and are not stored on the
// device; sampleIndices is a device addition keying the RNG.
// ---------------------------------------------------------------------------
struct RayQueueDev {
    float *ox, *oy, *oz, *dx, *dy, *dz;
    float *tr, *tg, *tb;
    float* pdf;
    int32_t *pixel, *depth, *sample;
    int32_t* job;  // device addition: the render job the path belongs to
    int64_t capacity;
};

// Compact hit queue: one entry per ray that hit (the ShadingQueue of the
// render loop).  The full HitRecord is rebuilt from the triangle on demand.
struct HitQueueDev {
    int32_t* ray;   // index into the ray queue
    int32_t* tri;   // leaf-order triangle position
    float* t;       // HitRecord::distance
    float* bu;      // barycentrics from Moller-Trumbore
    float* bv;
    int64_t capacity;
    // Shading order (a policy's permutation): k_shade reads entry order[k]
    // for its k-th hit; null = list order.
    const uint32_t* order = nullptr;
};

// Queue columns of the bounce loop are written once and read once per bounce,
// gigabytes per wave against a 126 MB L2: loads and stores with the
// evict-first (streaming) policy keep them from displacing the scene's tree
// and triangles, which every ray re-reads.
template <class T>
__device__ __forceinline__ T ldq(const T* p)
{
    return __ldcs(p);
}
template <class T>
__device__ __forceinline__ void stq(T* p, T v)
{
    __stcs(p, v);
}

// Shadow rays: origin, direction, max distance, the unoccluded contribution
// (already clamped) and the pixel it lands on.
struct ShadowQueueDev {
    float *ox, *oy, *oz, *dx, *dy, *dz, *dist;
    float *cr, *cg, *cb;
    int32_t* pixel;
    int32_t* job;
    int64_t capacity;
};

// A render job as the kernels see it: which resident scene, the shading
// parameters (WavefrontRenderer's public fields), its RNG key and where its
// per-pixel sums live.  Rays of many jobs share one wavefront; each ray finds
// its job, scene and accumulator through this table.
struct DeviceJob {
    int32_t scene;
    int32_t width, height;
    int32_t max_depth;
    int32_t rr_min_depth;
    int32_t cost_aware_rr;
    float firefly;
    uint32_t seed_lo, seed_hi;
    int32_t env_nee;                 // environment NEE + MIS on
    int64_t accum_offset;            // float index of the job's first pixel sum
    const float* rel_cost_material;  // float(relativeCost) per material, or null
    wf_camera camera;
    // Adaptive sampling: the wave's contributions land in per-sample sums
    // sample_buf[(sample - sample0) % wave_spp][pixel] (folded into the pixel
    // sums in sample order after the wave), and the camera draws only the
    // pixels of `active` (the chunk gives their count).  Null when off.
    float* sample_buf;
    const int32_t* active;
    int32_t sample0;
    int32_t wave_spp;
    // Live cost tracking: this bounce's timed cycles and counts per material
    // and per texture (null when off; single-job renders only).
    unsigned long long* cost_sum_mat;
    unsigned int* cost_cnt_mat;
    unsigned long long* cost_sum_tex;
    unsigned int* cost_cnt_tex;
};

// CostTracker state on the device (include/render/CostTracker.h:8-63).  Costs
// are SM clock cycles instead of nanoseconds: relativeCost is a ratio, so the
// unit cancels.
struct CostTrackerDev {
    unsigned long long* sum;  // per item: cycles recorded this bounce
    unsigned int* cnt;        // per item: timed calls this bounce
    double* avg;              // averageCostNanoseconds
    int32_t* samples;         // sampleCount
    int32_t* init;            // initialized
    double* total;            // cachedTotalCost (one value)
    int32_t* tracked;         // trackedItemCount (one value)
    double* rel;              // relativeCost per item
    float* rel_f;             // float(relativeCost) for RR, or null
    int32_t items;
};

// Where a path's contributions go: the job's pixel sums, or with adaptive
// sampling the per-sample slot of its pixel.
__device__ __forceinline__ float* job_accum(const DeviceJob& J, float* arena)
{
    return J.sample_buf ? J.sample_buf : arena + J.accum_offset;
}

__device__ __forceinline__ int32_t job_slot(const DeviceJob& J, int32_t pixel, int32_t sample)
{
    if (!J.sample_buf) return pixel;
    return ((sample - J.sample0) % J.wave_spp) * (J.width * J.height) + pixel;
}

// One slice of a wave: samples [first_sample, first_sample + nspp) of every
// pixel of a job, as paths [path_offset, path_offset + width*height*nspp),
// pixel-major (a pixel's nspp samples are consecutive paths).
struct WaveChunk {
    int32_t job;
    int32_t first_sample;
    int32_t nspp;
    int32_t active_count;  // > 0: paths cover job.active[0 .. active_count)
    int64_t path_offset;
};

// A streaming wave (path regeneration): the queue keeps a fixed capacity and,
// after every bounce, the paths that ended are replaced by new camera rays
// taken in order from an append-only list of chunks (absolute path offsets).
// The host appends chunks (total, nchunks); the device advances the cursor.
struct StreamState {
    int64_t cursor;        // paths generated so far
    int64_t total;         // paths appended to the chunk list
    int64_t refill_first;  // this bounce's refill: first path,
    int64_t refill_base;   //   queue position of its first ray,
    int64_t refill_count;  //   and number of rays
    int32_t nchunks;       // chunks in the device list (the first may be partly generated)
    int32_t pad;
};

// ---------------------------------------------------------------------------
// Small vector helpers (reference include/math/Vec3.h semantics).
// ---------------------------------------------------------------------------
struct V3 {
    float x, y, z;
};
__host__ __device__ __forceinline__ V3 v3(float x, float y, float z) { return V3{x, y, z}; }
__host__ __device__ __forceinline__ V3 operator+(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
__host__ __device__ __forceinline__ V3 operator-(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
__host__ __device__ __forceinline__ V3 operator*(V3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
__host__ __device__ __forceinline__ V3 operator/(V3 a, float s) { return {a.x / s, a.y / s, a.z / s}; }
__host__ __device__ __forceinline__ V3 operator*(V3 a, V3 b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
__host__ __device__ __forceinline__ float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__host__ __device__ __forceinline__ V3 cross(V3 a, V3 b)
{
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
__device__ __forceinline__ float length(V3 a) { return sqrtf(a.x * a.x + a.y * a.y + a.z * a.z); }
__device__ __forceinline__ V3 normalized(V3 a) { return a / length(a); }
__device__ __forceinline__ V3 vmin(V3 a, float c) { return {fminf(a.x, c), fminf(a.y, c), fminf(a.z, c)}; }

// ---------------------------------------------------------------------------
// Counter-based RNG: Philox4x32-10 (Salmon et al., SC'11).  A stream is keyed
// by the render seed and counted by (block, purpose<<16 | depth, pixel,
// sample), so a path's numbers do not depend on which thread, queue slot or
// wave handles it.  Floats carry 24 random bits in [0, 1).
// ---------------------------------------------------------------------------
enum : uint32_t {
    kPurposeCamera = 1,
    kPurposeLight = 2,
    kPurposeScatter = 3,
    kPurposeRoulette = 4,
    kPurposeEnvironment = 5,
    kPurposeCostSample = 6
};

__host__ __device__ __forceinline__ void philox10(uint32_t c[4], uint32_t k0, uint32_t k1)
{
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        if (r > 0) {
            k0 += 0x9E3779B9u;
            k1 += 0xBB67AE85u;
        }
#ifdef __CUDA_ARCH__
        uint32_t hi0 = __umulhi(0xD2511F53u, c[0]), lo0 = 0xD2511F53u * c[0];
        uint32_t hi1 = __umulhi(0xCD9E8D57u, c[2]), lo1 = 0xCD9E8D57u * c[2];
#else
        uint64_t p0 = (uint64_t)0xD2511F53u * c[0], p1 = (uint64_t)0xCD9E8D57u * c[2];
        uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
#endif
        uint32_t n0 = hi1 ^ c[1] ^ k0;
        uint32_t n2 = hi0 ^ c[3] ^ k1;
        c[0] = n0;
        c[1] = lo1;
        c[2] = n2;
        c[3] = lo0;
    }
}

struct Stream {
    uint32_t k0, k1;
    uint32_t block, tag, pixel, sample;
    uint32_t buf[4];
    int used;
    __device__ __forceinline__ Stream(uint32_t s0, uint32_t s1, uint32_t purpose, uint32_t depth,
                                      uint32_t px, uint32_t smp)
        : k0(s0), k1(s1), block(0), tag((purpose << 16) | (depth & 0xFFFFu)), pixel(px),
          sample(smp), used(4)
    {
    }
    __device__ __forceinline__ float next()
    {
        if (used == 4) {
            buf[0] = block;
            buf[1] = tag;
            buf[2] = pixel;
            buf[3] = sample;
            philox10(buf, k0, k1);
            ++block;
            used = 0;
        }
        uint32_t x = buf[used++];
        return (float)(x >> 8) * (1.0f / 16777216.0f);
    }
};

// ---------------------------------------------------------------------------
// Moller-Trumbore, reference include/geometry/Triangle.h:6-43, same operation
// order; e1 = v1 - v0 and e2 = v2 - v0 are precomputed with the same
// subtraction, so results are bit-identical.
// ---------------------------------------------------------------------------
__device__ __forceinline__ bool intersect_triangle(V3 o, V3 d, V3 v0, V3 e1, V3 e2, float tmin,
                                                   float tmax, float& t_out, float& u_out,
                                                   float& v_out)
{
    const float eps = 0.0000001f;
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

__device__ __forceinline__ float safe_inv(float d)
{
    if (fabsf(d) < 1e-20f) d = copysignf(1e-20f, d);
    return 1.0f / d;
}

// HitRecord rebuilt from a leaf-order triangle, as EmbreeAccelerator::
// intersect4 maps a hit (src/accelerator/Embree.cpp:224-252).
struct HitRec {
    V3 p, n;
    float t, u, v;
    int32_t geom, prim, global_tri, mat, tex;
    bool front;
};

__device__ __forceinline__ void rebuild_hit(const DeviceScene& S, V3 o, V3 d, int leafpos,
                                            float t, float bu, float bv, HitRec& h)
{
    float4 a = __ldg(S.tris + 3 * leafpos + 0);
    float4 b = __ldg(S.tris + 3 * leafpos + 1);
    float4 c = __ldg(S.tris + 3 * leafpos + 2);
    h.global_tri = __float_as_int(a.w);
    h.geom = __float_as_int(b.w);
    h.prim = __float_as_int(c.w);
    h.t = t;
    h.p = o + d * t;  // Ray::at
    h.mat = __ldg(S.mesh_material + h.geom);
    h.tex = S.materials[h.mat].texture_id;
    // Mesh::interpolateUV, src/geometry/Mesh.cpp:46-63
    if (S.has_any_uv && S.mesh_has_uv[h.geom]) {
        float2 c0 = S.corner_uv[3 * (int64_t)h.global_tri + 0];
        float2 c1 = S.corner_uv[3 * (int64_t)h.global_tri + 1];
        float2 c2 = S.corner_uv[3 * (int64_t)h.global_tri + 2];
        float w0 = 1.0f - bu - bv;
        h.u = w0 * c0.x + bu * c1.x + bv * c2.x;
        h.v = w0 * c0.y + bu * c1.y + bv * c2.y;
    } else {
        h.u = bu;
        h.v = bv;
    }
    V3 outward = normalized(cross(v3(b.x, b.y, b.z), v3(c.x, c.y, c.z)));
    h.front = dot(d, outward) < 0.0f;  // HitRecord::setFaceNormal
    h.n = h.front ? outward : outward * -1.0f;
}

// Texture::sample, include/shading/Texture.h:34-46.
__device__ __forceinline__ V3 texture_sample(const DeviceScene& S, int tid, float u, float v)
{
    const TexDesc td = S.textures[tid];
    u = u - floorf(u);
    v = v - floorf(v);
    int x = (int)(u * td.width);
    int y = (int)(v * td.height);
    x = max(0, min(x, td.width - 1));
    y = max(0, min(y, td.height - 1));
    int64_t k = (int64_t)y * td.width + x;
    if (td.format == WF_TEXEL_RGB32F) {
        const float* p = S.tex_f32 + td.offset + 3 * k;
        return {__ldg(p), __ldg(p + 1), __ldg(p + 2)};
    }
    uint32_t px = __ldg(S.tex_rgba8 + td.offset + k);
    return {__ldg(S.srgb_lut + (px & 0xFF)), __ldg(S.srgb_lut + ((px >> 8) & 0xFF)),
            __ldg(S.srgb_lut + ((px >> 16) & 0xFF))};
}

// Material::getSurfaceColor, src/shading/Material.cpp:143-163, with the
// spatial hash of include/math/SpatialHash.h:18-45.
__device__ __forceinline__ V3 surface_color(const DeviceScene& S, const wf_material& m, const HitRec& h)
{
    int tid = m.texture_id;
    bool valid = tid >= 0 && tid < S.num_textures;
    if (m.use_spatial_checker && valid) {
        int cx = (int)floorf(h.p.x / m.checker_cell_size);
        int cy = (int)floorf(h.p.y / m.checker_cell_size);
        int cz = (int)floorf(h.p.z / m.checker_cell_size);
        uint32_t hh = ((uint32_t)cx * 73856093u ^ (uint32_t)cy * 19349663u ^ (uint32_t)cz * 83492791u) *
                      2654435761u;
        float pu = ((hh >> 16) & 0xFFFFu) / 65535.0f;
        float pv = (hh & 0xFFFFu) / 65535.0f;
        return texture_sample(S, tid, pu, pv);
    }
    if (valid) return texture_sample(S, tid, h.u, h.v);
    return {m.albedo[0], m.albedo[1], m.albedo[2]};
}

// Material::emitted, src/shading/Material.cpp:268-296.
__device__ __forceinline__ V3 emitted(const wf_material& m, V3 light_normal, V3 dir_from_light)
{
    V3 alb = {m.albedo[0], m.albedo[1], m.albedo[2]};
    if (m.type == WF_MATERIAL_EMISSIVE) return alb * m.emission;
    if (m.type == WF_MATERIAL_SPOTLIGHT) {
        V3 radiance = alb * m.emission;
        float c = dot(light_normal, dir_from_light);
        float ang = acosf(fmaxf(-1.0f, fminf(1.0f, c))) * (180.0f / kPi);
        if (ang >= m.spot_outer_deg) return {0.0f, 0.0f, 0.0f};
        if (ang > m.spot_falloff_deg) {
            float t = (ang - m.spot_falloff_deg) / (m.spot_outer_deg - m.spot_falloff_deg);
            float f = 1.0f - t;
            f = f * f * (3.0f - 2.0f * f);
            radiance = radiance * f;
        }
        return radiance;
    }
    return {0.0f, 0.0f, 0.0f};
}

// randomInUnitSphere (Material.cpp:10-19), rejection loop bounded at 64
// tries (probability of reaching the bound ~1e-21); the origin after that.
__device__ __forceinline__ V3 random_in_unit_sphere(Stream& rng)
{
    for (int k = 0; k < 64; ++k) {
        V3 c;
        c.x = rng.next() * 2.0f - 1.0f;
        c.y = rng.next() * 2.0f - 1.0f;
        c.z = rng.next() * 2.0f - 1.0f;
        if (dot(c, c) < 1.0f) return c;
    }
    return {0.0f, 0.0f, 0.0f};
}

__device__ __forceinline__ V3 reflect(V3 in, V3 n) { return in - n * 2.0f * dot(in, n); }

__device__ __forceinline__ V3 refract(V3 in, V3 n, float eta)
{
    float c = fminf(1.0f, dot(in * -1.0f, n));
    V3 perp = (in + n * c) * eta;
    V3 par = n * -sqrtf(fabsf(1.0f - dot(perp, perp)));
    return perp + par;
}

__device__ __forceinline__ float schlick(float c, float eta)
{
    float r0 = (1.0f - eta) / (1.0f + eta);
    r0 = r0 * r0;
    return r0 + (1.0f - r0) * powf((1.0f - c), 5.0f);
}

__device__ __forceinline__ V3 cosine_sample_hemisphere(V3 n, Stream& rng)
{
    float r = sqrtf(rng.next());
    float a = 2.0f * kPi * rng.next();
    float x = r * cosf(a);
    float z = r * sinf(a);
    float y = sqrtf(fmaxf(0.0f, 1.0f - r * r));
    V3 up = fabsf(n.x) > 0.9f ? v3(0.0f, 1.0f, 0.0f) : v3(1.0f, 0.0f, 0.0f);
    V3 tangent = normalized(cross(n, up));
    V3 bitangent = cross(n, tangent);
    return normalized(tangent * x + n * y + bitangent * z);
}

// Material::scatter, src/shading/Material.cpp:165-266.  The diffuse and
// plastic cases share one cosine-lobe sampler and the metal and plastic
// cases one fuzzy-mirror sampler (one inlined copy of each in k_shade); the
// operations and the order of the random draws are the reference's.
__device__ __forceinline__ bool scatter(const wf_material& m, V3 surf, V3 in_dir, const HitRec& h, Stream& rng,
                                        V3& att, V3& out_dir, float& pdf)
{
    bool cosine_lobe = false;  // else the fuzzy mirror around `mirror`
    bool must_leave = false;   // metal: absorbed when the fuzzed ray points into the surface
    V3 mirror = {0.0f, 0.0f, 0.0f};
    switch (m.type) {
    case WF_MATERIAL_DIFFUSE:
        cosine_lobe = true;
        att = surf;
        break;
    case WF_MATERIAL_METAL:
        mirror = reflect(in_dir, h.n);
        must_leave = true;
        att = surf;
        break;
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
        float c = fminf(1.0f, dot(id * -1.0f, h.n));
        float s = sqrtf(1.0f - c * c);
        bool tir = eta * s > 1.0f;
        if (tir || schlick(c, eta) > rng.next())
            out_dir = reflect(id, h.n);
        else
            out_dir = refract(id, h.n, eta);
        return true;
    }
    case WF_MATERIAL_PLASTIC: {
        float c = fmaxf(0.0f, dot(in_dir * -1.0f, h.n));
        float refl = schlick(c, 1.5f);
        if (rng.next() < refl) {
            mirror = reflect(normalized(in_dir), h.n);
            att = v3(1.0f, 1.0f, 1.0f);
        } else {
            cosine_lobe = true;
            att = surf;
        }
        break;
    }
    default:
        pdf = -1.0f;
        return false;
    }
    if (cosine_lobe) {
        V3 d = cosine_sample_hemisphere(h.n, rng);
        out_dir = d;
        pdf = fmaxf(0.0f, dot(h.n, d)) / kPi;
        return true;
    }
    V3 fuzz = random_in_unit_sphere(rng) * m.roughness;
    out_dir = normalized(mirror + fuzz);
    pdf = -1.0f;
    return must_leave ? dot(out_dir, h.n) > 0.0f : true;
}

// MIS helpers, include/shading/MIS.h:6-32.
__device__ __forceinline__ float area_to_angle(float area, float dist, float cosine)
{
    float sc = fmaxf(fabsf(cosine), 1e-4f);
    return area * (dist * dist) / sc;
}
__device__ __forceinline__ float mis_balance(float a, float b)
{
    float den = a + b;
    if (den <= 0.0f) return 0.0f;
    return a / den;
}

// Texel of a normalized direction: EnvironmentMap::sample's mapping
// (src/core/EnvironmentMap.cpp:34-42), u = 0.5 + atan2(z,x)/2pi,
// v = 0.5 - asin(y)/pi, nearest texel.
__device__ __forceinline__ int64_t env_texel(const DeviceScene& S, V3 d)
{
    float u = 0.5f + atan2f(d.z, d.x) / (2.0f * 3.14159265358979323846f);
    float v = 0.5f - asinf(fmaxf(-1.0f, fminf(1.0f, d.y))) / 3.14159265358979323846f;
    int x = min(S.env_w - 1, max(0, (int)(u * S.env_w)));
    int y = min(S.env_h - 1, max(0, (int)(v * S.env_h)));
    return (int64_t)y * S.env_w + x;
}

// WavefrontRenderer::getSkyColor (.cpp:879-888) / EnvironmentMap::sample
// (src/core/EnvironmentMap.cpp:30-49).
__device__ __forceinline__ V3 sky_color(const DeviceScene& S, V3 dir)
{
    if (S.env_w > 0) {
        int64_t k = env_texel(S, normalized(dir)) * 3;
        V3 raw = {__ldg(S.env_rgb + k), __ldg(S.env_rgb + k + 1), __ldg(S.env_rgb + k + 2)};
        return raw * S.env_scale * v3(S.env_tint[0], S.env_tint[1], S.env_tint[2]);
    }
    float b = 0.5f * (normalized(dir).y + 1.0f);
    V3 dark = {0.02f, 0.02f, 0.05f};
    V3 horizon = {0.05f, 0.04f, 0.03f};
    return horizon * (1.0f - b) + dark * b;
}

// Solid-angle density of env_sample at a normalized direction: a texel's
// probability p spread uniformly over its (u, v) cell, whose solid angle is
// (2 pi / W)(pi / H) cos(elevation), gives p W H / (2 pi^2 cos(elevation)).
__device__ __forceinline__ float env_pdf(const DeviceScene& S, V3 d)
{
    const float c = sqrtf(fmaxf(0.0f, 1.0f - d.y * d.y));
    if (!(c > 0.0f)) return 0.0f;
    return __ldg(S.env_texel_pdf + env_texel(S, d)) / (2.0f * kPi * kPi * c);
}

// Draws a direction from the environment: texel i = floor(x1 N), kept when
// x2 < prob[i] else alias[i] (Walker's alias method), then a uniform point
// of the texel's (u, v) cell from x3, x4, mapped back through the inverse of
// env_texel's mapping.
__device__ __forceinline__ V3 env_sample(const DeviceScene& S, float x1, float x2, float x3, float x4)
{
    const int64_t n = (int64_t)S.env_w * S.env_h;
    int64_t i = min(n - 1, (int64_t)(x1 * (float)n));
    if (!(x2 < __ldg(S.env_alias_prob + i))) i = __ldg(S.env_alias + i);
    const int y = (int)(i / S.env_w);
    const int x = (int)(i - (int64_t)y * S.env_w);
    const float u = ((float)x + x3) / (float)S.env_w;
    const float v = ((float)y + x4) / (float)S.env_h;
    const float phi = (u - 0.5f) * (2.0f * kPi);
    const float el = (0.5f - v) * kPi;
    const float ce = cosf(el), se = sinf(el);
    return {ce * cosf(phi), se, ce * sinf(phi)};
}

// ---------------------------------------------------------------------------
// Warp-aggregated append: one atomic per warp, slots in lane order.
// ---------------------------------------------------------------------------
__device__ __forceinline__ int64_t warp_append(unsigned long long* counter, bool want)
{
    unsigned mask = __ballot_sync(__activemask(), want);
    if (!want) return -1;
    int lane = threadIdx.x & 31;
    int leader = __ffs(mask) - 1;
    unsigned long long base = 0;
    if (lane == leader) base = atomicAdd(counter, (unsigned long long)__popc(mask));
    base = __shfl_sync(mask, base, leader);
    return (int64_t)base + __popc(mask & ((1u << lane) - 1u));
}

}  // namespace wf
