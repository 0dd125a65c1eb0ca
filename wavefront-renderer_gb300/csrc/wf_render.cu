// wf_render.cu — camera, traversal, shading and scheduling kernels of the
// wavefront loop (reference src/render/WavefrontRenderer.cpp:401-877).
#include <cuda_runtime.h>

#include <type_traits>

#include "wf_kernels.h"
#include "wf_sort.h"
#include "wf_traverse.cuh"

namespace wf {

namespace {

// Loop over [0, n) in block-wide steps so every warp runs the same number of
// iterations (warp collectives stay converged).
#define WF_BLOCK_LOOP(base, n)                                                       \
    for (int64_t base = (int64_t)blockIdx.x * blockDim.x; base < (n);                \
         base += (int64_t)gridDim.x * blockDim.x)

// ---------------------------------------------------------------------------
// Camera rays: WavefrontRenderer::generatePrimaryRays (.cpp:401-457) with
// Camera::getRay (include/core/Camera.h:35-40) and RayQueue::addPrimary
// (RayQueue.h:113-116: throughput 1, depth 0, pdf -1).
// ---------------------------------------------------------------------------
__global__ void k_camera(wf_camera cam, int W, int H, uint32_t s0, uint32_t s1, int first_sample,
                         int nspp, RayQueueDev rq)
{
    const int64_t np = (int64_t)W * H;
    const int64_t n = np * nspp;
    const V3 org = {cam.origin[0], cam.origin[1], cam.origin[2]};
    const V3 tl = {cam.top_left[0], cam.top_left[1], cam.top_left[2]};
    const V3 hz = {cam.horizontal[0], cam.horizontal[1], cam.horizontal[2]};
    const V3 vt = {cam.vertical[0], cam.vertical[1], cam.vertical[2]};
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const int s = (int)(i / np);
        const int p = (int)(i - (int64_t)s * np);
        const int x = p % W, y = p / W;
        const int sample = first_sample + s;
        Stream rng(s0, s1, kPurposeCamera, 0, (uint32_t)p, (uint32_t)sample);
        float u = ((float)x + rng.next()) / (float)(W - 1);
        float v = 1.0f - ((float)y + rng.next()) / (float)(H - 1);
        V3 d = normalized(tl + hz * u + vt * v - org);
        rq.ox[i] = org.x;
        rq.oy[i] = org.y;
        rq.oz[i] = org.z;
        rq.dx[i] = d.x;
        rq.dy[i] = d.y;
        rq.dz[i] = d.z;
        rq.tr[i] = 1.0f;
        rq.tg[i] = 1.0f;
        rq.tb[i] = 1.0f;
        rq.pdf[i] = -1.0f;
        rq.pixel[i] = p;
        rq.depth[i] = 0;
        rq.sample[i] = sample;
        if (rq.job) rq.job[i] = 0;
    }
}

// Camera rays of one wave made of chunks (job, samples) of several jobs: the
// same arithmetic as k_camera, the job's camera and seed.
// Queue order of a chunk: pixel-major — a pixel's samples are consecutive
// paths, so a warp traces the samples of one pixel (or of 32 / nspp pixels)
// and, as its paths bounce, starts them from nearly the same point; the
// ray-ordered queues keep that grouping through later bounces.  Against
// sample-major order (all pixels of sample 0, then sample 1, ...): lattice
// scene +19.7%, dense mesh +2.3%, 4-sample groups half of that.  Pixels
// follow bands of 4 rows, each walked in 8x4 tiles (a narrower last tile
// where the width is not a multiple of 8; the last band may hold fewer rows).
// A bijection on the chunk's paths; the pixel and sample key the random
// streams, so the order changes no path.
__device__ __forceinline__ int tile_pixel(int q, int W, int H)
{
    const int band = q / (4 * W);
    const int r = q - band * 4 * W;
    const int hb = min(4, H - 4 * band);
    const int full = (W / 8) * 8 * hb;
    int x, y;
    if (r < full) {
        const int c = r / (8 * hb), w = r - c * 8 * hb;
        x = c * 8 + (w & 7);
        y = 4 * band + (w >> 3);
    } else {
        const int wl = W - (W / 8) * 8, w = r - full;
        x = (W / 8) * 8 + w % wl;
        y = 4 * band + w / wl;
    }
    return y * W + x;
}

// The camera ray of path g of a chunk list (chunks ordered by path_offset,
// g >= chunks[0].path_offset), written at queue position q.
__device__ __forceinline__ void camera_path(const WaveChunk* __restrict__ chunks, int nchunks,
                                            const DeviceJob* __restrict__ jobs, int64_t g, int64_t q,
                                            const RayQueueDev& rq)
{
    int lo = 0, hi = nchunks - 1;  // last chunk with path_offset <= g
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (chunks[mid].path_offset <= g) lo = mid; else hi = mid - 1;
    }
    const WaveChunk ch = chunks[lo];
    const DeviceJob& J = jobs[ch.job];
    const int64_t local = g - ch.path_offset;
    const int64_t pi = local / ch.nspp;
    const int s = (int)(local - pi * ch.nspp);
    int p = (int)pi;
    if (ch.active_count > 0)
        p = J.active[p];  // generatePrimaryRays' activePixels mask
    else
        p = tile_pixel(p, J.width, J.height);
    const int x = p % J.width, y = p / J.width;
    const int sample = ch.first_sample + s;
    const wf_camera& cam = J.camera;
    const V3 org = {cam.origin[0], cam.origin[1], cam.origin[2]};
    const V3 tl = {cam.top_left[0], cam.top_left[1], cam.top_left[2]};
    const V3 hz = {cam.horizontal[0], cam.horizontal[1], cam.horizontal[2]};
    const V3 vt = {cam.vertical[0], cam.vertical[1], cam.vertical[2]};
    Stream rng(J.seed_lo, J.seed_hi, kPurposeCamera, 0, (uint32_t)p, (uint32_t)sample);
    float u = ((float)x + rng.next()) / (float)(J.width - 1);
    float v = 1.0f - ((float)y + rng.next()) / (float)(J.height - 1);
    V3 d = normalized(tl + hz * u + vt * v - org);
    stq(&rq.ox[q], org.x);
    stq(&rq.oy[q], org.y);
    stq(&rq.oz[q], org.z);
    stq(&rq.dx[q], d.x);
    stq(&rq.dy[q], d.y);
    stq(&rq.dz[q], d.z);
    stq(&rq.tr[q], 1.0f);
    stq(&rq.tg[q], 1.0f);
    stq(&rq.tb[q], 1.0f);
    stq(&rq.pdf[q], -1.0f);
    stq(&rq.pixel[q], p);
    stq(&rq.depth[q], 0);
    stq(&rq.sample[q], sample);
    stq(&rq.job[q], ch.job);
}

__global__ void k_camera_chunks(const WaveChunk* __restrict__ chunks, const long long* __restrict__ header,
                                const DeviceJob* __restrict__ jobs, RayQueueDev rq)
{
    const int64_t total = header[0];
    const int nchunks = (int)header[1];
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total;
         i += (int64_t)gridDim.x * blockDim.x)
        camera_path(chunks, nchunks, jobs, i, i, rq);
}

// Streaming waves (path regeneration): one thread plans the refill of the
// next queue after a bounce's shading.  Every live path advances one bounce
// per iteration, so paths generated here are finished (depth limit) after
// max_depth more iterations; the cursor log lets the host tell when.
__global__ void k_stream_plan(ull* __restrict__ counters, StreamState* __restrict__ st, int64_t capacity,
                              int64_t* __restrict__ log, int iter)
{
    const int64_t live = (int64_t)counters[3];
    int64_t k = capacity - live;
    const int64_t left = st->total - st->cursor;
    if (k > left) k = left;
    if (k < 0) k = 0;
    st->refill_first = st->cursor;
    st->refill_base = live;
    st->refill_count = k;
    st->cursor += k;
    counters[3] = (ull)(live + k);
    log[iter] = st->cursor;
}

__global__ void k_camera_refill(const WaveChunk* __restrict__ chunks, const StreamState* __restrict__ st,
                                const DeviceJob* __restrict__ jobs, RayQueueDev rq)
{
    const int64_t n = st->refill_count, first = st->refill_first, base = st->refill_base;
    const int nchunks = st->nchunks;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        camera_path(chunks, nchunks, jobs, first + i, base + i, rq);
}

__global__ void k_add_floats(float* __restrict__ dst, const float* __restrict__ src, int64_t n)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        dst[i] += src[i];
}

// End of a bounce in a device-counted chain (no host round trip, or a
// captured graph): the per-bounce counters accumulated on the device
// (tally[0] += rays, [1] += hits, [2] += shadow rays, [3] += bounces that
// had rays), the next bounce's ray count (counters[0] = counters[3]) and its
// zeroed counters [1..5], in one launch instead of a kernel, a copy and a
// memset (Cornell box +3.3%).
__global__ void k_bounce_end(ull* __restrict__ counters, ull* tally)
{
    tally[0] += counters[0];
    tally[1] += counters[1];
    tally[2] += counters[2];
    tally[3] += counters[0] ? 1ull : 0ull;
    counters[0] = counters[3];
    for (int k = 1; k <= 5; ++k) counters[k] = 0ull;
}

// ---------------------------------------------------------------------------
// Host-API traversal: one HitRecord per ray.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(128) k_trace_api(DeviceScene S, int64_t n, const float* ox,
                                                   const float* oy, const float* oz,
                                                   const float* dx, const float* dy,
                                                   const float* dz, float tmin, float tmax,
                                                   HitColumnsDev out, int* err)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        V3 o = {ox[i], oy[i], oz[i]}, d = {dx[i], dy[i], dz[i]};
        TraceResult r;
        traverse<false>(S, o, d, tmin, tmax, r, err);
        if (r.leafpos < 0) {  // a miss: ids -1, every other column 0
            if (out.geom) out.geom[i] = -1;
            if (out.prim) out.prim[i] = -1;
            if (out.mat) out.mat[i] = -1;
            if (out.tex) out.tex[i] = -1;
            float* zf[] = {out.t, out.bu, out.bv, out.px, out.py, out.pz, out.nx, out.ny, out.nz, out.u, out.v};
            for (float* z : zf)
                if (z) z[i] = 0.0f;
            if (out.front) out.front[i] = 0;
            continue;
        }
        HitRec h;
        rebuild_hit(S, o, d, r.leafpos, r.t, r.bu, r.bv, h);
        if (out.geom) out.geom[i] = h.geom;
        if (out.prim) out.prim[i] = h.prim;
        if (out.t) out.t[i] = h.t;
        if (out.bu) out.bu[i] = r.bu;
        if (out.bv) out.bv[i] = r.bv;
        if (out.px) out.px[i] = h.p.x;
        if (out.py) out.py[i] = h.p.y;
        if (out.pz) out.pz[i] = h.p.z;
        if (out.nx) out.nx[i] = h.n.x;
        if (out.ny) out.ny[i] = h.n.y;
        if (out.nz) out.nz[i] = h.n.z;
        if (out.front) out.front[i] = h.front ? 1 : 0;
        if (out.u) out.u[i] = h.u;
        if (out.v) out.v[i] = h.v;
        if (out.mat) out.mat[i] = h.mat;
        if (out.tex) out.tex[i] = h.tex;
    }
}

__global__ void __launch_bounds__(128) k_occluded_api(DeviceScene S, int64_t n, const float* ox,
                                                      const float* oy, const float* oz,
                                                      const float* dx, const float* dy,
                                                      const float* dz, const float* maxd,
                                                      uint8_t* out, int* err)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        V3 o = {ox[i], oy[i], oz[i]}, d = {dx[i], dy[i], dz[i]};
        TraceResult r;
        traverse<true>(S, o, d, 0.001f, maxd[i] - 0.001f, r, err);
        out[i] = r.leafpos >= 0 ? 1 : 0;
    }
}

// Child order of the binary any-hit traversal: the farther child first
// measured faster on dense scenes (dense mesh +1.4%, lattice with environment
// NEE +0.8%) and slower on the Cornell-box scenes of 36 triangles, whose
// occluders are the two boxes standing on the surfaces that cast the shadow
// rays (Cornell box -1.1%, batched Cornell variants -2.8%); single-job
// renders of scenes from kFarFirstTriangles on use it (a kernel instance of
// its own: as a launch argument the choice cost the dense mesh 0.7%), and so
// do multi-job waves over a dense scene (served stream with dense-mesh jobs
// among Cornell-box ones: +1.7% device rate).
constexpr int kFarFirstTriangles = 4096;
using TraversalFar = Traversal<true, true>;
using Traversal4Far = Traversal4<true, true>;

__device__ __forceinline__ void accum_add(float* accum, int32_t slot, V3 c)
{
    float* p = accum + 3 * (int64_t)slot;
    atomicAdd(p + 0, c.x);
    atomicAdd(p + 1, c.y);
    atomicAdd(p + 2, c.z);
}

// ---------------------------------------------------------------------------
// Render-loop closest hit (intersectAll, .cpp:459-567) fused with the miss
// loop (.cpp:256-265): misses add throughput * sky to their pixel, hits are
// appended to the hit queue with one atomic per warp.
//
// Dynamic fetch refills a warp's idle lanes only once at least half of them
// are idle (or all are): the refilled lanes then take one run of consecutive
// queue entries — neighbouring paths of the ray-ordered queue, which traverse
// alike — instead of a lane or two at a time from wherever the global counter
// has moved.  Against refilling every idle lane every round: lattice scene
// +4.9%, dense mesh +0.1%, batched jobs +0.7%; 20 and more idle lanes starve
// the dense mesh (-0.9% at 20, -24% at 32).
#ifndef WF_REFILL_MIN
#define WF_REFILL_MIN 16
#endif

// Persistent threads with dynamic ray fetch (Aila & Laine 2009): between
// traversal rounds, lanes whose ray has finished emit its result and take a
// new ray from a global counter, so a warp is not held by its slowest ray.
// ---------------------------------------------------------------------------
// kMulti = false: every ray belongs to job0 on scene0 (passed by value, read
// from the constant bank); true: each ray looks its job and scene up.
template <bool kMulti, int kMinBlocks, class Tr>
__global__ void __launch_bounds__(128, kMinBlocks) k_trace_render(DeviceScene scene0, DeviceJob job0,
                                                                  const DeviceScene* __restrict__ scenes,
                                                                  const DeviceJob* __restrict__ jobs,
                                                                  RayQueueDev rq, const ull* __restrict__ d_n,
                                                                  HitQueueDev hq, ull* hq_n, float* accum,
                                                                  ull* work, int* err, int ray_order)
{
    const int64_t n = (int64_t)*d_n;
    const int lane = threadIdx.x & 31;
    const unsigned lt = (1u << lane) - 1u;
    Tr tr;
    typename Tr::Entry stack[Tr::kStack];
    const DeviceScene* S = kMulti ? scenes : &scene0;
    int job = 0;
    int64_t ray = -1;
    bool exhausted = false;
    bool overflow = false;
    tr.idle();
    for (;;) {
        // 1. lanes whose traversal ended emit their result
        const bool fin = ray >= 0 && tr.done();
        const bool hit = fin && tr.res.leafpos >= 0;
        const unsigned hm = __ballot_sync(0xFFFFFFFFu, hit);
        if (ray_order) {
            // hit record at the ray's own index, tri = -1 for a miss (the
            // hits are counted and listed by k_compact_hits)
            if (fin) {
                stq(&hq.tri[ray], hit ? tr.res.leafpos : -1);
                if (hit) {
                    stq(&hq.t[ray], tr.res.t);
                    stq(&hq.bu[ray], tr.res.bu);
                    stq(&hq.bv[ray], tr.res.bv);
                }
            }
        } else if (hm) {
            ull base = 0;
            const int leader = __ffs(hm) - 1;
            if (lane == leader) base = atomicAdd(hq_n, (ull)__popc(hm));
            base = __shfl_sync(0xFFFFFFFFu, base, leader);
            if (hit) {
                const int64_t pos = (int64_t)base + __popc(hm & lt);
                if (pos < hq.capacity) {
                    stq(&hq.ray[pos], (int32_t)ray);
                    stq(&hq.tri[pos], tr.res.leafpos);
                    stq(&hq.t[pos], tr.res.t);
                    stq(&hq.bu[pos], tr.res.bu);
                    stq(&hq.bv[pos], tr.res.bv);
                } else {
                    atomicOr(err, 2);
                }
            }
        }
        if (fin && !hit && ray_order != 2) {  // (2: k_compact_hits shades the misses)
            const DeviceJob& J = kMulti ? jobs[job] : job0;
            const V3 T = {ldq(&rq.tr[ray]), ldq(&rq.tg[ray]), ldq(&rq.tb[ray])};
            V3 c = T * sky_color(*S, tr.d);
            // With environment NEE the bounce that sampled this direction by
            // its BSDF (pdf > 0) shares the estimate: balance-heuristic weight.
            if (J.env_nee && S->env_alias_prob) {
                const float ip = ldq(&rq.pdf[ray]);
                if (ip > 0.0f) c = c * mis_balance(ip, env_pdf(*S, normalized(tr.d)));
            }
            const int32_t slot = job_slot(J, ldq(&rq.pixel[ray]), J.sample_buf ? ldq(&rq.sample[ray]) : 0);
            accum_add(job_accum(J, accum), slot, c);
        }
        if (fin) {
            overflow = overflow || tr.overflow;
            ray = -1;
        }
        // 2. lanes without a ray take new ones
        const bool need = ray < 0 && !exhausted;
        const unsigned nm = __ballot_sync(0xFFFFFFFFu, need);
        if (nm && (__popc(nm) >= WF_REFILL_MIN || __all_sync(0xFFFFFFFFu, ray < 0))) {
            ull base = 0;
            const int leader = __ffs(nm) - 1;
            if (lane == leader) base = atomicAdd(work, (ull)__popc(nm));
            base = __shfl_sync(0xFFFFFFFFu, base, leader);
            if (need) {
                const int64_t idx = (int64_t)base + __popc(nm & lt);
                if (idx < n) {
                    ray = idx;
                    if (kMulti) {
                        job = ldq(&rq.job[idx]);
                        S = scenes + jobs[job].scene;
                    }
                    tr.init(*S, stack, v3(ldq(&rq.ox[idx]), ldq(&rq.oy[idx]), ldq(&rq.oz[idx])),
                            v3(ldq(&rq.dx[idx]), ldq(&rq.dy[idx]), ldq(&rq.dz[idx])), 0.001f, 1e9f);
                } else {
                    exhausted = true;
                }
            }
        }
        if (__all_sync(0xFFFFFFFFu, ray < 0)) break;
        // 3. one traversal round
        if (ray >= 0 && !tr.done()) {
            tr.round(*S, stack);
        }
    }
    if (overflow) atomicOr(err, 1);
}

// A ray that left the scene (the miss loop of renderScene, .cpp:256-265):
// throughput x sky (or environment map) added to its pixel, with the
// balance-heuristic weight against environment NEE when the job samples it.
template <bool kMulti>
__device__ __forceinline__ void shade_miss(const DeviceScene& scene0, const DeviceJob& job0,
                                           const DeviceScene* __restrict__ scenes,
                                           const DeviceJob* __restrict__ jobs, const RayQueueDev& rq, int64_t ray,
                                           float* accum)
{
    const int job = kMulti ? ldq(&rq.job[ray]) : 0;
    const DeviceJob& J = kMulti ? jobs[job] : job0;
    const DeviceScene& S = kMulti ? scenes[J.scene] : scene0;
    const V3 d = {ldq(&rq.dx[ray]), ldq(&rq.dy[ray]), ldq(&rq.dz[ray])};
    const V3 T = {ldq(&rq.tr[ray]), ldq(&rq.tg[ray]), ldq(&rq.tb[ray])};
    V3 c = T * sky_color(S, d);
    if (J.env_nee && S.env_alias_prob) {
        const float ip = ldq(&rq.pdf[ray]);
        if (ip > 0.0f) c = c * mis_balance(ip, env_pdf(S, normalized(d)));
    }
    const int32_t slot = job_slot(J, ldq(&rq.pixel[ray]), J.sample_buf ? ldq(&rq.sample[ray]) : 0);
    accum_add(job_accum(J, accum), slot, c);
}

// The rays that hit, listed in queue order for shading after a ray-order
// trace (records at the rays' indices, tri = -1 for a miss).  A block takes
// tiles of kCompactIters x 256 rays, ranks the hits of a tile in ray order
// (ballots, then one warp scans the 64 warp counts) and reserves the tile's
// run of the list with one atomic, so the list is sorted within a tile and
// the tiles follow the blocks' sweep.  Shading in this order keeps the next
// rays and the shadow rays in queue order too.
constexpr int kCompactIters = 8;  // 8 x 8 warps = 64 counts: two per lane of the scanning warp

template <bool kMulti, bool kMisses>
__global__ void __launch_bounds__(256) k_compact_hits(DeviceScene scene0, DeviceJob job0,
                                                      const DeviceScene* __restrict__ scenes,
                                                      const DeviceJob* __restrict__ jobs, RayQueueDev rq,
                                                      const ull* __restrict__ d_n, HitQueueDev hq, ull* hq_n,
                                                      float* accum)
{
    __shared__ unsigned offs[kCompactIters * 8];
    __shared__ ull tile_first;
    const int64_t n = (int64_t)*d_n;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const unsigned lt = (1u << lane) - 1u;
    const int64_t tile = 256 * kCompactIters;
    for (int64_t t0 = (int64_t)blockIdx.x * tile; t0 < n; t0 += (int64_t)gridDim.x * tile) {
        unsigned masks[kCompactIters];
#pragma unroll
        for (int j = 0; j < kCompactIters; ++j) {
            const int64_t k = t0 + j * 256 + threadIdx.x;
            const int32_t tri = k < n ? ldq(&hq.tri[k]) : 0;
            masks[j] = __ballot_sync(0xFFFFFFFFu, k < n && tri >= 0);
            if (lane == 0) offs[j * 8 + warp] = (unsigned)__popc(masks[j]);
            if (kMisses && tri < 0) shade_miss<kMulti>(scene0, job0, scenes, jobs, rq, k, accum);
        }
        __syncthreads();
        if (warp == 0) {  // exclusive scan of the counts in ray order (j, then warp)
            const unsigned a = offs[2 * lane], b = offs[2 * lane + 1];
            unsigned incl = a + b;
#pragma unroll
            for (int d = 1; d < 32; d <<= 1) {
                const unsigned y = __shfl_up_sync(0xFFFFFFFFu, incl, d);
                if (lane >= d) incl += y;
            }
            const unsigned excl = incl - (a + b);
            offs[2 * lane] = excl;
            offs[2 * lane + 1] = excl + a;
            const unsigned total = __shfl_sync(0xFFFFFFFFu, incl, 31);
            if (lane == 0) tile_first = total ? atomicAdd(hq_n, (ull)total) : 0ull;
        }
        __syncthreads();
#pragma unroll
        for (int j = 0; j < kCompactIters; ++j) {
            if ((masks[j] >> lane) & 1u) {
                const int64_t k = t0 + j * 256 + threadIdx.x;
                stq(&hq.ray[(int64_t)tile_first + offs[j * 8 + warp] + __popc(masks[j] & lt)], (int32_t)k);
            }
        }
        __syncthreads();  // offs and tile_first are reused by the next tile
    }
}

// Adds the cycles of the lanes timing the same item with one atomic per item
// and warp (all 32 lanes call; id < 0 = nothing timed).
__device__ __forceinline__ void warp_cost_add(unsigned long long* sum, unsigned int* cnt, int id, unsigned cyc)
{
    const unsigned peers = __match_any_sync(0xFFFFFFFFu, id);
    unsigned long long total = 0;
    for (int k = 0; k < 32; ++k) {
        const unsigned v = __shfl_sync(0xFFFFFFFFu, cyc, k);
        if ((peers >> k) & 1u) total += v;
    }
    if (id >= 0 && (threadIdx.x & 31) == (unsigned)(__ffs(peers) - 1)) {
        atomicAdd(sum + id, total);
        atomicAdd(cnt + id, (unsigned)__popc(peers));
    }
}

// CostTracker::record for every item timed in the last bounce, in item order
// (WavefrontRenderer.cpp:833-844), then relativeCost (CostTracker.h:42-55);
// the bounce's sums are cleared.  The reference records once per bounce of a
// one-sample pass; a wave of k samples per pixel records its bounce mean k
// times (`repeat`), so the EMA and the 50-record floor see the same number
// of records.  Block 0 runs the materials, block 1 the textures, each on one
// thread (the EMA total is a serial dependency).
__device__ void cost_update_one(CostTrackerDev T, int repeat)
{
    if (T.items <= 0) return;
    double total = *T.total;
    int tracked = *T.tracked;
    for (int i = 0; i < T.items; ++i) {
        const unsigned n = T.cnt[i];
        if (n == 0) continue;
        const double c = (double)T.sum[i] / (double)n;
        T.sum[i] = 0ull;
        T.cnt[i] = 0u;
        for (int r = 0; r < repeat; ++r) {
            T.samples[i] += 1;
            if (!T.init[i]) {
                T.avg[i] = c;
                T.init[i] = 1;
                tracked += 1;
                total += c;
            } else {
                const double old = T.avg[i];
                const double nw = (1.0 - 0.05) * old + 0.05 * c;
                T.avg[i] = nw;
                total += (nw - old);
            }
        }
    }
    *T.total = total;
    *T.tracked = tracked;
    for (int i = 0; i < T.items; ++i) {
        double r = 1.0;
        if (T.samples[i] >= 50 && tracked != 0) {
            const double g = total / tracked;
            if (g > 0.0) r = T.avg[i] / g;
        }
        T.rel[i] = r;
        if (T.rel_f) T.rel_f[i] = (float)r;
    }
}

__global__ void k_cost_update(CostTrackerDev mat, CostTrackerDev tex, int repeat)
{
    if (threadIdx.x != 0) return;
    cost_update_one(blockIdx.x == 0 ? mat : tex, repeat);
}

// ---------------------------------------------------------------------------
// shadeAll per-hit body (.cpp:602-797): emission with MIS, area-light NEE
// (Scene::sampleLight, src/core/Scene.cpp:192-238) and directional NEE become
// shadow rays carrying their (clamped) contribution; scatter, Russian
// roulette and the next ray.  Random streams per (purpose, depth, pixel,
// sample) — the oracle uses the same ones.
// ---------------------------------------------------------------------------
constexpr int kShadeWarps = 4;  // k_shade's grid is sized in 128-thread blocks
// Resident blocks of k_shade per SM: the multi-job and cost-timed instances,
// and the plain single-job instance, each bounded where it still compiles
// without spills.
#ifndef WF_SHADE_MIN_BLOCKS
#define WF_SHADE_MIN_BLOCKS 7
#endif
#ifndef WF_SHADE_MIN_BLOCKS_PLAIN
#define WF_SHADE_MIN_BLOCKS_PLAIN 8
#endif
// Warps per block of each k_shade form (the same threads per SM whatever the
// block).  The octant grouping of the next rays spans a block, and the warps
// of a larger block walk the large kernel together, sharing its instruction
// cache lines (no_instruction stalls 3.1 -> 0.5 per issue at 512 threads).
// The single-job grouped forms run 512 threads (against 128: dense mesh +1.3%,
// lattice +3.4%; 256: dense mesh the same, lattice -1.3%; 1024: dense mesh
// -0.3%), the cost-timed one too although its 72 registers then spill (dense
// mesh with live cost-aware RR +4.0%); the lean multi-job forms 256 threads at
// 4 blocks per SM, where they still need no spills (served stream +0.7%,
// batched Cornell jobs +1.9%; 512: batched -2%).  The other multi-job forms
// need 72 registers and stay at 128, and so does the plain single-job form,
// whose barrier waits cost more than its cache gains (256: Cornell box -1%,
// 512: -3%).
template <bool kMulti, bool kTimed, bool kLean, bool kGroup>
__host__ __device__ constexpr int shade_warps()
{
    return !kMulti ? (kGroup ? 16 : kShadeWarps) : kLean ? 8 : kShadeWarps;
}
template <bool kMulti, bool kTimed, bool kLean, bool kGroup>
__host__ __device__ constexpr int shade_min_blocks()
{
    return shade_warps<kMulti, kTimed, kLean, kGroup>() == kShadeWarps
               ? ((kMulti || kTimed) ? WF_SHADE_MIN_BLOCKS : WF_SHADE_MIN_BLOCKS_PLAIN)
               : 2048 / (32 * shade_warps<kMulti, kTimed, kLean, kGroup>()) / 2;  // 64 registers a thread
}
// kTimed: the live CostTracker times a quarter of the hits (single-job
// renders only); the other instances carry no clock reads.  kLean: a
// single-job render of a scene without an environment map, textures or a
// directional light runs an instance without the environment-NEE block (two
// map lookups), the texture lookups and the directional NEE — a smaller
// kernel that waits less on the instruction cache (dense mesh +0.9%,
// Cornell box +1.7% for the environment block alone).
template <bool kMulti, bool kTimed, bool kLean = false, bool kGroup = false>
__global__ void __launch_bounds__(32 * shade_warps<kMulti, kTimed, kLean, kGroup>(),
                                  shade_min_blocks<kMulti, kTimed, kLean, kGroup>())
    k_shade(DeviceScene scene0, DeviceJob job0,
                                               const DeviceScene* __restrict__ scenes,
                                               const DeviceJob* __restrict__ jobs, RayQueueDev rq,
                                               HitQueueDev hq, const ull* __restrict__ hq_n, int ray_order,
                                               ShadowQueueDev sh, ull* sh_n, RayQueueDev nx,
                                               ull* nx_n, float* accum_base, int* err)
{
    // hq.ray lists the rays that hit; their records (tri, t, u, v) sit at the
    // list position, or with ray_order at the ray's own index.
    constexpr int kW = shade_warps<kMulti, kTimed, kLean, kGroup>();
    __shared__ unsigned blk_sh[kW], blk_nx[kW];
    __shared__ unsigned blk_oct[8 * kW];  // next rays per (octant, warp), octant-major
    __shared__ ull blk_first[2];
    static_assert(8 * kW == 32 || 8 * kW == 64 || 8 * kW == 128 || 8 * kW == 256, "1, 2, 4 or 8 scan entries per lane");
    const int64_t n = (int64_t)*hq_n;
    WF_BLOCK_LOOP(base, n)
    {
        const int64_t k = base + threadIdx.x;
        const bool active = k < n;
        bool want_area = false, want_dir = false, want_env = false, want_next = false;
        V3 p = {0, 0, 0}, dir_area = {0, 0, 0}, c_area = {0, 0, 0}, dir_sun = {0, 0, 0},
           c_sun = {0, 0, 0}, dir_env = {0, 0, 0}, c_env = {0, 0, 0}, nd = {0, 0, 0}, Tn = {0, 0, 0};
        float dist_area = 0.0f, next_pdf = 0.0f;
        int pixel = 0, depth = 0, sample = 0, job = 0, slot = 0;
        int cost_mat = -1, cost_tex = -1;
        unsigned cyc_mat = 0, cyc_tex = 0;
        if (active) {
            const int64_t pk = hq.order ? (int64_t)hq.order[k] : k;
            const int ri = ldq(&hq.ray[pk]);
            const int64_t hk = ray_order ? (int64_t)ri : pk;
            job = kMulti ? ldq(&rq.job[ri]) : 0;
            const DeviceJob& J = kMulti ? jobs[job] : job0;
            const DeviceScene& S = kMulti ? scenes[J.scene] : scene0;
            float* accum = job_accum(J, accum_base);
            const float ff = J.firefly;
            const uint32_t seed_lo = J.seed_lo, seed_hi = J.seed_hi;
            const V3 o = {ldq(&rq.ox[ri]), ldq(&rq.oy[ri]), ldq(&rq.oz[ri])};
            const V3 d = {ldq(&rq.dx[ri]), ldq(&rq.dy[ri]), ldq(&rq.dz[ri])};
            const V3 T = {ldq(&rq.tr[ri]), ldq(&rq.tg[ri]), ldq(&rq.tb[ri])};
            const float in_pdf = ldq(&rq.pdf[ri]);
            pixel = ldq(&rq.pixel[ri]);
            depth = ldq(&rq.depth[ri]);
            sample = ldq(&rq.sample[ri]);
            slot = job_slot(J, pixel, sample);
            HitRec h;
            rebuild_hit(S, o, d, ldq(&hq.tri[hk]), ldq(&hq.t[hk]), ldq(&hq.bu[hk]), ldq(&hq.bv[hk]), h);
            p = h.p;
            const wf_material m = S.materials[h.mat];
            // Live cost tracking (.cpp:612-625): a quarter of the hits time
            // their surface colour lookup (textured materials) and their
            // scatter with the SM clock.
            bool timed = false;
            if (kTimed && !kMulti && J.cost_sum_mat) {
                Stream cs(seed_lo, seed_hi, kPurposeCostSample, (uint32_t)depth, (uint32_t)pixel,
                          (uint32_t)sample);
                timed = cs.next() < 0.25f;
            }
            // Material::getSurfaceColor, evaluated once per hit: scatter
            // (which starts with it, Material.cpp:165-169) and every NEE term
            // use the same value of this pure lookup.  A timed hit charges
            // its cycles to the texture and, as part of scatter, to the
            // material, as the reference's two timers do.
            const long long tc0 = timed ? clock64() : 0;
            const V3 surf = kLean ? v3(m.albedo[0], m.albedo[1], m.albedo[2]) : surface_color(S, m, h);
            unsigned cyc_surf = 0;
            if (timed) {
                cyc_surf = (unsigned)min(clock64() - tc0, (long long)(1 << 26));
                if (m.texture_id >= 0) {
                    cost_tex = m.texture_id;
                    cyc_tex = cyc_surf;
                }
            }
            // Emission with MIS (.cpp:629-658)
            V3 Le = emitted(m, h.n, d * -1.0f);
            if (Le.x > 0.0f || Le.y > 0.0f || Le.z > 0.0f) {
                float w = 1.0f;
                if (depth > 0 && in_pdf > 0.0f) {
                    float cos_l = fmaxf(0.0f, dot(d * -1.0f, h.n));
                    if (cos_l > 0.0f) {
                        float lp = area_to_angle(S.light_area_pdf, h.t, cos_l);
                        w = mis_balance(in_pdf, lp);
                    }
                }
                Le = vmin(Le, ff);
                accum_add(accum, slot, T * Le * w);
            }
            // Area-light NEE (.cpp:660-710)
            if ((m.type == WF_MATERIAL_DIFFUSE || m.type == WF_MATERIAL_PLASTIC) &&
                S.num_emissive_meshes > 0) {
                Stream lr(seed_lo, seed_hi, kPurposeLight, (uint32_t)depth, (uint32_t)pixel,
                          (uint32_t)sample);
                const int ne = S.num_emissive_meshes;
                const EmissiveMesh em = S.emissive_meshes[(int)(lr.next() * (float)ne) % ne];
                const float xi_tri = lr.next();
                if (em.count > 0) {
                    const int local = (int)(xi_tri * (float)em.count) % em.count;
                    const float4* et = S.emissive_tris + 3 * (int64_t)(em.first + local);
                    const float4 a = __ldg(et), b = __ldg(et + 1), c = __ldg(et + 2);
                    const V3 v0 = {a.x, a.y, a.z}, v1 = {b.x, b.y, b.z}, v2 = {c.x, c.y, c.z};
                    float r1 = lr.next();
                    float r2 = lr.next();
                    if (r1 + r2 > 1.0f) {
                        r1 = 1.0f - r1;
                        r2 = 1.0f - r2;
                    }
                    const float r3 = 1.0f - r1 - r2;
                    const V3 lpnt = v0 * r3 + v1 * r1 + v2 * r2;
                    const V3 ln = normalized(cross(v1 - v0, v2 - v0));
                    const V3 from_light = normalized(p - lpnt);
                    const V3 le = emitted(S.materials[em.material], ln, from_light);
                    const V3 to = lpnt - p;
                    const float dist = length(to);
                    const V3 dl = to / dist;
                    const float cos_s = dot(h.n, dl);
                    const float cos_l = dot(dl * -1.0f, ln);
                    if (cos_s > 0.0f && cos_l > 0.0f) {
                        const float g = (cos_s * cos_l) / (dist * dist);
                        const V3 brdf = surf * (1.0f / kPi);
                        const float lp = area_to_angle(S.light_area_pdf, dist, cos_l);
                        const float bp = cos_s / kPi;
                        const float w = mis_balance(lp, bp);
                        const V3 direct = T * brdf * le * g * S.total_emissive_area * w;
                        c_area = vmin(direct, ff);
                        dir_area = dl;
                        dist_area = dist;
                        want_area = true;
                    }
                }
            }
            // Directional NEE (.cpp:712-737)
            if (!kLean && S.directional.intensity > 0.0f) {
                const V3 to = v3(S.directional.direction[0], S.directional.direction[1],
                                 S.directional.direction[2]) * -1.0f;
                const float cos_s = dot(h.n, to);
                if (cos_s > 0.0f) {
                    const V3 brdf = surf * (1.0f / kPi);
                    const V3 col = {S.directional.color[0], S.directional.color[1], S.directional.color[2]};
                    const V3 direct = T * brdf * col * S.directional.intensity * cos_s;
                    c_sun = vmin(direct, ff);
                    dir_sun = to;
                    want_dir = true;
                }
            }
            // Environment NEE (device addition, off unless the job asks): one
            // importance-sampled direction, balance-heuristic MIS against the
            // cosine lobe (pdf cos/pi, the pdf scatter records), unclamped like
            // the miss term it shares the estimate with.  Plastic's diffuse
            // lobe is chosen with probability 1 - F (Material.cpp:235-260), so
            // its NEE carries that factor.  The last depth gets none: the ray
            // it would share with is never traced (.cpp:154), so the mean stays
            // the miss-only estimator's.
            if (!kLean && J.env_nee && S.env_alias_prob && depth + 1 < J.max_depth &&
                (m.type == WF_MATERIAL_DIFFUSE || m.type == WF_MATERIAL_PLASTIC)) {
                Stream er(seed_lo, seed_hi, kPurposeEnvironment, (uint32_t)depth, (uint32_t)pixel,
                          (uint32_t)sample);
                const float x1 = er.next();
                const float x2 = er.next();
                const float x3 = er.next();
                const float x4 = er.next();
                const V3 wi = env_sample(S, x1, x2, x3, x4);
                const float cos_s = dot(h.n, wi);
                const float pe = env_pdf(S, wi);
                if (cos_s > 0.0f && pe > 0.0f) {
                    float kd = 1.0f;
                    if (m.type == WF_MATERIAL_PLASTIC)
                        kd = 1.0f - schlick(fmaxf(0.0f, dot(d * -1.0f, h.n)), 1.5f);
                    const float bp = cos_s / kPi;
                    c_env = T * surf * (kd / kPi) * sky_color(S, wi) * (cos_s / (pe + bp));
                    dir_env = wi;
                    want_env = true;
                }
            }
            // Scatter + Russian roulette (.cpp:739-796)
            Stream sr(seed_lo, seed_hi, kPurposeScatter, (uint32_t)depth, (uint32_t)pixel,
                      (uint32_t)sample);
            V3 att;
            float spdf;
            const long long ts0 = timed ? clock64() : 0;
            const bool scattered = scatter(m, surf, d, h, sr, att, nd, spdf);
            if (timed) {
                cost_mat = h.mat;
                cyc_mat = (unsigned)min(clock64() - ts0 + (long long)cyc_surf, (long long)(1 << 26));
            }
            if (scattered) {
                Tn = T * att;
                bool alive = true;
                if (depth + 1 >= J.rr_min_depth) {
                    float q = fminf(0.95f, fmaxf(Tn.x, fmaxf(Tn.y, Tn.z)));
                    if (J.cost_aware_rr) {
                        float rc = J.rel_cost_material ? J.rel_cost_material[h.mat] : 1.0f;
                        q = fminf(fmaxf(q / rc, 0.05f), 0.95f);
                    }
                    Stream rr(seed_lo, seed_hi, kPurposeRoulette, (uint32_t)depth,
                              (uint32_t)pixel, (uint32_t)sample);
                    if (rr.next() > q)
                        alive = false;
                    else
                        Tn = Tn / q;
                }
                // the reference traces depths 0 .. maxDepth-1 (.cpp:154)
                if (alive && depth + 1 < J.max_depth) {
                    want_next = true;
                    next_pdf = spdf;
                }
            }
        }
        __syncwarp();
        if (kTimed && !kMulti && job0.cost_sum_mat) {
            warp_cost_add(job0.cost_sum_mat, job0.cost_cnt_mat, cost_mat, cyc_mat);
            warp_cost_add(job0.cost_sum_tex, job0.cost_cnt_tex, cost_tex, cyc_tex);
        }
        // One reservation per block and queue: the block's shadow rays (each
        // warp's area, then directional, then environment rays) and next rays
        // keep the order of the hits, with one atomic per block and counter.
        const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
        const unsigned lt = (1u << lane) - 1u;
        const unsigned ma = __ballot_sync(0xFFFFFFFFu, want_area), md = __ballot_sync(0xFFFFFFFFu, want_dir);
        const unsigned me = __ballot_sync(0xFFFFFFFFu, want_env);
        int64_t sh0, pn;
        if constexpr (kGroup) {
            // The block's next rays are written grouped by the octant of their
            // direction (octant-major, then warp, then lane), so the warps that
            // fetch them get rays whose traversals take the same child order.
            const unsigned oct = (__float_as_uint(nd.x) >> 31) | (__float_as_uint(nd.y) >> 31) << 1 |
                                 (__float_as_uint(nd.z) >> 31) << 2;
            // Lanes of octant o among those with a next ray: mn with every bit
            // of o matched against the ballot of that bit.
            const unsigned mn = __ballot_sync(0xFFFFFFFFu, want_next);
            const unsigned b0 = __ballot_sync(0xFFFFFFFFu, oct & 1u), b1 = __ballot_sync(0xFFFFFFFFu, oct & 2u),
                           b2 = __ballot_sync(0xFFFFFFFFu, oct & 4u);
            const auto peers = [&](unsigned o) {
                return mn & ~((b0 ^ (0u - (o & 1u))) | (b1 ^ (0u - ((o >> 1) & 1u))) | (b2 ^ (0u - ((o >> 2) & 1u))));
            };
            const unsigned oct_rank = (unsigned)__popc(peers(oct) & lt);
            if (lane < 8) blk_oct[lane * kW + warp] = (unsigned)__popc(peers((unsigned)lane));
            if (lane == 0) blk_sh[warp] = (unsigned)(__popc(ma) + __popc(md) + __popc(me));
            __syncthreads();
            if (warp == 0) {
                constexpr int kPer = 8 * kW / 32;  // entries per lane
                unsigned e[kPer], v = 0;
#pragma unroll
                for (int q = 0; q < kPer; ++q) {
                    e[q] = blk_oct[kPer * lane + q];
                    v += e[q];
                }
                unsigned x = v;
#pragma unroll
                for (int dd = 1; dd < 32; dd <<= 1) {
                    const unsigned y = __shfl_up_sync(0xFFFFFFFFu, x, dd);
                    if (lane >= dd) x += y;
                }
                unsigned ex = x - v;
#pragma unroll
                for (int q = 0; q < kPer; ++q) {
                    blk_oct[kPer * lane + q] = ex;
                    ex += e[q];
                }
                const unsigned tn = __shfl_sync(0xFFFFFFFFu, x, 31);
                if (lane == 0) {
                    unsigned ts = 0;
                    for (int w = 0; w < kW; ++w) {
                        const unsigned a = blk_sh[w];
                        blk_sh[w] = ts;
                        ts += a;
                    }
                    blk_first[0] = ts ? atomicAdd(sh_n, (ull)ts) : 0ull;
                    blk_first[1] = tn ? atomicAdd(nx_n, (ull)tn) : 0ull;
                }
            }
            __syncthreads();
            sh0 = (int64_t)blk_first[0] + blk_sh[warp];
            pn = (int64_t)blk_first[1] + blk_oct[(want_next ? oct : 0u) * kW + warp] + oct_rank;
        } else {
            const unsigned mn = __ballot_sync(0xFFFFFFFFu, want_next);
            if (lane == 0) {
                blk_sh[warp] = (unsigned)(__popc(ma) + __popc(md) + __popc(me));
                blk_nx[warp] = (unsigned)__popc(mn);
            }
            __syncthreads();
            if (threadIdx.x == 0) {
                unsigned ts = 0, tn = 0;
                for (int w = 0; w < kW; ++w) {
                    const unsigned a = blk_sh[w], b = blk_nx[w];
                    blk_sh[w] = ts;
                    blk_nx[w] = tn;
                    ts += a;
                    tn += b;
                }
                blk_first[0] = ts ? atomicAdd(sh_n, (ull)ts) : 0ull;
                blk_first[1] = tn ? atomicAdd(nx_n, (ull)tn) : 0ull;
            }
            __syncthreads();
            sh0 = (int64_t)blk_first[0] + blk_sh[warp];
            pn = (int64_t)blk_first[1] + blk_nx[warp] + __popc(mn & lt);
        }
        __syncthreads();  // the block's words are rewritten by the next iteration
        const int64_t pa = sh0 + __popc(ma & lt);
        const int64_t pd = sh0 + __popc(ma) + __popc(md & lt);
        const int64_t pe = sh0 + __popc(ma) + __popc(md) + __popc(me & lt);
        if (want_area) {
            if (pa < sh.capacity) {
                stq(&sh.ox[pa], p.x); stq(&sh.oy[pa], p.y); stq(&sh.oz[pa], p.z);
                stq(&sh.dx[pa], dir_area.x); stq(&sh.dy[pa], dir_area.y); stq(&sh.dz[pa], dir_area.z);
                stq(&sh.dist[pa], dist_area);
                stq(&sh.cr[pa], c_area.x); stq(&sh.cg[pa], c_area.y); stq(&sh.cb[pa], c_area.z);
                stq(&sh.pixel[pa], slot);
                stq(&sh.job[pa], job);
            } else {
                atomicOr(err, 4);
            }
        }
        if (want_dir) {
            if (pd < sh.capacity) {
                stq(&sh.ox[pd], p.x); stq(&sh.oy[pd], p.y); stq(&sh.oz[pd], p.z);
                stq(&sh.dx[pd], dir_sun.x); stq(&sh.dy[pd], dir_sun.y); stq(&sh.dz[pd], dir_sun.z);
                stq(&sh.dist[pd], 1e6f);
                stq(&sh.cr[pd], c_sun.x); stq(&sh.cg[pd], c_sun.y); stq(&sh.cb[pd], c_sun.z);
                stq(&sh.pixel[pd], slot);
                stq(&sh.job[pd], job);
            } else {
                atomicOr(err, 4);
            }
        }
        if (want_env) {
            if (pe < sh.capacity) {
                stq(&sh.ox[pe], p.x); stq(&sh.oy[pe], p.y); stq(&sh.oz[pe], p.z);
                stq(&sh.dx[pe], dir_env.x); stq(&sh.dy[pe], dir_env.y); stq(&sh.dz[pe], dir_env.z);
                stq(&sh.dist[pe], 1e6f);
                stq(&sh.cr[pe], c_env.x); stq(&sh.cg[pe], c_env.y); stq(&sh.cb[pe], c_env.z);
                stq(&sh.pixel[pe], slot);
                stq(&sh.job[pe], job);
            } else {
                atomicOr(err, 4);
            }
        }
        if (want_next) {
            if (pn < nx.capacity) {
                stq(&nx.ox[pn], p.x); stq(&nx.oy[pn], p.y); stq(&nx.oz[pn], p.z);
                stq(&nx.dx[pn], nd.x); stq(&nx.dy[pn], nd.y); stq(&nx.dz[pn], nd.z);
                stq(&nx.tr[pn], Tn.x); stq(&nx.tg[pn], Tn.y); stq(&nx.tb[pn], Tn.z);
                stq(&nx.pdf[pn], next_pdf);
                stq(&nx.pixel[pn], pixel);
                stq(&nx.depth[pn], depth + 1);
                stq(&nx.sample[pn], sample);
                stq(&nx.job[pn], job);
            } else {
                atomicOr(err, 8);
            }
        }
    }
}

// Shadow rays (EmbreeAccelerator::occluded): unblocked contributions are
// added to their pixel.  Same persistent, dynamic-fetch structure as
// k_trace_render.
template <bool kMulti, int kMinBlocks, class Tr>
__global__ void __launch_bounds__(128, kMinBlocks) k_occluded_render(DeviceScene scene0, DeviceJob job0,
                                                                     const DeviceScene* __restrict__ scenes,
                                                                     const DeviceJob* __restrict__ jobs,
                                                                     ShadowQueueDev sh,
                                                                     const ull* __restrict__ d_n,
                                                                     float* accum, ull* work, int* err)
{
    const int64_t n = (int64_t)*d_n;
    const int lane = threadIdx.x & 31;
    const unsigned lt = (1u << lane) - 1u;
    Tr tr;
    typename Tr::Entry stack[Tr::kStack];
    const DeviceScene* S = kMulti ? scenes : &scene0;
    int job = 0;
    int64_t ray = -1;
    bool exhausted = false;
    bool overflow = false;
    tr.idle();
    for (;;) {
        if (ray >= 0 && tr.done()) {
            if (tr.res.leafpos < 0)  // sh.pixel holds the slot (job_slot)
                accum_add(job_accum(kMulti ? jobs[job] : job0, accum), ldq(&sh.pixel[ray]),
                          v3(ldq(&sh.cr[ray]), ldq(&sh.cg[ray]), ldq(&sh.cb[ray])));
            overflow = overflow || tr.overflow;
            ray = -1;
        }
        const bool need = ray < 0 && !exhausted;
        const unsigned nm = __ballot_sync(0xFFFFFFFFu, need);
        if (nm && (__popc(nm) >= WF_REFILL_MIN || __all_sync(0xFFFFFFFFu, ray < 0))) {
            ull base = 0;
            const int leader = __ffs(nm) - 1;
            if (lane == leader) base = atomicAdd(work, (ull)__popc(nm));
            base = __shfl_sync(0xFFFFFFFFu, base, leader);
            if (need) {
                const int64_t idx = (int64_t)base + __popc(nm & lt);
                if (idx < n) {
                    ray = idx;
                    if (kMulti) {
                        job = ldq(&sh.job[idx]);
                        S = scenes + jobs[job].scene;
                    }
                    tr.init(*S, stack, v3(ldq(&sh.ox[idx]), ldq(&sh.oy[idx]), ldq(&sh.oz[idx])),
                            v3(ldq(&sh.dx[idx]), ldq(&sh.dy[idx]), ldq(&sh.dz[idx])), 0.001f, ldq(&sh.dist[idx]) - 0.001f);
                } else {
                    exhausted = true;
                }
            }
        }
        if (__all_sync(0xFFFFFFFFu, ray < 0)) break;
        if (ray >= 0 && !tr.done()) {
            tr.round(*S, stack);
        }
    }
    if (overflow) atomicOr(err, 1);
}

// ---------------------------------------------------------------------------
// RayQueue::sortKey (include/scheduling/RayQueue.h:135-162).
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t spread10(uint32_t v)
{
    v &= 0x3FFu;
    v = (v | (v << 16)) & 0x30000FFu;
    v = (v | (v << 8)) & 0x300F00Fu;
    v = (v | (v << 4)) & 0x30C30C3u;
    v = (v | (v << 2)) & 0x9249249u;
    return v;
}

__device__ __forceinline__ uint32_t quant_ray(float v, float mn, float ex)
{
    float t = (v - mn) / ex;
    t = fminf(fmaxf(t, 0.0f), 1.0f);
    return (uint32_t)(t * 1023.0f);
}

__device__ __forceinline__ uint64_t ray_key(float ox, float oy, float oz, float dx, float dy, float dz,
                                            float3 mn, float3 ex)
{
    uint64_t oct = (dx < 0.0f ? 1u : 0u) | (dy < 0.0f ? 2u : 0u) | (dz < 0.0f ? 4u : 0u);
    uint64_t m = spread10(quant_ray(ox, mn.x, ex.x)) | (spread10(quant_ray(oy, mn.y, ex.y)) << 1) |
                 (spread10(quant_ray(oz, mn.z, ex.z)) << 2);
    return (oct << 30) | m;
}

// Scene bounds of each ray's own scene (Scene::computeBounds), extent
// floored at 1e-6 (RayQueue.h:143-145).
__global__ void k_ray_keys(const DeviceScene* __restrict__ scenes, const DeviceJob* __restrict__ jobs,
                           RayQueueDev rq, const ull* __restrict__ d_n, uint64_t* keys, uint32_t* vals)
{
    const int64_t n = (int64_t)*d_n;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const DeviceScene& S = scenes[jobs[rq.job[i]].scene];
        const float3 mn = make_float3(S.bmin[0], S.bmin[1], S.bmin[2]);
        const float3 ex = make_float3(fmaxf(S.bmax[0] - S.bmin[0], 1e-6f), fmaxf(S.bmax[1] - S.bmin[1], 1e-6f),
                                      fmaxf(S.bmax[2] - S.bmin[2], 1e-6f));
        keys[i] = ray_key(rq.ox[i], rq.oy[i], rq.oz[i], rq.dx[i], rq.dy[i], rq.dz[i], mn, ex);
        vals[i] = (uint32_t)i;
    }
}

__global__ void k_ray_keys_raw(int64_t n, const float* ox, const float* oy, const float* oz,
                               const float* dx, const float* dy, const float* dz, float3 mn,
                               float3 ex, uint64_t* keys, uint32_t* vals)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        keys[i] = ray_key(ox[i], oy[i], oz[i], dx[i], dy[i], dz[i], mn, ex);
        vals[i] = (uint32_t)i;
    }
}

__global__ void k_gather_rays(RayQueueDev in, const uint32_t* __restrict__ perm,
                              const ull* __restrict__ d_n, RayQueueDev out)
{
    const int64_t n = (int64_t)*d_n;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const uint32_t j = perm[i];
        out.ox[i] = in.ox[j];
        out.oy[i] = in.oy[j];
        out.oz[i] = in.oz[j];
        out.dx[i] = in.dx[j];
        out.dy[i] = in.dy[j];
        out.dz[i] = in.dz[j];
        out.tr[i] = in.tr[j];
        out.tg[i] = in.tg[j];
        out.tb[i] = in.tb[j];
        out.pdf[i] = in.pdf[j];
        out.pixel[i] = in.pixel[j];
        out.depth[i] = in.depth[j];
        out.sample[i] = in.sample[j];
        out.job[i] = in.job[j];
    }
}

// ---------------------------------------------------------------------------
// ShadingQueue scheduling (include/scheduling/ShadingQueue.h:90-141,
// 277-329, 437-550).
// ---------------------------------------------------------------------------
constexpr int kCbSharedMaterials = 4096;  // per-block benefit sums up to 32 KB

__global__ void k_type_stats(ShadeColumnsDev c, const ull* __restrict__ d_n,
                             const wf_material* __restrict__ mats, int num_tex,
                             const int64_t* __restrict__ tex_bytes, ull* counts, ull* mem,
                             int* first)
{
    __shared__ unsigned long long s_cnt[8], s_mem[8];
    __shared__ int s_first[8];
    if (threadIdx.x < 8) {
        s_cnt[threadIdx.x] = 0;
        s_mem[threadIdx.x] = 0;
        s_first[threadIdx.x] = 0x7FFFFFFF;
    }
    __syncthreads();
    const int64_t n = (int64_t)*d_n;
    const int lane = threadIdx.x & 31;
    // whole warps iterate together so that equal types aggregate per warp
    for (int64_t b = blockIdx.x * (int64_t)blockDim.x; b < n; b += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = b + threadIdx.x;
        const bool ok = i < n;
        const int ty = ok ? (mats[c.mat[i]].type & 7) : -1;
        const int tid = ok ? c.tex[i] : -1;
        const ull mem = (tid >= 0 && tid < num_tex) ? (ull)tex_bytes[tid] : 0ull;
        const unsigned peers = __match_any_sync(0xFFFFFFFFu, ty);
        ull msum = 0;
        for (int k = 0; k < 32; ++k) {
            const ull v = __shfl_sync(0xFFFFFFFFu, mem, k);
            if ((peers >> k) & 1u) msum += v;
        }
        if (ok && lane == __ffs(peers) - 1) {  // the lowest lane holds the group's first index
            atomicAdd(&s_cnt[ty], (ull)__popc(peers));
            atomicMin(&s_first[ty], (int)i);
            if (msum) atomicAdd(&s_mem[ty], msum);
        }
    }
    __syncthreads();
    if (threadIdx.x < 8) {
        if (s_cnt[threadIdx.x]) {
            atomicAdd(&counts[threadIdx.x], s_cnt[threadIdx.x]);
            atomicAdd(&mem[threadIdx.x], s_mem[threadIdx.x]);
            atomicMin(&first[threadIdx.x], s_first[threadIdx.x]);
        }
    }
}

struct Rank8 {
    int r[8];
};

__global__ void k_policy_keys(ShadeColumnsDev c, const ull* __restrict__ d_n,
                              const wf_material* __restrict__ mats, int policy, Rank8 type_rank,
                              const int* __restrict__ cost_rank, const int* __restrict__ tex_rank,
                              int num_tex, int shift, uint64_t* keys, uint32_t* vals)
{
    const int64_t n = (int64_t)*d_n;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const int m = c.mat[i];
        const uint64_t tr = (uint64_t)type_rank.r[mats[m].type & 7];
        uint64_t sec;
        if (policy == WF_POLICY_TEXTURE_AWARE) {
            const int tid = c.tex[i];
            sec = (uint64_t)tex_rank[(tid >= 0 && tid < num_tex) ? tid : num_tex];
        } else {
            sec = (uint64_t)cost_rank[m];
        }
        keys[i] = (tr << shift) | sec;
        vals[i] = (uint32_t)i;
    }
}

__device__ __forceinline__ unsigned float_to_ordered(float f)
{
    unsigned b = __float_as_uint(f);
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}
__device__ __forceinline__ float ordered_to_float(unsigned u)
{
    unsigned b = (u & 0x80000000u) ? (u & 0x7FFFFFFFu) : ~u;
    return __uint_as_float(b);
}

// Per-material benefit (sum of luminance(throughput), in double) and the hit
// points' bounds.  Lanes of a warp hitting the same material add their sum
// once; with few enough materials a block first sums into shared memory.
__global__ void k_cb_reduce(ShadeColumnsDev c, const ull* __restrict__ d_n, double* benefit,
                            int* present, unsigned* bounds6, int num_materials)
{
    extern __shared__ double s_benefit[];
    const bool staged = num_materials <= kCbSharedMaterials;
    if (staged)
        for (int m = threadIdx.x; m < num_materials; m += blockDim.x) s_benefit[m] = 0.0;
    __syncthreads();
    __shared__ float s_lum[8][32];  // 256-thread blocks: one row per warp
    const int64_t n = (int64_t)*d_n;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    unsigned mn[3] = {0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu}, mx[3] = {0u, 0u, 0u};
    for (int64_t b = blockIdx.x * (int64_t)blockDim.x; b < n; b += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = b + threadIdx.x;
        const bool ok = i < n;
        const int m = ok ? c.mat[i] : -1;
        // luminance, include/render/AdaptiveSampler.h:21-27 (float), summed in double
        s_lum[warp][lane] = ok ? 0.2126f * c.tr[i] + 0.7152f * c.tg[i] + 0.0722f * c.tb[i] : 0.0f;
        const unsigned peers = __match_any_sync(0xFFFFFFFFu, m);
        __syncwarp();
        // The leader of each material's lanes sums their luminances in
        // float-float (two-sum, then renormalised: ~2^-48 relative), one FP64
        // add per group: a 32-step double loop per warp made this kernel wait
        // on the FP64 pipe, which takes 16 cycles per warp-wide add here.
        if (ok && lane == __ffs(peers) - 1) {
            float hi = 0.0f, lo = 0.0f;
            for (unsigned rest = peers; rest; rest &= rest - 1) {
                const float v = s_lum[warp][__ffs(rest) - 1];
                const float s = hi + v;
                const float bv = s - hi;
                float e = (hi - (s - bv)) + (v - bv);
                e += lo;
                hi = s + e;
                lo = e - (hi - s);
            }
            const double sum = (double)hi + (double)lo;
            if (staged)
                atomicAdd(&s_benefit[m], sum);
            else
                atomicAdd(&benefit[m], sum);
            present[m] = 1;
        }
        __syncwarp();
        if (ok) {
            const float p3[3] = {c.px[i], c.py[i], c.pz[i]};
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                unsigned o = float_to_ordered(p3[k]);
                mn[k] = min(mn[k], o);
                mx[k] = max(mx[k], o);
            }
        }
    }
    __syncthreads();
    if (staged)
        for (int m = threadIdx.x; m < num_materials; m += blockDim.x)
            if (s_benefit[m] != 0.0) atomicAdd(&benefit[m], s_benefit[m]);
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        for (int off = 16; off > 0; off >>= 1) {
            mn[k] = min(mn[k], __shfl_xor_sync(0xFFFFFFFFu, mn[k], off));
            mx[k] = max(mx[k], __shfl_xor_sync(0xFFFFFFFFu, mx[k], off));
        }
    }
    if ((threadIdx.x & 31) == 0) {
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            atomicMin(&bounds6[k], mn[k]);
            atomicMax(&bounds6[3 + k], mx[k]);
        }
    }
}

// computeMortonCode quantisation (ShadingQueue.h:523-529).
__device__ __forceinline__ uint32_t quant_cb(float v, float lo, float hi)
{
    float t = (hi > lo) ? (v - lo) / (hi - lo) : 0.0f;
    return (uint32_t)(fminf(fmaxf(t, 0.0f), 1.0f) * 1023.0f);
}

__global__ void k_cb_keys(ShadeColumnsDev c, const ull* __restrict__ d_n,
                          const wf_material* __restrict__ mats, const int* __restrict__ prio_rank,
                          int prio_bits, const unsigned* __restrict__ bounds6, uint64_t* keys,
                          uint32_t* vals)
{
    const int64_t n = (int64_t)*d_n;
    float lo[3], hi[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        lo[k] = ordered_to_float(bounds6[k]);
        hi[k] = ordered_to_float(bounds6[3 + k]);
    }
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const int m = c.mat[i];
        const uint64_t ty = (uint64_t)(mats[m].type & 7);
        const uint64_t pr = (uint64_t)prio_rank[m];
        const uint64_t morton = (uint64_t)spread10(quant_cb(c.px[i], lo[0], hi[0])) |
                                ((uint64_t)spread10(quant_cb(c.py[i], lo[1], hi[1])) << 1) |
                                ((uint64_t)spread10(quant_cb(c.pz[i], lo[2], hi[2])) << 2);
        keys[i] = (ty << (prio_bits + 30)) | (pr << 30) | morton;
        vals[i] = (uint32_t)i;
    }
}

// kFull: also the throughput and hit point (costBenefit's benefit and Morton
// keys); the material and texture policies read only the ids (C2 material
// schedule: the full columns took 8.5 of its 17.6 ms per step).  scene:
// every hit's scene when the wave has one job, else null (looked up per ray).
template <bool kFull>
__global__ void k_hit_columns(const DeviceScene* __restrict__ scenes, const DeviceJob* __restrict__ jobs,
                              const DeviceScene* __restrict__ scene, RayQueueDev rq, HitQueueDev hq,
                              const ull* __restrict__ d_n, ShadeColumnsMut out)
{
    const int64_t n = (int64_t)*d_n;
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n;
         k += (int64_t)gridDim.x * blockDim.x) {
        const int ri = (kFull || !scene) ? hq.ray[k] : 0;
        const DeviceScene& S = scene ? *scene : scenes[jobs[rq.job[ri]].scene];
        const float4 b = __ldg(S.tris + 3 * (int64_t)hq.tri[k] + 1);
        const int m = S.mesh_material[__float_as_int(b.w)];
        out.mat[k] = m;
        out.tex[k] = S.materials[m].texture_id;
        if (!kFull) continue;
        out.tr[k] = rq.tr[ri];
        out.tg[k] = rq.tg[ri];
        out.tb[k] = rq.tb[ri];
        const float t = hq.t[k];
        out.px[k] = rq.ox[ri] + rq.dx[ri] * t;
        out.py[k] = rq.oy[ri] + rq.dy[ri] * t;
        out.pz[k] = rq.oz[ri] + rq.dz[ri] * t;
    }
}

__global__ void k_permute_hits(HitQueueDev in, const uint32_t* __restrict__ perm,
                               const ull* __restrict__ d_n, HitQueueDev out)
{
    const int64_t n = (int64_t)*d_n;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const uint32_t j = perm[i];
        out.ray[i] = in.ray[j];
        out.tri[i] = in.tri[j];
        out.t[i] = in.t[j];
        out.bu[i] = in.bu[j];
        out.bv[i] = in.bv[j];
    }
}

// ---------------------------------------------------------------------------
// Per-bounce stages on caller-held queues (the wf_intersect / wf_miss /
// wf_shading_queue_* entry points).
// ---------------------------------------------------------------------------

// The rays of a ray-order trace that missed (record tri < 0), listed with one
// atomic per warp.
__global__ void k_list_misses(const int32_t* __restrict__ tri, const ull* __restrict__ d_n, uint32_t* list,
                              ull* list_n)
{
    const int64_t n = (int64_t)*d_n;
    const int lane = threadIdx.x & 31;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t base = (int64_t)blockIdx.x * blockDim.x; base < n; base += stride) {
        const int64_t i = base + threadIdx.x;
        const bool miss = i < n && tri[i] < 0;
        const unsigned m = __ballot_sync(0xFFFFFFFFu, miss);
        if (!m) continue;
        ull first = 0;
        if (lane == 0) first = atomicAdd(list_n, (ull)__popc(m));
        first = __shfl_sync(0xFFFFFFFFu, first, 0);
        if (miss) list[first + __popc(m & ((1u << lane) - 1u))] = (uint32_t)i;
    }
}

// The miss loop over a queue of missed rays (renderScene, .cpp:256-265).
__global__ void k_miss_queue(DeviceScene scene0, DeviceJob job0, RayQueueDev rq, const ull* __restrict__ d_n,
                             float* accum)
{
    const int64_t n = (int64_t)*d_n;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        shade_miss<false>(scene0, job0, nullptr, nullptr, rq, i, accum);
}

// A hit queue in list order: entry i of `out` is entry perm[i] (or i) of `in`,
// whose record sits at the entry's position or, with at_ray, at its ray's
// index.  ShadingQueue::materialize for the compact queue.
__global__ void k_materialize_hits(HitQueueDev in, int at_ray, const uint32_t* __restrict__ perm,
                                   const ull* __restrict__ d_n, HitQueueDev out)
{
    const int64_t n = (int64_t)*d_n;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t j = perm ? (int64_t)perm[i] : i;
        const int32_t ray = in.ray[j];
        const int64_t r = at_ray ? (int64_t)ray : j;
        out.ray[i] = ray;
        out.tri[i] = in.tri[r];
        out.t[i] = in.t[r];
        out.bu[i] = in.bu[r];
        out.bv[i] = in.bv[r];
    }
}

// The 24 columns of a ShadingQueue, in queue order: the HitRecord rebuilt from
// the triangle (as the traversal's epilogue builds it) and the ray's columns.
__global__ void k_shading_columns(DeviceScene S, RayQueueDev rq, HitQueueDev hq, int at_ray,
                                  const ull* __restrict__ d_n, HitColumnsDev out, RayQueueDev ro)
{
    const int64_t n = (int64_t)*d_n;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int32_t ray = hq.ray[i];
        const int64_t r = at_ray ? (int64_t)ray : i;
        const V3 o = {rq.ox[ray], rq.oy[ray], rq.oz[ray]}, d = {rq.dx[ray], rq.dy[ray], rq.dz[ray]};
        HitRec h;
        rebuild_hit(S, o, d, hq.tri[r], hq.t[r], hq.bu[r], hq.bv[r], h);
        out.geom[i] = h.geom;
        out.prim[i] = h.prim;
        out.t[i] = h.t;
        out.bu[i] = hq.bu[r];
        out.bv[i] = hq.bv[r];
        out.px[i] = h.p.x;
        out.py[i] = h.p.y;
        out.pz[i] = h.p.z;
        out.nx[i] = h.n.x;
        out.ny[i] = h.n.y;
        out.nz[i] = h.n.z;
        out.front[i] = h.front ? 1 : 0;
        out.u[i] = h.u;
        out.v[i] = h.v;
        out.mat[i] = h.mat;
        out.tex[i] = h.tex;
        ro.ox[i] = o.x;
        ro.oy[i] = o.y;
        ro.oz[i] = o.z;
        ro.dx[i] = d.x;
        ro.dy[i] = d.y;
        ro.dz[i] = d.z;
        ro.tr[i] = rq.tr[ray];
        ro.tg[i] = rq.tg[ray];
        ro.tb[i] = rq.tb[ray];
        ro.pdf[i] = rq.pdf[ray];
        ro.pixel[i] = rq.pixel[ray];
        ro.depth[i] = rq.depth[ray];
        ro.sample[i] = rq.sample[ray];
    }
}

__global__ void k_finalize(const float* accum, int64_t n, float spp, float* image)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
        image[i] = accum[i] / spp;  // writeAveragedImage, WavefrontRenderer.cpp:127-137
}

// ---------------------------------------------------------------------------
// Adaptive sampling (AdaptiveSampler.h:27-105 and its use in renderScene,
// WavefrontRenderer.cpp:141-145, 270-294, 127-137).
// ---------------------------------------------------------------------------

// After a wave: every sample of every active pixel, in sample order, is added
// to the pixel sum and luminance(sum after - sum before) goes to Welford's
// update (AdaptiveSampler::addSample, :41-53); the slot is cleared.
__global__ void k_adaptive_fold(float* __restrict__ sample_buf, int64_t np, int nspp, int slot0, int wave_spp,
                                float* __restrict__ accum, float* __restrict__ mean, float* __restrict__ m2,
                                int32_t* __restrict__ count, const int32_t* __restrict__ active, int32_t n_active)
{
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n_active;
         r += (int64_t)gridDim.x * blockDim.x) {
        const int64_t p = active[r];
        float ar = accum[3 * p], ag = accum[3 * p + 1], ab = accum[3 * p + 2];
        float mu = mean[p], M2 = m2[p];
        int n = count[p];
        for (int k = 0; k < nspp; ++k) {
            float* b = sample_buf + 3 * ((int64_t)((slot0 + k) % wave_spp) * np + p);
            const float nr = ar + b[0], ng = ag + b[1], nb = ab + b[2];
            b[0] = 0.0f;
            b[1] = 0.0f;
            b[2] = 0.0f;
            const float lum = 0.2126f * (nr - ar) + 0.7152f * (ng - ag) + 0.0722f * (nb - ab);
            ar = nr;
            ag = ng;
            ab = nb;
            n += 1;
            const float d1 = lum - mu;
            mu += d1 / (float)n;
            const float d2 = lum - mu;
            M2 += d1 * d2;
        }
        accum[3 * p] = ar;
        accum[3 * p + 1] = ag;
        accum[3 * p + 2] = ab;
        mean[p] = mu;
        m2[p] = M2;
        count[p] = n;
    }
}

// AdaptiveSampler::updateConvergence (:55-78): from 32 samples on, a pixel
// whose standard error of the mean falls below threshold * (mean + 0.01)
// stops.
__global__ void k_adaptive_check(const float* __restrict__ mean, const float* __restrict__ m2,
                                 const int32_t* __restrict__ count, const int32_t* __restrict__ active,
                                 int32_t n_active, float threshold, int32_t* __restrict__ flag)
{
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n_active;
         r += (int64_t)gridDim.x * blockDim.x) {
        const int32_t p = active[r];
        const int n = count[p];
        if (n < 32) continue;
        const float var = m2[p] / (float)(n - 1);
        const float se = sqrtf(var / (float)n);
        if (se < threshold * (mean[p] + 0.01f)) flag[p] = 0;
    }
}

// The pixels still active, in index order: their flags' exclusive prefix sum
// gives each one its position.
__global__ void k_scatter_active(const int32_t* __restrict__ flag, const int32_t* __restrict__ pos, int64_t np,
                                 int32_t* __restrict__ out)
{
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < np; p += (int64_t)gridDim.x * blockDim.x)
        if (flag[p]) out[pos[p]] = (int32_t)p;
}

// writeAveragedImage with per-pixel counts (.cpp:127-137).
__global__ void k_finalize_counts(const float* __restrict__ accum, const int32_t* __restrict__ count, int64_t np,
                                  float* __restrict__ image)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < 3 * np;
         i += (int64_t)gridDim.x * blockDim.x)
        image[i] = accum[i] / (float)max(count[i / 3], 1);
}

__global__ void k_fill_i32(int32_t* __restrict__ a, int64_t n, int32_t v, int identity)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        a[i] = identity ? (int32_t)i : v;
}

inline int grid_for(int64_t n, int block, int cap)
{
    int64_t g = (n + block - 1) / block;
    if (g > cap) g = cap;
    if (g < 1) g = 1;
    return (int)g;
}

}  // namespace

void launch_camera(const wf_camera& cam, int W, int H, uint32_t s0, uint32_t s1, int first_sample,
                   int nspp, RayQueueDev rq, cudaStream_t s)
{
    int64_t n = (int64_t)W * H * nspp;
    k_camera<<<grid_for(n, 256, 65535), 256, 0, s>>>(cam, W, H, s0, s1, first_sample, nspp, rq);
}

void launch_trace_api(const DeviceScene& S, int64_t n, const float* ox, const float* oy,
                      const float* oz, const float* dx, const float* dy, const float* dz,
                      float tmin, float tmax, HitColumnsDev out, int* err, LaunchCfg cfg,
                      cudaStream_t s)
{
    k_trace_api<<<grid_for(n, 128, cfg.grid), 128, 0, s>>>(S, n, ox, oy, oz, dx, dy, dz, tmin, tmax,
                                                          out, err);
}

void launch_occluded_api(const DeviceScene& S, int64_t n, const float* ox, const float* oy,
                         const float* oz, const float* dx, const float* dy, const float* dz,
                         const float* maxd, uint8_t* out, int* err, LaunchCfg cfg, cudaStream_t s)
{
    k_occluded_api<<<grid_for(n, 128, cfg.grid), 128, 0, s>>>(S, n, ox, oy, oz, dx, dy, dz, maxd,
                                                             out, err);
}

// variant: 0 = no occupancy hint, 1 = 9 blocks of 128 per SM; the traversal
// follows the scene's tree (binary or 4-wide).  (The stack in shared memory,
// whole or its bottom six entries, the tree's top nodes staged in shared
// memory, speculative while-while, a compressed 8-wide tree and an L2
// persistence window over the tree all measured slower on every workload and
// were taken out.)
// Where a ray-order bounce shades its misses: an environment-map lookup
// (atan2, asin, a texel fetch) evaluated by finished lanes inside the
// traversal loop stalls their warp, so for a single-job render of a scene
// with a map the compaction pass shades the misses in ray order (lattice
// scene +1.3%); the gradient sky stays in the traversal kernel, where it is
// cheaper than a second pass over the ray columns (Cornell box, dense mesh,
// batched jobs measured 1-5% slower with the move).
static bool misses_in_compaction(const WaveTables& t, bool ray_order)
{
    return ray_order && !t.multi && t.scene0.env_rgb != nullptr;
}

// Multi-job waves: the binary traversal kernels hold 68 (closest hit) and 60
// (shadow rays) registers, 7 and 8 resident blocks per SM.  Where one of the
// resident scenes is dense (its tree and triangles from kDenseSceneBytes on)
// variant 0 runs them at 9 blocks (56 registers), which hides more of the
// dense scene's memory latency: the served mix of the Cornell box, the dense
// mesh and Cornell variants +3.7%, while the batched
// Cornell variants alone keep 7 (9 blocks: -3.6%; 8 blocks: -3.7%).
static LaunchCfg multi_job_occupancy(const WaveTables& t, LaunchCfg cfg)
{
    if (cfg.variant == 0 && t.multi && t.tree == kTreeBinary && cfg.max_scene_bytes >= kDenseSceneBytes)
        cfg.variant = 1;
    return cfg;
}

void launch_trace_render(const WaveTables& t, RayQueueDev rq, const ull* d_n, HitQueueDev hq, ull* hq_n,
                         float* accum, ull* work, int* err, LaunchCfg cfg, cudaStream_t s)
{
    if (misses_in_compaction(t, cfg.ray_order != 0)) cfg.ray_order = 2;
    // A single scene whose binary tree and triangles exceed L2 waits on DRAM:
    // 9 resident blocks (56 registers) hide more of that latency than 8 (64
    // registers), which an L2-resident scene prefers (lattice +0.9%, dense
    // mesh -0.6% at 9).
    if (cfg.variant == 0 && !t.multi && t.tree == kTreeBinary && cfg.l2_bytes > 0 &&
        (int64_t)t.scene0.num_nodes * (int64_t)sizeof(BvhNode) + (int64_t)t.scene0.num_tris * 48 > cfg.l2_bytes)
        cfg.variant = 1;
    cfg = multi_job_occupancy(t, cfg);
#define WF_TRACE(M, B, T)                                                                                   \
    k_trace_render<M, B, T><<<cfg.grid, 128, 0, s>>>(t.scene0, t.job0, t.scenes, t.jobs, rq, d_n, hq, hq_n, \
                                                     accum, work, err, cfg.ray_order)
#define WF_TRACE2(M, T) \
    if (cfg.variant == 1) WF_TRACE(M, 9, T); else WF_TRACE(M, 1, T)
    if (t.tree == kTreeFour) {
        if (t.multi) { WF_TRACE2(true, Traversal4<false>); } else { WF_TRACE2(false, Traversal4<false>); }
    } else {
        if (t.multi) { WF_TRACE2(true, Traversal<false>); } else { WF_TRACE2(false, Traversal<false>); }
    }
#undef WF_TRACE2
#undef WF_TRACE
}

void launch_camera_chunks(const WaveChunk* chunks, const long long* header, const DeviceJob* jobs, RayQueueDev rq,
                          LaunchCfg cfg, cudaStream_t s)
{
    k_camera_chunks<<<cfg.grid, 256, 0, s>>>(chunks, header, jobs, rq);
}

void launch_bounce_end(ull* counters, ull* tally, cudaStream_t s) { k_bounce_end<<<1, 1, 0, s>>>(counters, tally); }

void launch_stream_plan(ull* counters, StreamState* st, int64_t capacity, int64_t* log, int iter, cudaStream_t s)
{
    k_stream_plan<<<1, 1, 0, s>>>(counters, st, capacity, log, iter);
}

void launch_camera_refill(const WaveChunk* chunks, const StreamState* st, const DeviceJob* jobs, RayQueueDev rq,
                          LaunchCfg cfg, cudaStream_t s)
{
    k_camera_refill<<<cfg.grid, 256, 0, s>>>(chunks, st, jobs, rq);
}

void launch_add_floats(float* dst, const float* src, int64_t n, cudaStream_t s)
{
    k_add_floats<<<grid_for(n, 256, 65535), 256, 0, s>>>(dst, src, n);
}

int shade_blocks_per_sm(bool plain)
{
    int a = 0, b = 0;
    cudaError_t e = plain ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&a, k_shade<false, false>, 128, 0)
                          : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&a, k_shade<true, false>, 128, 0);
    if (e == cudaSuccess && plain) {  // the lean instance shares the plain grid
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_shade<false, false, true>, 128, 0);
        if (e == cudaSuccess && b < a) a = b;
        b = 0;
    }
    if (e == cudaSuccess && !plain) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_shade<false, true>, 128, 0);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    const int m = (!plain && b < a) ? b : a;
    return m > 0 ? m : 1;
}

// k_shade walks the hit list with a block-stride loop, every block taking an
// equal share; its grid is therefore one full wave of resident blocks.  A grid
// that is not a multiple of them (16 blocks per SM against 6 resident: 2.67
// waves) leaves a partial last wave whose blocks start late and end late.
// One full wave of resident blocks of a k_shade form: the context's grid
// counts 128-thread blocks; a form with other blocks takes its own from the
// occupancy calculator (fallback: the 128-thread grid scaled to its block),
// computed once per process (the devices of one process are one GPU model).
template <bool M, bool T, bool L, bool G>
static int shade_grid(int grid128)
{
    if (shade_warps<M, T, L, G>() == kShadeWarps) return grid128;
    static int grid = 0;
    if (grid == 0) {
        int dev = 0, sms = 0, occ = 0;
        if (cudaGetDevice(&dev) != cudaSuccess ||
            cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_shade<M, T, L, G>, 32 * shade_warps<M, T, L, G>(),
                                                          0) != cudaSuccess ||
            occ <= 0 || sms <= 0) {
            cudaGetLastError();
            return std::max(1, grid128 * kShadeWarps / shade_warps<M, T, L, G>());
        }
        grid = occ * sms;
    }
    return grid;
}

void launch_shade(const WaveTables& t, RayQueueDev rq, HitQueueDev hq, const ull* hq_n, ShadowQueueDev sh,
                  ull* sh_n, RayQueueDev next, ull* next_n, float* accum, int* err, LaunchCfg cfg, cudaStream_t s)
{
    const int plain_grid = cfg.shade_grid > 0 ? cfg.shade_grid : cfg.grid;
    const int grid = cfg.shade_grid_other > 0 ? cfg.shade_grid_other : cfg.grid;
    // Next rays grouped by octant where the traversal gains more than the
    // grouping costs k_shade: single scenes from kFarFirstTriangles on, waves
    // over a dense scene.
    const bool group = t.multi ? cfg.max_scene_bytes >= kDenseSceneBytes : t.scene0.num_tris >= kFarFirstTriangles;
#define WF_SHADE(M, T, L, GRID)                                                                                   \
    do {                                                                                                          \
        if (group)                                                                                                \
            k_shade<M, T, L, true><<<shade_grid<M, T, L, true>(GRID), 32 * shade_warps<M, T, L, true>(), 0, s>>>( \
                t.scene0, t.job0, t.scenes, t.jobs, rq, hq, hq_n, cfg.ray_order, sh, sh_n, next, next_n, accum,   \
                err);                                                                                             \
        else                                                                                                      \
            k_shade<M, T, L, false><<<shade_grid<M, T, L, false>(GRID), 32 * shade_warps<M, T, L, false>(), 0,    \
                                      s>>>(t.scene0, t.job0, t.scenes, t.jobs, rq, hq, hq_n, cfg.ray_order, sh,   \
                                           sh_n, next, next_n, accum, err);                                       \
    } while (0)
    if (t.multi && cfg.lean_multi)  // every resident scene fits the lean instance
        WF_SHADE(true, false, true, grid);
    else if (t.multi)
        WF_SHADE(true, false, false, grid);
    else if (t.job0.cost_sum_mat)
        WF_SHADE(false, true, false, grid);
    else if (!t.scene0.env_alias_prob && t.scene0.num_textures == 0 && !(t.scene0.directional.intensity > 0.0f))
        WF_SHADE(false, false, true, plain_grid);
    else
        WF_SHADE(false, false, false, plain_grid);
#undef WF_SHADE
}

void launch_compact_hits(const WaveTables& t, RayQueueDev rq, const ull* d_n, HitQueueDev hq, ull* hq_n,
                         float* accum, LaunchCfg cfg, cudaStream_t s)
{
    // only ray-order bounces compact; misses move here for single-job scenes with a map
    if (t.multi)
        k_compact_hits<true, false><<<cfg.grid, 256, 0, s>>>(t.scene0, t.job0, t.scenes, t.jobs, rq, d_n, hq, hq_n,
                                                              accum);
    else if (misses_in_compaction(t, true))
        k_compact_hits<false, true><<<cfg.grid, 256, 0, s>>>(t.scene0, t.job0, t.scenes, t.jobs, rq, d_n, hq, hq_n,
                                                              accum);
    else
        k_compact_hits<false, false><<<cfg.grid, 256, 0, s>>>(t.scene0, t.job0, t.scenes, t.jobs, rq, d_n, hq, hq_n,
                                                               accum);
}

void launch_occluded_render(const WaveTables& t, ShadowQueueDev sh, const ull* sh_n, float* accum, ull* work,
                            int* err, LaunchCfg cfg, cudaStream_t s)
{
    // farther child first where a dense scene's rays are in the queue: single
    // scenes from kFarFirstTriangles on, multi-job waves over a dense scene
    const bool far_first = t.multi ? cfg.max_scene_bytes >= kDenseSceneBytes : t.scene0.num_tris >= kFarFirstTriangles;
    cfg = multi_job_occupancy(t, cfg);
#define WF_OCC(M, B, T)                                                                                       \
    k_occluded_render<M, B, T><<<cfg.grid, 128, 0, s>>>(t.scene0, t.job0, t.scenes, t.jobs, sh, sh_n, accum, work, \
                                                        err)
#define WF_OCC2(M, T) \
    if (cfg.variant == 1) WF_OCC(M, 9, T); else WF_OCC(M, 1, T)
    if (t.tree == kTreeFour) {
        if (t.multi) {
            if (far_first) { WF_OCC2(true, Traversal4Far); } else { WF_OCC2(true, Traversal4<true>); }
        } else if (far_first) { WF_OCC2(false, Traversal4Far); }
        else { WF_OCC2(false, Traversal4<true>); }
    } else if (t.multi) {
        if (far_first) { WF_OCC2(true, TraversalFar); } else { WF_OCC2(true, Traversal<true>); }
    } else if (far_first) {
        WF_OCC2(false, TraversalFar);
    } else {
        WF_OCC2(false, Traversal<true>);
    }
#undef WF_OCC2
#undef WF_OCC
}

void launch_ray_keys(const DeviceScene* scenes, const DeviceJob* jobs, RayQueueDev rq, const ull* d_n,
                     uint64_t* keys, uint32_t* vals, LaunchCfg cfg, cudaStream_t s)
{
    k_ray_keys<<<cfg.grid, 256, 0, s>>>(scenes, jobs, rq, d_n, keys, vals);
}

void launch_ray_keys_raw(int64_t n, const float* ox, const float* oy, const float* oz,
                         const float* dx, const float* dy, const float* dz, const float bmin[3],
                         const float bmax[3], uint64_t* keys, uint32_t* vals, LaunchCfg cfg,
                         cudaStream_t s)
{
    float3 mn = make_float3(bmin[0], bmin[1], bmin[2]);
    float3 ex = make_float3(fmaxf(bmax[0] - bmin[0], 1e-6f), fmaxf(bmax[1] - bmin[1], 1e-6f),
                            fmaxf(bmax[2] - bmin[2], 1e-6f));
    k_ray_keys_raw<<<grid_for(n, 256, cfg.grid), 256, 0, s>>>(n, ox, oy, oz, dx, dy, dz, mn, ex,
                                                             keys, vals);
}

void launch_gather_rays(RayQueueDev in, const uint32_t* perm, const ull* d_n, RayQueueDev out,
                        LaunchCfg cfg, cudaStream_t s)
{
    k_gather_rays<<<cfg.grid, 256, 0, s>>>(in, perm, d_n, out);
}

void launch_type_stats(ShadeColumnsDev c, const ull* d_n, const wf_material* mats, int num_tex,
                       const int64_t* tex_bytes, ull* counts, ull* mem, int* first, LaunchCfg cfg,
                       cudaStream_t s)
{
    k_type_stats<<<cfg.grid, 256, 0, s>>>(c, d_n, mats, num_tex, tex_bytes, counts, mem, first);
}

void launch_policy_keys(ShadeColumnsDev c, const ull* d_n, const wf_material* mats, int policy,
                        const int* type_rank8, const int* cost_rank, const int* tex_rank,
                        int num_tex, int shift, uint64_t* keys, uint32_t* vals, LaunchCfg cfg,
                        cudaStream_t s)
{
    Rank8 r;
    for (int k = 0; k < 8; ++k) r.r[k] = type_rank8[k];
    k_policy_keys<<<cfg.grid, 256, 0, s>>>(c, d_n, mats, policy, r, cost_rank, tex_rank, num_tex,
                                           shift, keys, vals);
}

void launch_cb_reduce(ShadeColumnsDev c, const ull* d_n, double* benefit, int* present,
                      unsigned* bounds6, int num_materials, LaunchCfg cfg, cudaStream_t s)
{
    const size_t shm = num_materials <= kCbSharedMaterials ? sizeof(double) * (size_t)num_materials : 0;
    k_cb_reduce<<<cfg.grid, 256, shm, s>>>(c, d_n, benefit, present, bounds6, num_materials);
}

void launch_cb_keys(ShadeColumnsDev c, const ull* d_n, const wf_material* mats,
                    const int* prio_rank, int prio_bits, const unsigned* bounds6, uint64_t* keys,
                    uint32_t* vals, LaunchCfg cfg, cudaStream_t s)
{
    k_cb_keys<<<cfg.grid, 256, 0, s>>>(c, d_n, mats, prio_rank, prio_bits, bounds6, keys, vals);
}

void launch_hit_columns(const DeviceScene* scenes, const DeviceJob* jobs, const DeviceScene* scene, bool full,
                        RayQueueDev rq, HitQueueDev hq, const ull* d_n, ShadeColumnsMut out, LaunchCfg cfg,
                        cudaStream_t s)
{
    if (full)
        k_hit_columns<true><<<cfg.grid, 256, 0, s>>>(scenes, jobs, scene, rq, hq, d_n, out);
    else
        k_hit_columns<false><<<cfg.grid, 256, 0, s>>>(scenes, jobs, scene, rq, hq, d_n, out);
}

void launch_permute_hits(HitQueueDev in, const uint32_t* perm, const ull* d_n, HitQueueDev out,
                         LaunchCfg cfg, cudaStream_t s)
{
    k_permute_hits<<<cfg.grid, 256, 0, s>>>(in, perm, d_n, out);
}

void launch_finalize(const float* accum, int64_t n, float spp, float* image, cudaStream_t s)
{
    k_finalize<<<grid_for(n, 256, 65535), 256, 0, s>>>(accum, n, spp, image);
}

void launch_cost_update(const CostTrackerDev& mat, const CostTrackerDev& tex, int repeat, cudaStream_t s)
{
    k_cost_update<<<2, 32, 0, s>>>(mat, tex, repeat);
}

void launch_adaptive_fold(float* sample_buf, int64_t np, int nspp, int slot0, int wave_spp, float* accum,
                          float* mean, float* m2, int32_t* count, const int32_t* active, int32_t n_active,
                          cudaStream_t s)
{
    if (n_active <= 0) return;
    k_adaptive_fold<<<grid_for(n_active, 256, 65535), 256, 0, s>>>(sample_buf, np, nspp, slot0, wave_spp, accum,
                                                                   mean, m2, count, active, n_active);
}

void launch_adaptive_check(const float* mean, const float* m2, const int32_t* count, const int32_t* active,
                           int32_t n_active, float threshold, int32_t* flag, cudaStream_t s)
{
    if (n_active <= 0) return;
    k_adaptive_check<<<grid_for(n_active, 256, 65535), 256, 0, s>>>(mean, m2, count, active, n_active, threshold,
                                                                    flag);
}

void launch_compact_active(const int32_t* flag, int64_t np, int32_t* pos, int32_t* block_sums, int32_t* out,
                           int32_t* n_out, cudaStream_t s)
{
    exclusive_scan_i32(flag, (int)np, pos, block_sums, n_out, s);
    k_scatter_active<<<grid_for(np, 256, 65535), 256, 0, s>>>(flag, pos, np, out);
}

void launch_finalize_counts(const float* accum, const int32_t* count, int64_t np, float* image, cudaStream_t s)
{
    k_finalize_counts<<<grid_for(3 * np, 256, 65535), 256, 0, s>>>(accum, count, np, image);
}

void launch_fill_i32(int32_t* a, int64_t n, int32_t v, bool identity, cudaStream_t s)
{
    k_fill_i32<<<grid_for(n, 256, 65535), 256, 0, s>>>(a, n, v, identity ? 1 : 0);
}

void launch_split_hits(const WaveTables& t, RayQueueDev rq, const ull* d_n, HitQueueDev hq, ull* hq_n,
                       uint32_t* miss_list, ull* miss_n, LaunchCfg cfg, cudaStream_t s)
{
    k_compact_hits<false, false><<<cfg.grid, 256, 0, s>>>(t.scene0, t.job0, t.scenes, t.jobs, rq, d_n, hq, hq_n,
                                                           nullptr);
    k_list_misses<<<cfg.grid, 256, 0, s>>>(hq.tri, d_n, miss_list, miss_n);
}

void launch_miss_queue(const WaveTables& t, RayQueueDev misses, const ull* d_n, float* accum, LaunchCfg cfg,
                       cudaStream_t s)
{
    k_miss_queue<<<cfg.grid, 256, 0, s>>>(t.scene0, t.job0, misses, d_n, accum);
}

void launch_materialize_hits(HitQueueDev in, bool at_ray, const uint32_t* perm, const ull* d_n, HitQueueDev out,
                             LaunchCfg cfg, cudaStream_t s)
{
    k_materialize_hits<<<cfg.grid, 256, 0, s>>>(in, at_ray ? 1 : 0, perm, d_n, out);
}

void launch_shading_columns(const DeviceScene& S, RayQueueDev rq, HitQueueDev hq, bool at_ray, const ull* d_n,
                            HitColumnsDev out, RayQueueDev rays_out, LaunchCfg cfg, cudaStream_t s)
{
    k_shading_columns<<<cfg.grid, 256, 0, s>>>(S, rq, hq, at_ray ? 1 : 0, d_n, out, rays_out);
}

}  // namespace wf
