// wf_sort.cu — stable LSD radix sort of (uint64 key, uint32 value) pairs.
//
// Used for the BVH Morton order, the RayQueue sort (RayQueue::schedule,
// reference include/scheduling/RayQueue.h:165-179) and the ShadingQueue
// policy sorts (ShadingQueue.h:90-141, 437-510).  Stability matters: the
// reference comparators tie often, and a stable sort of the policy key gives
// exactly the permutation std::stable_sort gives with the reference
// comparator.
//
// One pass per 8-bit digit:
//   hist    — each block counts the digits of its contiguous chunk
//   scan    — the [digit][block] counts become offsets (multi-block scan)
//   scatter — each block walks its chunk in tiles of 2048 keys; a key's rank
//             among equal digits comes from __match_any_sync within a warp
//             and per-digit prefixes across warps and rounds, so order within
//             a digit follows input order (stable); the tile is staged
//             digit-sorted in shared memory and written out in runs.
// The element count is read from device memory, so a pass can be launched
// (and graph-captured) before the count is known on the host.
#include "wf_sort.h"

#include <cuda_runtime.h>

namespace wf {

namespace {

constexpr int kTile = 256;  // threads per block = keys per tile
constexpr int kDigits = 256;

__device__ __forceinline__ void chunk_of(int64_t n, int nb, int b, int64_t& start, int64_t& end)
{
    int64_t per = (n + nb - 1) / nb;
    per = (per + kTile - 1) / kTile * kTile;
    start = (int64_t)b * per;
    end = start + per;
    if (end > n) end = n;
    if (start > n) start = n;
}

__global__ void __launch_bounds__(kTile) k_hist(const uint64_t* __restrict__ keys,
                                                const unsigned long long* __restrict__ d_n,
                                                int shift, uint32_t* __restrict__ hist, int nb)
{
    __shared__ uint32_t h[kDigits];
    h[threadIdx.x] = 0;
    __syncthreads();
    int64_t start, end;
    chunk_of((int64_t)*d_n, nb, blockIdx.x, start, end);
    // one shared atomic per distinct digit of a warp: policy keys use a few
    // digits, and lanes adding to one counter would queue behind each other
    const unsigned lt = (1u << (threadIdx.x & 31)) - 1u;
    for (int64_t b = start; b < end; b += kTile) {
        const int64_t i = b + threadIdx.x;
        const bool valid = i < end;
        const unsigned vmask = __ballot_sync(0xFFFFFFFFu, valid);
        if (valid) {
            const uint32_t d = (uint32_t)(__ldg(keys + i) >> shift) & 0xFFu;
            const unsigned peers = __match_any_sync(vmask, d);
            if ((peers & lt) == 0u) atomicAdd(&h[d], (uint32_t)__popc(peers));
        }
    }
    __syncthreads();
    hist[(int64_t)threadIdx.x * nb + blockIdx.x] = h[threadIdx.x];
}

constexpr int kItems = 8;                   // keys per thread per tile
constexpr int kTileKeys = kTile * kItems;   // 2048 keys staged per tile

// Exclusive scan of v over the 256 threads of a block (thread = digit).
__device__ __forceinline__ uint32_t block_exclusive_scan256(uint32_t v, uint32_t* warp_sums)
{
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t u = __shfl_up_sync(0xFFFFFFFFu, x, o);
        if (lane >= o) x += u;
    }
    if (lane == 31) warp_sums[w] = x;
    __syncthreads();
    uint32_t before = 0;
    for (int k = 0; k < w; ++k) before += warp_sums[k];
    __syncthreads();
    return before + x - v;
}

// Scatter of one digit pass.  A tile of 2048 keys: warp w ranks the 256 keys
// [base + 256 w, base + 256 w + 256) in 8 rounds of 32 (coalesced loads); a
// key's rank among its warp's equal digits comes from __match_any_sync and a
// per-warp digit count in shared memory, updated warp-synchronously (no block
// barrier per round).  Then per digit an exclusive scan over the 8 warps and
// one over the 256 digits place every key in the tile, staged digit-sorted in
// shared memory and written out as one contiguous run per digit, so the
// global writes coalesce.  Stable: within a digit, keys keep their input
// order (warp, round, lane).  Six block barriers per tile; ranking every
// round across the block took thirty-seven.  Six resident blocks per SM (40
// registers; at 64 only four fit, and the grid of six per SM ran in 1.5
// waves).
__global__ void __launch_bounds__(kTile, 6) k_scatter(const uint64_t* __restrict__ kin,
                                                   const uint32_t* __restrict__ vin,
                                                   uint64_t* __restrict__ kout,
                                                   uint32_t* __restrict__ vout,
                                                   const unsigned long long* __restrict__ d_n,
                                                   int shift, const uint32_t* __restrict__ offs,
                                                   int nb)
{
    constexpr int kWarps = kTile / 32;
    __shared__ uint32_t running[kDigits];
    __shared__ uint32_t tile_start[kDigits];
    __shared__ uint32_t wcnt[kWarps][kDigits];  // per-warp digit counts, then the warp's offsets
    __shared__ uint32_t warp_sums[kWarps];
    __shared__ uint64_t skey[kTileKeys];
    __shared__ uint32_t sval[kTileKeys];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const unsigned lt = (1u << lane) - 1u;
    running[tid] = offs[(int64_t)tid * nb + blockIdx.x];
    int64_t start, end;
    chunk_of((int64_t)*d_n, nb, blockIdx.x, start, end);
    for (int64_t base = start; base < end; base += kTileKeys) {
        for (int d = lane; d < kDigits; d += 32) wcnt[warp][d] = 0;  // this warp's row
        __syncwarp();
        uint64_t key[kItems];
        uint32_t val[kItems], rank[kItems];
        const int64_t wbase = base + (int64_t)warp * 32 * kItems;
#pragma unroll
        for (int r = 0; r < kItems; ++r) {
            const int64_t i = wbase + (int64_t)r * 32 + lane;
            const bool valid = i < end;
            const unsigned vmask = __ballot_sync(0xFFFFFFFFu, valid);
            key[r] = 0;
            val[r] = 0;
            rank[r] = 0;
            if (valid) {
                key[r] = kin[i];
                val[r] = vin[i];
                const uint32_t digit = (uint32_t)(key[r] >> shift) & 0xFFu;
                const unsigned peers = __match_any_sync(vmask, digit);
                const uint32_t before = wcnt[warp][digit];
                rank[r] = before + (uint32_t)__popc(peers & lt);
                __syncwarp(vmask);  // every peer has read the count
                if ((peers & lt) == 0u) wcnt[warp][digit] = before + (uint32_t)__popc(peers);
            }
            __syncwarp();
        }
        __syncthreads();
        // thread = digit: the warps' offsets within the digit, the digit's total
        uint32_t tot = 0;
#pragma unroll
        for (int w = 0; w < kWarps; ++w) {
            const uint32_t c = wcnt[w][tid];
            wcnt[w][tid] = tot;
            tot += c;
        }
        const uint32_t first = block_exclusive_scan256(tot, warp_sums);
        tile_start[tid] = first;
        __syncthreads();
#pragma unroll
        for (int r = 0; r < kItems; ++r) {
            if (wbase + (int64_t)r * 32 + lane < end) {
                const uint32_t d = (uint32_t)(key[r] >> shift) & 0xFFu;
                const uint32_t pos = tile_start[d] + wcnt[warp][d] + rank[r];
                skey[pos] = key[r];
                sval[pos] = val[r];
            }
        }
        __syncthreads();
        const int tile_n = (int)min((int64_t)kTileKeys, end - base);
        for (int idx = tid; idx < tile_n; idx += kTile) {
            const uint64_t k = skey[idx];
            const uint32_t d = (uint32_t)(k >> shift) & 0xFFu;
            const uint32_t gpos = running[d] + (uint32_t)idx - tile_start[d];
            kout[gpos] = k;
            vout[gpos] = sval[idx];
        }
        __syncthreads();
        running[tid] += tot;
    }
}

__global__ void k_iota(uint32_t* __restrict__ v, const unsigned long long* __restrict__ d_n)
{
    const int64_t n = (int64_t)*d_n;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
        v[i] = (uint32_t)i;
}

}  // namespace

int radix_blocks_for(int64_t capacity, int num_sms)
{
    // Enough blocks to fill the GPU, few enough that the scan stays cheap
    // (256 * nb counts) and each chunk is at least a few tiles.
    int64_t want = (capacity + 4 * kTile - 1) / (4 * kTile);
    int64_t cap = (int64_t)num_sms * 6;
    if (want > cap) want = cap;
    if (want > 1024) want = 1024;
    if (want < 1) want = 1;
    return (int)want;
}

size_t radix_hist_words(int nb) { return radix_hist_words_for(nb); }

void radix_sort_pairs(RadixSortArgs a, cudaStream_t s)
{
    uint64_t* kin = a.keys;
    uint32_t* vin = a.vals;
    uint64_t* kout = a.keys_tmp;
    uint32_t* vout = a.vals_tmp;
    for (int shift = a.begin_bit; shift < a.end_bit; shift += 8) {
        k_hist<<<a.nb, kTile, 0, s>>>(kin, a.d_n, shift, a.hist, a.nb);
        {   // [digit][block] counts -> offsets (multi-block scan)
            int* counts = reinterpret_cast<int*>(a.hist);
            int* block_sums = counts + kDigits * a.nb;
            int* total = block_sums + ((kDigits * a.nb + 1023) / 1024 + 1);
            exclusive_scan_i32(counts, kDigits * a.nb, counts, block_sums, total, s);
        }
        k_scatter<<<a.nb, kTile, 0, s>>>(kin, vin, kout, vout, a.d_n, shift, a.hist, a.nb);
        uint64_t* tk = kin;
        kin = kout;
        kout = tk;
        uint32_t* tv = vin;
        vin = vout;
        vout = tv;
    }
    *a.result_keys = kin;
    *a.result_vals = vin;
}

void launch_iota(uint32_t* v, const unsigned long long* d_n, int grid, cudaStream_t s)
{
    k_iota<<<grid, 256, 0, s>>>(v, d_n);
}

namespace {

// Exclusive scan of n ints (three passes: per-block scans of 1024, one block
// scanning the block totals, then the carries); *total gets the sum.  In and
// out may be the same array (each thread reads its element before writing).
__global__ void __launch_bounds__(1024) k_scan_blocks(const int* in, int n, int* out, int* __restrict__ block_sums)
{
    __shared__ int warp_incl[32];
    const int i = blockIdx.x * 1024 + threadIdx.x;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int v = i < n ? in[i] : 0;
    int x = v;
    for (int o = 1; o < 32; o <<= 1) {
        const int u = __shfl_up_sync(0xFFFFFFFFu, x, o);
        if (lane >= o) x += u;
    }
    if (lane == 31) warp_incl[w] = x;
    __syncthreads();
    if (w == 0) {
        int y = warp_incl[lane];
        for (int o = 1; o < 32; o <<= 1) {
            const int u = __shfl_up_sync(0xFFFFFFFFu, y, o);
            if (lane >= o) y += u;
        }
        warp_incl[lane] = y;
    }
    __syncthreads();
    const int excl = x - v + (w > 0 ? warp_incl[w - 1] : 0);
    if (i < n) out[i] = excl;
    if (threadIdx.x == 0) block_sums[blockIdx.x] = warp_incl[31];
}

__global__ void __launch_bounds__(1024) k_scan_sums(int* __restrict__ sums, int nb, int* __restrict__ total)
{
    __shared__ int warp_incl[32];
    __shared__ int carry;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int t0 = 0; t0 < nb; t0 += 1024) {
        const int i = t0 + threadIdx.x;
        const int v = i < nb ? sums[i] : 0;
        int x = v;
        for (int o = 1; o < 32; o <<= 1) {
            const int u = __shfl_up_sync(0xFFFFFFFFu, x, o);
            if (lane >= o) x += u;
        }
        if (lane == 31) warp_incl[w] = x;
        __syncthreads();
        if (w == 0) {
            int y = warp_incl[lane];
            for (int o = 1; o < 32; o <<= 1) {
                const int u = __shfl_up_sync(0xFFFFFFFFu, y, o);
                if (lane >= o) y += u;
            }
            warp_incl[lane] = y;
        }
        __syncthreads();
        const int excl = x - v + (w > 0 ? warp_incl[w - 1] : 0);
        if (i < nb) sums[i] = carry + excl;
        __syncthreads();
        if (threadIdx.x == 0) carry += warp_incl[31];
        __syncthreads();
    }
    if (threadIdx.x == 0) *total = carry;
}

__global__ void k_scan_add(int* __restrict__ out, int n, const int* __restrict__ sums)
{
    const int i = blockIdx.x * 1024 + threadIdx.x;
    if (i < n) out[i] += sums[blockIdx.x];
}

}  // namespace

void exclusive_scan_i32(const int* in, int n, int* out, int* block_sums, int* total, cudaStream_t s)
{
    const int nb = (n + 1023) / 1024;
    k_scan_blocks<<<nb, 1024, 0, s>>>(in, n, out, block_sums);
    k_scan_sums<<<1, 1024, 0, s>>>(block_sums, nb, total);
    k_scan_add<<<nb, 1024, 0, s>>>(out, n, block_sums);
}

}  // namespace wf
