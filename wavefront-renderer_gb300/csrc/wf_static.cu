// wf_static.cu — the RayQueue sort for callers that cannot allocate device
// memory.
//
// Who needs it: code that must not call cudaMalloc / cudaFree while it runs —
// a renderer embedded in another framework that owns the device heap, a
// real-time loop with a no-allocation rule, or code that sets up work while a
// stream is being captured.  They own their input and output buffers already;
// what the sort needs beyond them (keys, values, their ping-pong copies, the
// digit histogram, the element count) lives here in one file-scope __device__
// array, sized for WF_STATIC_SCHEDULE_MAX_RAYS rays.  Every GPU that loads the
// library holds this array (~25 MB) until the process exits.
//
// The kernels are the ones wf_ray_schedule_host runs (RayQueue::sortKey keys,
// the stable radix sort); only the storage differs.
#include <cuda_runtime.h>

#include <mutex>

#include "../../include/wf_api.h"
#include "wf_kernels.h"
#include "wf_sort.h"

namespace {

constexpr int64_t kMaxRays = WF_STATIC_SCHEDULE_MAX_RAYS;
constexpr int kMaxSortBlocks = 1024;  // radix_blocks_for never exceeds this
constexpr size_t kAlign = 256;
constexpr size_t align_up(size_t x) { return (x + kAlign - 1) / kAlign * kAlign; }
constexpr size_t kOffKeys = 0;
constexpr size_t kOffKeysTmp = align_up(kOffKeys + sizeof(uint64_t) * kMaxRays);
constexpr size_t kOffVals = align_up(kOffKeysTmp + sizeof(uint64_t) * kMaxRays);
constexpr size_t kOffValsTmp = align_up(kOffVals + sizeof(uint32_t) * kMaxRays);
constexpr size_t kOffHist = align_up(kOffValsTmp + sizeof(uint32_t) * kMaxRays);
constexpr size_t kOffCount = align_up(kOffHist + sizeof(uint32_t) * wf::radix_hist_words_for(kMaxSortBlocks));
constexpr size_t kScratchBytes = align_up(kOffCount + sizeof(unsigned long long));

// The scratch.  In host code this name is only a host-side stand-in for the
// device symbol: its device address comes from cudaGetSymbolAddress below.
static __device__ __align__(256) unsigned char g_schedule_scratch[kScratchBytes];

struct DeviceSetup {
    bool ready = false;
    unsigned char* base = nullptr;  // device address of g_schedule_scratch
    int num_sms = 0;
};
constexpr int kMaxDevices = 64;
DeviceSetup g_setup[kMaxDevices];
std::mutex g_setup_mu;

__global__ void k_store_count(unsigned long long* count, unsigned long long n) { *count = n; }

__global__ void k_emit_permutation(const uint32_t* __restrict__ vals, int32_t* __restrict__ out, int64_t n)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        out[i] = (int32_t)vals[i];
}

// Once per device, with that device current: the array's device address.
int setup_current_device(DeviceSetup** out)
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return WF_ERR_CUDA;
    if (dev < 0 || dev >= kMaxDevices) return WF_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lock(g_setup_mu);
    DeviceSetup& s = g_setup[dev];
    if (!s.ready) {
        void* p = nullptr;
        if (cudaGetSymbolAddress(&p, g_schedule_scratch) != cudaSuccess || p == nullptr) return WF_ERR_CUDA;
        int sms = 0;
        if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0)
            return WF_ERR_CUDA;
        s.base = static_cast<unsigned char*>(p);
        s.num_sms = sms;
        s.ready = true;
    }
    *out = &s;
    return WF_OK;
}

}  // namespace

extern "C" int wf_ray_schedule_static(void* stream, int64_t n, const float* ox, const float* oy,
                                      const float* oz, const float* dx, const float* dy, const float* dz,
                                      const float bounds_min[3], const float bounds_max[3],
                                      int32_t* out_sorted_indices, uint64_t* out_keys)
{
    if (n < 0 || !bounds_min || !bounds_max) return WF_ERR_INVALID_ARGUMENT;
    if (n > kMaxRays) return WF_ERR_CAPACITY;  // beyond the static scratch
    if (n > 0 && (!ox || !oy || !oz || !dx || !dy || !dz || !out_sorted_indices)) return WF_ERR_INVALID_ARGUMENT;
    // An error left pending by earlier work on this thread stays the caller's:
    // report it without clearing it, and enqueue nothing.
    if (cudaPeekAtLastError() != cudaSuccess) return WF_ERR_CUDA;
    DeviceSetup* dev = nullptr;
    int rc = setup_current_device(&dev);
    if (rc != WF_OK) return rc;
    if (n == 0) return WF_OK;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    uint64_t* keys = reinterpret_cast<uint64_t*>(dev->base + kOffKeys);
    uint64_t* keys_tmp = reinterpret_cast<uint64_t*>(dev->base + kOffKeysTmp);
    uint32_t* vals = reinterpret_cast<uint32_t*>(dev->base + kOffVals);
    uint32_t* vals_tmp = reinterpret_cast<uint32_t*>(dev->base + kOffValsTmp);
    uint32_t* hist = reinterpret_cast<uint32_t*>(dev->base + kOffHist);
    unsigned long long* count = reinterpret_cast<unsigned long long*>(dev->base + kOffCount);
    const int nb = wf::radix_blocks_for(n, dev->num_sms);
    if (nb > kMaxSortBlocks) return WF_ERR_CAPACITY;
    // Keys, values and histogram are overwritten in full by every call; only
    // the element count has to be stored first.
    k_store_count<<<1, 1, 0, s>>>(count, (unsigned long long)n);
    wf::launch_ray_keys_raw(n, ox, oy, oz, dx, dy, dz, bounds_min, bounds_max, keys, vals,
                            wf::LaunchCfg{dev->num_sms * 8, 256}, s);
    if (cudaGetLastError() != cudaSuccess) return WF_ERR_CUDA;
    if (out_keys && cudaMemcpyAsync(out_keys, keys, sizeof(uint64_t) * (size_t)n, cudaMemcpyDeviceToDevice, s) !=
                        cudaSuccess)
        return WF_ERR_CUDA;
    uint64_t* rk = nullptr;
    uint32_t* rv = nullptr;
    wf::RadixSortArgs a{keys, vals, keys_tmp, vals_tmp, hist, count, nb, 0, 33, &rk, &rv};
    wf::radix_sort_pairs(a, s);
    if (cudaGetLastError() != cudaSuccess) return WF_ERR_CUDA;
    int grid = (int)((n + 255) / 256);
    if (grid > dev->num_sms * 8) grid = dev->num_sms * 8;
    k_emit_permutation<<<grid, 256, 0, s>>>(rv, out_sorted_indices, n);
    return cudaGetLastError() == cudaSuccess ? WF_OK : WF_ERR_CUDA;
}
