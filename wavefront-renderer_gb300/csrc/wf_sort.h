// wf_sort.h — launchers of the stable device radix sort (wf_sort.cu).
#pragma once

#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

namespace wf {

struct RadixSortArgs {
    uint64_t* keys;      // input keys (overwritten)
    uint32_t* vals;      // input values (overwritten)
    uint64_t* keys_tmp;  // ping-pong buffers, same capacity
    uint32_t* vals_tmp;
    uint32_t* hist;      // radix_hist_words(nb) words
    const unsigned long long* d_n;  // element count, device memory
    int nb;              // blocks per pass (radix_blocks_for)
    int begin_bit;       // sort bits [begin_bit, end_bit), 8 per pass
    int end_bit;
    uint64_t** result_keys;  // set to the buffer holding the sorted keys
    uint32_t** result_vals;
};

// Kernels per 8-bit pass: digit counts, the three-kernel offset scan, scatter.
constexpr int kSortKernelsPerPass = 5;

int radix_blocks_for(int64_t capacity, int num_sms);
// Scratch of one sort: 256 digit counts per block plus the scan's block
// totals and its total.
constexpr size_t radix_hist_words_for(int nb)
{
    return (size_t)256 * nb + ((size_t)256 * nb + 1023) / 1024 + 2;
}
size_t radix_hist_words(int nb);
void radix_sort_pairs(RadixSortArgs args, cudaStream_t stream);
void launch_iota(uint32_t* v, const unsigned long long* d_n, int grid, cudaStream_t stream);

// Exclusive prefix sum of n ints (n > 0): per-block scans of 1024, one block
// over the block totals, then the carries.  block_sums needs
// scan_block_words(n) ints; *total (device) receives the sum.
void exclusive_scan_i32(const int* in, int n, int* out, int* block_sums, int* total, cudaStream_t stream);
inline int scan_block_words(int64_t n) { return (int)((n + 1023) / 1024) + 1; }

}  // namespace wf
