// Shim for oneTBB's parallel_for: a fixed number of std::threads; worker t
// takes chunks t, t+W, t+2W, ... (static, so a run is reproducible).  Chunk
// boundaries are multiples of the range's grain size, as TBB's splitting
// keeps them for the reference's power-of-two-sized ranges.
#pragma once
#include <thread>
#include <vector>

#include "blocked_range.h"
#include "wf_workers.h"

namespace tbb {
template <class T, class Body>
void parallel_for(const blocked_range<T>& r, const Body& body)
{
    const int nw = wfshim::num_workers();
    const long long n = (long long)(r.end() - r.begin());
    if (n <= 0) return;
    const long long g = (long long)r.grainsize();
    long long chunk = (n + 4LL * nw - 1) / (4LL * nw);
    chunk = ((chunk + g - 1) / g) * g;
    if (chunk < g) chunk = g;
    const long long nchunks = (n + chunk - 1) / chunk;
    auto run = [&](int w) {
        wfshim::worker_index() = w;
        for (long long c = w; c < nchunks; c += nw) {
            T b = (T)(r.begin() + c * chunk);
            T e = (T)((c + 1) * chunk < n ? r.begin() + (c + 1) * chunk : r.end());
            body(blocked_range<T>(b, e, r.grainsize()));
        }
    };
    std::vector<std::thread> pool;
    for (int w = 1; w < nw; ++w) pool.emplace_back(run, w);
    run(0);
    for (auto& t : pool) t.join();
    wfshim::worker_index() = 0;
}
}  // namespace tbb
