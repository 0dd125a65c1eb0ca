// Shim for the reference's include/math/Random.h: same randomFloat() API, but
// each worker of the TBB shim owns an std::mt19937 that a test can reseed, so
// batches of an oracle render are independent and reproducible.
#pragma once
#include <random>

#include "../tbb/wf_workers.h"

namespace wfshim {
std::mt19937& worker_rng();
void set_seed(unsigned long long seed);
}  // namespace wfshim

inline std::mt19937& getThreadRNG() { return wfshim::worker_rng(); }

inline float randomFloat()
{
    std::uniform_real_distribution<float> dist(0.0f, 1.0f);
    return dist(wfshim::worker_rng());
}
