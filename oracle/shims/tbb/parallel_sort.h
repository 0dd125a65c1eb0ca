// Shim for oneTBB's parallel_sort: std::stable_sort, i.e. the reference's
// comparator with ties kept in index order.
#pragma once
#include <algorithm>
// The real oneTBB headers pull these in; the reference relies on it
// (ShadingQueue.h uses std::unordered_map without including it).
#include <functional>
#include <string>
#include <unordered_map>

namespace tbb {
template <class It, class Cmp>
void parallel_sort(It b, It e, const Cmp& cmp)
{
    std::stable_sort(b, e, cmp);
}
}  // namespace tbb
