// Shim for oneTBB's combinable: one lazily built T per worker; combine_each
// visits them in worker order.
#pragma once
#include <functional>
#include <memory>
#include <vector>

#include "wf_workers.h"

namespace tbb {
template <class T>
class combinable {
  public:
    combinable() : init_([] { return T(); }) { slots_.resize(64); }
    template <class F>
    explicit combinable(F f) : init_(f) { slots_.resize(64); }
    T& local()
    {
        auto& s = slots_[wfshim::worker_index()];
        if (!s) s.reset(new T(init_()));
        return *s;
    }
    template <class F>
    void combine_each(F f)
    {
        for (auto& s : slots_)
            if (s) f(*s);
    }

  private:
    std::function<T()> init_;
    std::vector<std::unique_ptr<T>> slots_;
};
}  // namespace tbb
