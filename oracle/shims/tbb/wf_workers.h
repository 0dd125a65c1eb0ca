// Worker bookkeeping shared by the TBB and Random shims.
#pragma once

namespace wfshim {
int num_workers();
void set_num_workers(int n);
inline int& worker_index()
{
    thread_local int w = 0;
    return w;
}
}  // namespace wfshim
