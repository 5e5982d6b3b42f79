// Stand-in for <tbb/tbb.h> used only when the reference OptCuts core is
// compiled as the oracle.  The reference calls exactly one TBB entry point,
// tbb::parallel_for(int first, int last, int step, F body) (e.g.
// src/Energy/SymDirichletEnergy.cpp:317, src/TriMesh.cpp:686), and no
// arithmetic lives inside TBB.  Every call site writes disjoint per-index
// slots, so a std::thread fan-out over contiguous chunks gives the same
// results as TBB's work stealing.
//
// OC_REF_THREADS (environment) sets the thread count; default: all cores.
#ifndef OC_ORACLE_TBB_SHIM_H
#define OC_ORACLE_TBB_SHIM_H

#include <algorithm>
#include <cstdlib>
#include <thread>
#include <vector>

namespace tbb {

inline int oc_shim_threads()
{
    static int n = [] {
        const char* e = std::getenv("OC_REF_THREADS");
        int v = e ? std::atoi(e) : 0;
        if (v <= 0) v = static_cast<int>(std::thread::hardware_concurrency());
        return v > 0 ? v : 1;
    }();
    return n;
}

template <typename Index, typename Body>
void parallel_for(Index first, Index last, Index step, const Body& body)
{
    if (last <= first) return;
    const long long count = (static_cast<long long>(last) - first + step - 1) / step;
    const int nt = static_cast<int>(std::min<long long>(oc_shim_threads(), count));
    if (nt <= 1) {
        for (Index i = first; i < last; i += step) body(i);
        return;
    }
    std::vector<std::thread> pool;
    pool.reserve(nt);
    for (int t = 0; t < nt; ++t) {
        const long long b = count * t / nt, e = count * (t + 1) / nt;
        pool.emplace_back([=, &body] {
            for (long long k = b; k < e; ++k) body(static_cast<Index>(first + k * step));
        });
    }
    for (auto& th : pool) th.join();
}

} // namespace tbb

#endif
