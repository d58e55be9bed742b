/*
 * Stand-in for Intel TBB's tbb::parallel_for(first, last, f), used by the
 * reference's +mex/source/das_c.cpp:358.  TEST INFRASTRUCTURE ONLY.
 *
 * Work is handed out in chunks from an atomic counter to
 * std::thread::hardware_concurrency() threads (or USTB_REF_THREADS when set).
 * das_c's body writes only the outputs of its own pixel, so any schedule gives
 * the same bits.
 */
#ifndef USTB_ORACLE_TBB_SHIM_H
#define USTB_ORACLE_TBB_SHIM_H

#include <algorithm>
#include <atomic>
#include <cstdlib>
#include <thread>
#include <vector>

namespace tbb {

inline int ustb_shim_threads() {
    const char* e = std::getenv("USTB_REF_THREADS");
    int n = e ? std::atoi(e) : 0;
    if (n <= 0) n = (int)std::thread::hardware_concurrency();
    return n > 0 ? n : 1;
}

template <class Index, class Func>
void parallel_for(Index first, Index last, const Func& f) {
    const Index n = last - first;
    if (n <= 0) return;
    const int nt = std::min<long long>(ustb_shim_threads(), (long long)n);
    const Index chunk = std::max<Index>(1, n / (Index)(nt * 16));
    std::atomic<long long> next(first);
    auto worker = [&]() {
        for (;;) {
            long long b = next.fetch_add(chunk);
            if (b >= (long long)last) break;
            Index e = (Index)std::min<long long>(b + chunk, (long long)last);
            for (Index i = (Index)b; i < e; ++i) f(i);
        }
    };
    if (nt == 1) { worker(); return; }
    std::vector<std::thread> ts;
    ts.reserve(nt - 1);
    for (int t = 0; t < nt - 1; ++t) ts.emplace_back(worker);
    worker();
    for (auto& t : ts) t.join();
}

}  // namespace tbb

#endif
