/*
 * Row partitioning shared by the oracle's batch runners (TEST INFRASTRUCTURE ONLY).
 */
#ifndef PGX_ORACLE_ROWS_HPP
#define PGX_ORACLE_ROWS_HPP
#include <cstdint>
#include <thread>
#include <vector>

namespace orc_detail
{

inline int resolve_threads(int nthreads)
{
    if (nthreads > 0) return nthreads;
    unsigned h = std::thread::hardware_concurrency();
    return h ? static_cast<int>(h) : 1;
}

// Static partition of [0, n) over nthreads std::threads (the stand-in for the
// TBB parallel_for of src/batch_evaluators/thread_bfe.cpp:125-137).
template <typename F>
inline void parallel_rows(uint64_t n, int nthreads, F &&body)
{
    uint64_t nt = static_cast<uint64_t>(resolve_threads(nthreads));
    if (nt > n) nt = n;
    if (nt <= 1u) {
        if (n) body(uint64_t(0), n);
        return;
    }
    std::vector<std::thread> pool;
    const uint64_t chunk = n / nt, rem = n % nt;
    uint64_t b = 0;
    for (uint64_t t = 0; t < nt; ++t) {
        const uint64_t e = b + chunk + (t < rem ? 1u : 0u);
        pool.emplace_back([&body, b, e]() { body(b, e); });
        b = e;
    }
    for (auto &th : pool) th.join();
}

} // namespace orc_detail

#endif
