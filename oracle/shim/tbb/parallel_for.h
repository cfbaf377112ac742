// tbb::parallel_for stand-in: splits the range into one contiguous chunk per
// hardware thread (std::thread::hardware_concurrency(), or PGX_REF_THREADS if
// set) and runs the body on each chunk. TBB proper uses work stealing over
// finer chunks; for the uniform-cost rows of a batch fitness evaluation a
// static partition is equivalent.
#ifndef PGX_SHIM_TBB_PARALLEL_FOR_H
#define PGX_SHIM_TBB_PARALLEL_FOR_H
#include <cstdlib>
#include <exception>
#include <thread>
#include <vector>
#include "blocked_range.h"
namespace tbb
{
inline unsigned shim_thread_count()
{
    if (const char *s = std::getenv("PGX_REF_THREADS")) {
        const int v = std::atoi(s);
        if (v > 0) return static_cast<unsigned>(v);
    }
    const unsigned h = std::thread::hardware_concurrency();
    return h ? h : 1u;
}
template <typename T, typename Body>
inline void parallel_for(const blocked_range<T> &r, const Body &body)
{
    const T n = r.end() - r.begin();
    if (n == T(0)) return;
    T nt = static_cast<T>(shim_thread_count());
    if (nt > n) nt = n;
    if (nt <= T(1)) {
        body(r);
        return;
    }
    std::vector<std::thread> pool;
    std::vector<std::exception_ptr> errs(static_cast<std::size_t>(nt));
    const T chunk = n / nt, rem = n % nt;
    T b = r.begin();
    for (T t = 0; t < nt; ++t) {
        const T e = b + chunk + (t < rem ? T(1) : T(0));
        pool.emplace_back([&body, &errs, t, b, e]() {
            try {
                body(blocked_range<T>(b, e));
            } catch (...) {
                errs[static_cast<std::size_t>(t)] = std::current_exception();
            }
        });
        b = e;
    }
    for (auto &th : pool) th.join();
    for (auto &e : errs)
        if (e) std::rethrow_exception(e);
}
} // namespace tbb
#endif
