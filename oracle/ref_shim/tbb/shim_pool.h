// Minimal std::thread work splitter used by the TBB-compatible shim headers.
// Test infrastructure only: lets the reference's CPU sources compile without
// oneTBB so that their outputs can serve as golden vectors for the oracle.
#ifndef FG_TBB_SHIM_POOL_H
#define FG_TBB_SHIM_POOL_H
#include <algorithm>
#include <cstddef>
#include <cstdlib>
#include <thread>
#include <vector>

namespace tbb { namespace shim {
inline unsigned num_threads()
{
    const char* env = std::getenv("FG_REF_THREADS");
    if (env != nullptr && std::atoi(env) > 0)
    {
        return static_cast<unsigned>(std::atoi(env));
    }
    unsigned n = std::thread::hardware_concurrency();
    return n == 0 ? 1 : n;
}

// Run fn(begin, end) over [begin, end) split into contiguous chunks, one per thread.
template<typename F> void split_run(std::size_t begin, std::size_t end, const F& fn)
{
    if (end <= begin)
    {
        return;
    }
    const std::size_t n = end - begin;
    const std::size_t nt = std::min<std::size_t>(num_threads(), n);
    if (nt <= 1)
    {
        fn(begin, end);
        return;
    }
    std::vector<std::thread> threads;
    threads.reserve(nt);
    const std::size_t chunk = (n + nt - 1) / nt;
    for (std::size_t t = 0; t < nt; ++t)
    {
        const std::size_t b = begin + t * chunk;
        const std::size_t e = std::min(end, b + chunk);
        if (b >= e)
        {
            break;
        }
        threads.emplace_back([&fn, b, e]() { fn(b, e); });
    }
    for (auto& th : threads)
    {
        th.join();
    }
}
}; }; // namespace tbb::shim
#endif
